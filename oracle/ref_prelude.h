/* Forced-include prelude for compiling the BlochLib reference sources with g++ 13.
 * Test infrastructure only (builds the reference that pins the oracle).
 * The 2002-era sources call unqualified libm functions inside namespace BlochLib. */
#include <cmath>
#include <cstdlib>
#include <ctime>
#include <cstring>
#include <climits>
#include <cstdio>
#ifndef BL_QL_REAL
#define BL_QL_REAL float
#endif
namespace BlochLib {
using std::sin; using std::cos; using std::tan; using std::sqrt; using std::exp; using std::log;
using std::pow; using std::fabs; using std::atan2; using std::atan; using std::acos; using std::asin;
using std::sinh; using std::cosh; using std::tanh; using std::floor; using std::ceil; using std::log10;
using std::abs;
}
