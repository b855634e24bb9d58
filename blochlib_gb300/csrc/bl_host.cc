// Host-side spin-system model: parsing, spin operators, Hamiltonian terms, block
// structure, powder sets and FID text output.  See bl_host.h for the reference map.
#include "bl_host.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <numeric>
#include <sstream>

namespace bl {

namespace {
const double kPi = 3.14159265358979323846;
const double kDeg2Rad = kPi / 180.0;

std::vector<std::string> split_ws(const std::string &s) {
  std::vector<std::string> out;
  std::string cur;
  for (char ch : s) {
    if (ch == ' ' || ch == '\t' || ch == '\n' || ch == '\r' || ch == ',') {
      if (!cur.empty()) out.push_back(cur), cur.clear();
    } else {
      cur.push_back(ch);
    }
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

std::string trim(const std::string &s) {
  size_t a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  size_t b = s.find_last_not_of(" \t\r\n");
  return s.substr(a, b - a + 1);
}

void mat3mul(const double A[3][3], const double B[3][3], double C[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C[i][j] = A[i][0] * B[0][j] + A[i][1] * B[1][j] + A[i][2] * B[2][j];
}

// PAS' = R diag(d) R^T, R = rotation3 of the interaction's Euler angles (degrees).
void crystal_tensor(Interaction &it, double d0, double d1, double d2) {
  double R[3][3], D[3][3] = {{d0, 0, 0}, {0, d1, 0}, {0, 0, d2}}, T[3][3], Rt[3][3];
  rotation3(it.alpha * kDeg2Rad, it.beta * kDeg2Rad, it.gamma * kDeg2Rad, R);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Rt[i][j] = R[j][i];
  mat3mul(R, D, T);
  mat3mul(T, Rt, it.pas);
}

// Real part of a real-valued product of two expanded single-spin operators.
std::vector<double> real_of(const CMatrix &m) {
  std::vector<double> r(m.a.size());
  for (size_t i = 0; i < r.size(); ++i) r[i] = m.a[i].real();
  return r;
}

CMatrix mul(const CMatrix &x, const CMatrix &y) {
  CMatrix z(x.n);
  for (int i = 0; i < x.n; ++i)
    for (int k = 0; k < x.n; ++k) {
      cplx v = x(i, k);
      if (v == cplx(0, 0)) continue;
      for (int j = 0; j < x.n; ++j) z(i, j) += v * y(k, j);
    }
  return z;
}
}  // namespace

double isotope_rel_freq(const std::string &iso) {
  // Larmor frequencies in MHz at 400.13 MHz for 1H, as tabulated by the reference
  // (src/bloch/Isotope.cc:154-263); only quadrupolar nuclei need them here
  static const std::map<std::string, double> t = {
      {"2H", 61.424},   {"6Li", 58.883},  {"7Li", 155.503}, {"9Be", 56.226},   {"10B", 42.99},   {"11B", 128.33},
      {"14N", 28.913},  {"17O", 54.242},  {"21Ne", 31.586}, {"23Na", 105.842}, {"25Mg", 24.496}, {"27Al", 104.262},
      {"33S", 30.714},  {"35Cl", 39.205}, {"37Cl", 32.635}, {"39K", 18.67},    {"43Ca", 26.925}, {"45Sc", 97.2},
      {"47Ti", 22.563}, {"49Ti", 22.557}, {"51V", 105.246}, {"53Cr", 22.615},  {"55Mn", 99.012}, {"59Co", 94.939},
      {"61Ni", 35.756}, {"63Cu", 106.146}, {"65Cu", 113.705}, {"67Zn", 25.036}, {"69Ga", 96.035}, {"71Ga", 122.028},
      {"79Br", 100.249}, {"81Br", 108.063}, {"87Rb", 130.927}, {"93Nb", 97.936}, {"95Mo", 26.076},
      {"115In", 87.68}, {"127I", 80.062}, {"131Xe", 32.811}, {"133Cs", 52.481}};
  auto it = t.find(iso);
  if (it == t.end()) throw Error(2, "no relative frequency for isotope '" + iso + "'");
  return it->second / 400.13;
}

double isotope_spin(const std::string &iso) {
  // nuclear spin quantum numbers of common NMR isotopes (physical constants)
  static const std::map<std::string, double> t = {
      {"1H", 0.5},    {"2H", 1.0},    {"3H", 0.5},    {"3He", 0.5},   {"6Li", 1.0},   {"7Li", 1.5},
      {"9Be", 1.5},   {"10B", 3.0},   {"11B", 1.5},   {"13C", 0.5},   {"14N", 1.0},   {"15N", 0.5},
      {"17O", 2.5},   {"19F", 0.5},   {"21Ne", 1.5},  {"23Na", 1.5},  {"25Mg", 2.5},  {"27Al", 2.5},
      {"29Si", 0.5},  {"31P", 0.5},   {"33S", 1.5},   {"35Cl", 1.5},  {"37Cl", 1.5},  {"39K", 1.5},
      {"43Ca", 3.5},  {"45Sc", 3.5},  {"47Ti", 2.5},  {"49Ti", 3.5},  {"51V", 3.5},   {"53Cr", 1.5},
      {"55Mn", 2.5},  {"57Fe", 0.5},  {"59Co", 3.5},  {"61Ni", 1.5},  {"63Cu", 1.5},  {"65Cu", 1.5},
      {"67Zn", 2.5},  {"69Ga", 1.5},  {"71Ga", 1.5},  {"77Se", 0.5},  {"79Br", 1.5},  {"81Br", 1.5},
      {"87Rb", 1.5},  {"89Y", 0.5},   {"93Nb", 4.5},  {"95Mo", 2.5},  {"103Rh", 0.5}, {"107Ag", 0.5},
      {"109Ag", 0.5}, {"111Cd", 0.5}, {"113Cd", 0.5}, {"115In", 4.5}, {"117Sn", 0.5}, {"119Sn", 0.5},
      {"125Te", 0.5}, {"127I", 2.5},  {"129Xe", 0.5}, {"131Xe", 1.5}, {"133Cs", 3.5}, {"183W", 0.5},
      {"195Pt", 0.5}, {"199Hg", 0.5}, {"205Tl", 0.5}, {"207Pb", 0.5}, {"e", 0.5}};
  auto it = t.find(iso);
  if (it == t.end()) throw Error(2, "unknown isotope '" + iso + "'");
  return it->second;
}

void rotation3(double a, double b, double g, double R[3][3]) {
  double cg = std::cos(g), cb = std::cos(b), ca = std::cos(a);
  double sg = std::sin(g), sb = std::sin(b), sa = std::sin(a);
  R[0][0] = ca * cb * cg - sa * sg;
  R[0][1] = sa * cb * cg + ca * sg;
  R[0][2] = -sb * cg;
  R[1][0] = -ca * cb * sg - sa * cg;
  R[1][1] = -sa * cb * sg + ca * cg;
  R[1][2] = sb * sg;
  R[2][0] = ca * sb;
  R[2][1] = sa * sb;
  R[2][2] = cb;
}

void rotation2(double phi, double theta, double R[3][3]) {
  double ct = std::cos(theta), cp = std::cos(phi), sp = std::sin(phi), st = std::sin(theta);
  R[0][0] = cp;
  R[0][1] = sp;
  R[0][2] = 0.0;
  R[1][0] = -ct * sp;
  R[1][1] = cp * ct;
  R[1][2] = st;
  R[2][0] = sp * st;
  R[2][1] = -cp * st;
  R[2][2] = ct;
}

SpinSystem SpinSystem::from_text(const std::string &text) {
  std::vector<std::string> lines;
  std::stringstream ss(text);
  std::string l;
  while (std::getline(ss, l)) lines.push_back(l);
  return SpinSystem(lines);
}

SpinSystem::SpinSystem(const std::vector<std::string> &lines) {
  std::vector<std::pair<std::string, int>> types;
  for (const auto &l : lines) {
    auto t = split_ws(l);
    if (t.size() >= 2 && (t[0] == "numspin" || t[0] == "spins")) nspin_ = std::atoi(t[1].c_str());
    if (t.size() >= 1 && (t[0] == "T" || t[0] == "type" || t[0] == "Type")) {
      if (t.size() < 3) throw Error(2, "'T' line needs: T <isotope> <spin>");
      types.push_back({t[1], std::atoi(t[2].c_str())});
    }
  }
  if (nspin_ < 1) throw Error(2, "numspin must be >= 1");
  iso_.assign(nspin_, "1H");
  for (auto &p : types) {
    if (p.second < 0 || p.second >= nspin_) throw Error(2, "isotope assigned to a spin outside numspin");
    iso_[p.second] = p.first;
  }
  dims_.resize(nspin_);
  N_ = 1;
  for (int i = 0; i < nspin_; ++i) {
    dims_[i] = int(std::lround(2 * isotope_spin(iso_[i]) + 1));
    N_ *= dims_[i];
    if (N_ > 4096) throw Error(5, "Hilbert space dimension above 4096 is not supported");
  }
  std::vector<Interaction> csa, dip, jj, qua;
  auto check_spin = [&](int s) {
    if (s < 0 || s >= nspin_) throw Error(2, "interaction names a spin outside numspin");
  };
  for (const auto &l : lines) {
    auto t = split_ws(l);
    if (t.empty() || t[0][0] == '#') continue;
    auto num = [&](size_t i) { return i < t.size() ? std::atof(t[i].c_str()) : 0.0; };
    const std::string &k = t[0];
    if (k == "C" || k == "CSA" || k == "csa") {
      if (t.size() < 5) throw Error(2, "a CSA needs: C <iso> <del> <eta> <spin> [alpha beta gamma]");
      Interaction it;
      it.kind = 'C';
      it.iso = num(1), it.del = num(2), it.eta = num(3), it.s1 = std::atoi(t[4].c_str());
      it.alpha = num(5), it.beta = num(6), it.gamma = num(7);
      check_spin(it.s1);
      crystal_tensor(it, it.del * (it.eta - 1.0) / 2.0, -it.del * (it.eta + 1.0) / 2.0, 1.0 * it.del);
      it.op_scale = 1.0;
      csa.push_back(it);
    } else if (k == "D" || k == "Dip" || k == "dip" || k == "DIP") {
      if (t.size() < 4) throw Error(2, "a dipole needs: D <coupling> <spin1> <spin2> [alpha beta gamma]");
      Interaction it;
      it.kind = 'D';
      it.del = num(1), it.s1 = int(num(2)), it.s2 = int(num(3));
      it.alpha = num(4), it.beta = num(5), it.gamma = num(6);
      check_spin(it.s1), check_spin(it.s2);
      double r6 = std::pow(6.0, 0.5);
      crystal_tensor(it, -0.5 * it.del * r6, -0.5 * it.del * r6, 1.0 * it.del * r6);
      it.op_scale = 1.0;
      dip.push_back(it);
    } else if (k == "J" || k == "j" || k == "jcop" || k == "Jcop") {
      if (t.size() < 4) throw Error(2, "a J coupling needs: J <coupling> <spin1> <spin2> [strong]");
      Interaction it;
      it.kind = 'J';
      it.iso = num(1), it.s1 = std::atoi(t[2].c_str()), it.s2 = std::atoi(t[3].c_str());
      it.strong = t.size() >= 5 ? std::atoi(t[4].c_str()) : 0;
      check_spin(it.s1), check_spin(it.s2);
      jj.push_back(it);
    } else if (k == "Q" || k == "QUAD" || k == "Quad") {
      if (t.size() < 4) throw Error(2, "a quadrupole needs: Q <coupling> <eta> <spin> [alpha beta gamma]");
      Interaction it;
      it.kind = 'Q';
      it.del = num(1), it.eta = num(2), it.s1 = std::atoi(t[3].c_str());
      it.alpha = num(4), it.beta = num(5), it.gamma = num(6);
      it.order = t.size() >= 8 ? int(num(7)) : 0;  // qua.cc:557-560
      check_spin(it.s1);
      crystal_tensor(it, (it.eta - 1.0) / 2.0, -(it.eta + 1.0) / 2.0, 1.0);
      qua.push_back(it);
    }
  }
  // evaluation order of SolidSys::Hamiltonian: CSA, dipoles, J, quadrupoles
  for (auto *v : {&csa, &dip, &jj, &qua}) ints_.insert(ints_.end(), v->begin(), v->end());
  build();
}

namespace {
// Single-spin operator of a spin with hs levels (m from +I down), hs x hs.
CMatrix small_op(char which, int hs) {
  CMatrix m(hs);
  double q = (hs - 1.0) / 2.0, q1 = q * (q + 1.0);
  if (which == 'z') {
    double mm = q;
    for (int k = 0; k < hs; ++k, mm -= 1) m(k, k) = mm;
  } else if (which == 'e') {
    for (int k = 0; k < hs; ++k) m(k, k) = 1.0;
  } else {
    double mm = q - 1;
    for (int k = 0; k < hs - 1; ++k, mm -= 1) {
      double c = std::sqrt(q1 - mm * (mm + 1));
      if (which == 'x') m(k + 1, k) = c / 2, m(k, k + 1) = c / 2;
      else if (which == 'y') m(k + 1, k) = cplx(0, c / 2), m(k, k + 1) = cplx(0, -c / 2);
      else if (which == 'p') m(k, k + 1) = c;
      else if (which == 'm') m(k + 1, k) = c;
      else throw Error(1, "unknown single-spin operator");
    }
  }
  return m;
}
}  // namespace

// For the two spins s1 != s2: every element (row, col) of the full space where a product of
// single-spin operators of these spins can be non-zero, with the real parts of the xx, yy and
// zz products there, f(row, col, xx, yy, zz).  A product of operators on different spins has
// one term per element (the Kronecker digits of s1 and s2 change, all others agree), so the
// values equal the dense products exactly.
template <class F>
void SpinSystem::pair_terms(int s1, int s2, F f) const {
  const int h1 = dims_[s1], h2 = dims_[s2];
  long R1 = 1, R2 = 1;
  for (int i = s1 + 1; i < nspin_; ++i) R1 *= dims_[i];
  for (int i = s2 + 1; i < nspin_; ++i) R2 *= dims_[i];
  const CMatrix ax = small_op('x', h1), ay = small_op('y', h1), az = small_op('z', h1);
  const CMatrix bx = small_op('x', h2), by = small_op('y', h2), bz = small_op('z', h2);
  for (long row = 0; row < N_; ++row) {
    const int d1 = int((row / R1) % h1), d2 = int((row / R2) % h2);
    for (int c1 = 0; c1 < h1; ++c1)
      for (int c2 = 0; c2 < h2; ++c2) {
        const cplx xx = ax(d1, c1) * bx(d2, c2), yy = ay(d1, c1) * by(d2, c2), zz = az(d1, c1) * bz(d2, c2);
        if (xx == cplx(0, 0) && yy == cplx(0, 0) && zz == cplx(0, 0)) continue;
        f(row, row + (c1 - d1) * R1 + (c2 - d2) * R2, xx.real(), yy.real(), zz.real());
      }
  }
}

// Diagonal of Iz of one spin in the full space.
std::vector<double> SpinSystem::iz_diag(int s) const {
  long R = 1;
  for (int i = s + 1; i < nspin_; ++i) R *= dims_[i];
  const double q = (dims_[s] - 1.0) / 2.0;
  std::vector<double> z(N_);
  for (long row = 0; row < N_; ++row) z[row] = q - double((row / R) % dims_[s]);
  return z;
}

CMatrix SpinSystem::single(char which, int spin) const {
  if (spin < 0 || spin >= nspin_) throw Error(1, "spin index out of range");
  int hs = dims_[spin];
  CMatrix m = small_op(which, hs);
  // Kronecker expansion, spin 0 most significant (multispinop.cc:51-74)
  int left = 1, right = 1;
  for (int i = 0; i < spin; ++i) left *= dims_[i];
  for (int i = spin + 1; i < nspin_; ++i) right *= dims_[i];
  CMatrix out(N_);
  for (int l = 0; l < left; ++l)
    for (int r1 = 0; r1 < hs; ++r1)
      for (int c1 = 0; c1 < hs; ++c1) {
        cplx v = m(r1, c1);
        if (v == cplx(0, 0)) continue;
        for (int r = 0; r < right; ++r) {
          int row = (l * hs + r1) * right + r, col = (l * hs + c1) * right + r;
          out(row, col) = v;
        }
      }
  return out;
}

CMatrix SpinSystem::op(const std::string &expr) const {
  CMatrix acc(N_);
  std::stringstream ss(expr);
  std::string term;
  bool any = false;
  while (std::getline(ss, term, '+')) {
    term = trim(term);
    if (term.empty()) continue;
    double coef = 1.0;
    size_t star = term.find('*');
    if (star != std::string::npos) {
      char *end = nullptr;
      std::string cs = trim(term.substr(0, star));
      coef = std::strtod(cs.c_str(), &end);
      if (end == cs.c_str()) throw Error(1, "bad coefficient in operator expression '" + expr + "'");
      term = trim(term.substr(star + 1));
    }
    std::istringstream is(term);
    std::string name;
    int k = -1;
    is >> name >> k;
    CMatrix m(N_);
    auto total = [&](char w) {
      CMatrix t(N_);
      for (int s = 0; s < nspin_; ++s) {
        CMatrix x = single(w, s);
        for (size_t i = 0; i < t.a.size(); ++i) t.a[i] += x.a[i];
      }
      return t;
    };
    if (name == "Fx") m = total('x');
    else if (name == "Fy") m = total('y');
    else if (name == "Fz") m = total('z');
    else if (name == "Fp") m = total('p');
    else if (name == "Fm") m = total('m');
    else if (name == "Fe") { for (int i = 0; i < N_; ++i) m(i, i) = 1.0; }
    else if (name.size() == 2 && name[0] == 'I' && std::string("xyzpm").find(name[1]) != std::string::npos) {
      if (k < 0) throw Error(1, "single-spin operator '" + name + "' needs a spin index");
      m = single(name[1], k);
    } else {
      throw Error(1, "unknown operator '" + name + "' in '" + expr + "'");
    }
    for (size_t i = 0; i < acc.a.size(); ++i) acc.a[i] += coef * m.a[i];
    any = true;
  }
  if (!any) throw Error(1, "empty operator expression");
  return acc;
}

void SpinSystem::build() {
  size_t NN = size_t(N_) * N_;
  hc_.assign(NN, 0.0);
  hops_.clear();
  hq4_.assign(ints_.size(), {});
  hq2_.assign(ints_.size(), {});
  const double inv_r3 = 1.0 / std::pow(3., 0.5), r3 = std::pow(3., 0.5);
  for (auto &it : ints_) {
    std::vector<double> T(NN, 0.0);
    if (it.kind == 'C') {
      // a*Iz + (1/sqrt3 Iz)(-sqrt3 iso)   (csa.cc:289-329, spin_ten.cc:211-236)
      const std::vector<double> Iz = iz_diag(it.s1);
      for (int k = 0; k < N_; ++k) {
        double z = Iz[k];
        T[size_t(k) * N_ + k] = z;
        if (it.iso != 0) hc_[size_t(k) * N_ + k] += (inv_r3 * z) * (-r3 * it.iso);
      }
    } else if (it.kind == 'D') {
      // homonuclear sqrt(1/6)(2IzIz - IxIx - IyIy); heteronuclear sqrt(4/6) IzIz (spin_ten.cc:431-452)
      if (iso_[it.s1] == iso_[it.s2]) {
        double f = std::pow(1. / 6., 0.5);
        pair_terms(it.s1, it.s2, [&](long r, long c, double xx, double yy, double zz) {
          T[size_t(r) * N_ + c] = f * (2.0 * zz - xx - yy);
        });
      } else {
        double f = std::pow(4. / 6., 0.5);
        pair_terms(it.s1, it.s2, [&](long r, long c, double, double, double zz) {
          T[size_t(r) * N_ + c] = f * zz;
        });
      }
    } else if (it.kind == 'J') {
      // iso*sqrt3 * (1/sqrt3)(IzIz [+IxIx+IyIy])   (j.cc:129-137, spin_ten.cc:455-465)
      pair_terms(it.s1, it.s2, [&](long r, long c, double xx, double yy, double zz) {
        double v = zz;
        if (it.strong) v = v + xx + yy;
        hc_[size_t(r) * N_ + c] += (inv_r3 * v) * (it.iso * std::sqrt(3.));
      });
    } else if (it.kind == 'Q') {
      // first order: Qp * a * 3 Iz^2, Qp = Q / (4 I (2I-1))   (qua.cc:219-267, spin_ten.cc:285-300)
      double spin = isotope_spin(iso_[it.s1]);
      if (spin < 1.0) throw Error(2, "a quadrupole needs a spin >= 1");
      it.op_scale = it.del / (4.0 * spin * (2.0 * spin - 1.0));
      const std::vector<double> Iz = iz_diag(it.s1);
      const size_t ki = size_t(&it - ints_.data());
      hq4_[ki].assign(NN, 0.0), hq2_[ki].assign(NN, 0.0);
      const double q = spin;
      for (int k = 0; k < N_; ++k) {
        double z = Iz[k];
        T[size_t(k) * N_ + k] = 3.0 * (z * z);
        // T_QuadTotal: Iz 2 (-8 Iz^2 - 1 + 4 I(I+1)) (rank 2), Iz 2 (-2 Iz^2 - 1 + 2 I(I+1)) (rank 4)
        hq2_[ki][size_t(k) * N_ + k] = (z * 2.0) * ((-8.0 * (z * z) - 1.0) + 4.0 * q * (q + 1));
        hq4_[ki][size_t(k) * N_ + k] = (z * 2.0) * ((-2.0 * (z * z) - 1.0) + 2.0 * q * (q + 1));
      }
    }
    hops_.push_back(T);
  }
  // rf fields (PulseData::Pulse, pulsedata.cc:110-125): per isotope the sum of its fields
  // amp e^{i phase}; the real axis goes into hc_, a phase off it into the frame
  frame_.clear();
  if (!rf_.empty()) {
    std::map<std::string, std::pair<cplx, double>> chan;  // iso -> (sum amp e^{i phase}, offsets)
    for (const RfField &f : rf_) {
      if (f.amp == 0.0) continue;
      const double r = std::fmod(f.phase_deg, 360.0);
      cplx e;
      if (std::fmod(f.phase_deg, 180.0) == 0.0) e = (r == 0.0) ? 1.0 : -1.0;  // x or -x: exact
      else e = cplx(std::cos(f.phase_deg * 3.14159265358979323846 / 180.0),
                    std::sin(f.phase_deg * 3.14159265358979323846 / 180.0));
      chan[f.iso].first += f.amp * e;
      chan[f.iso].second += f.offset;
    }
    std::vector<double> frame_phase(N_, 0.0);
    bool any_phase = false;
    for (auto &kv : chan) {
      const cplx c = kv.second.first;
      double ax = c.real();
      std::vector<double> m(N_, 0.0);  // Fz of the isotope, diagonal
      bool present = false;
      for (int s = 0; s < nspin_; ++s) {
        if (iso_[s] != kv.first) continue;
        present = true;
        const std::vector<double> z = iz_diag(s);
        for (int k = 0; k < N_; ++k) m[k] += z[k];
      }
      if (!present) continue;
      if (c.imag() != 0.0) {
        // the rest of H must commute with Fz of this isotope for the frame to be exact
        auto commutes = [&](const std::vector<double> &M) {
          for (int r = 0; r < N_; ++r)
            for (int q = 0; q < N_; ++q)
              if (M[size_t(r) * N_ + q] != 0.0 && m[r] != m[q]) return false;
          return true;
        };
        bool ok = commutes(hc_);
        for (const auto &T : hops_) ok = ok && commutes(T);
        if (!ok)
          throw Error(5, "an rf phase off the x axis on " + kv.first +
                             " needs a Hamiltonian that commutes with its Fz (a strong J coupling to another "
                             "isotope does not)");
        ax = std::abs(c);
        const double ph = std::atan2(c.imag(), c.real());
        for (int k = 0; k < N_; ++k) frame_phase[k] -= ph * m[k];
        any_phase = true;
      }
      for (int s = 0; s < nspin_; ++s) {
        if (iso_[s] != kv.first) continue;
        const CMatrix x = single('x', s);
        const std::vector<double> z = iz_diag(s);
        for (size_t i = 0; i < hc_.size(); ++i) hc_[i] += ax * x.a[i].real();
        for (int k = 0; k < N_; ++k) hc_[size_t(k) * N_ + k] += kv.second.second * z[k];
      }
    }
    if (any_phase) {
      frame_.resize(N_);
      for (int k = 0; k < N_; ++k) frame_[k] = cplx(std::cos(frame_phase[k]), std::sin(frame_phase[k]));
    }
  }
  // Block structure: connected components of the union non-zero pattern.
  std::vector<int> parent(N_);
  std::iota(parent.begin(), parent.end(), 0);
  auto find = [&](int x) {
    while (parent[x] != x) x = parent[x] = parent[parent[x]];
    return x;
  };
  auto scan = [&](const std::vector<double> &M) {  // row by row: both triangles
    for (int r = 0; r < N_; ++r) {
      const double *row = M.data() + size_t(r) * N_;
      for (int c = 0; c < N_; ++c)
        if (c != r && row[c] != 0.0) {
          int a = find(r), b = find(c);
          if (a != b) parent[std::max(a, b)] = std::min(a, b);
        }
    }
  };
  scan(hc_);
  for (auto &T : hops_) scan(T);
  std::map<int, std::vector<int>> comps;
  for (int s = 0; s < N_; ++s) comps[find(s)].push_back(s);
  BlockLayout &L = layout_;
  L = BlockLayout();
  L.N = N_;
  L.inv.assign(N_, -1);
  for (auto &kv : comps) {
    L.off.push_back(int(L.perm.size()));
    L.size.push_back(int(kv.second.size()));
    L.poff.push_back(L.S2);
    L.S2 += int(kv.second.size() * kv.second.size());
    L.max_block = std::max(L.max_block, int(kv.second.size()));
    for (int s : kv.second) {
      L.inv[s] = int(L.perm.size());
      L.block_of.push_back(int(L.size.size()) - 1);
      L.perm.push_back(s);
    }
  }
}

void SpinSystem::add_rf(const RfField &f) {
  rf_.push_back(f);
  try {
    build();
  } catch (...) {
    rf_.pop_back();
    build();
    throw;
  }
}

CMatrix SpinSystem::to_frame(const CMatrix &X) const {
  if (frame_.empty()) return X;
  CMatrix Y = X;
  for (int r = 0; r < N_; ++r)
    for (int c = 0; c < N_; ++c) Y(r, c) = std::conj(frame_[r]) * X(r, c) * frame_[c];
  return Y;
}

std::vector<double> SpinSystem::hamiltonian(const double Rp[3][3], double alpha_rot, double rotb_rad) const {
  size_t NN = size_t(N_) * N_;
  std::vector<double> H = hc_;
  double Rr[3][3], M[3][3];
  rotation2(alpha_rot, rotb_rad, Rr);
  mat3mul(Rr, Rp, M);
  for (size_t k = 0; k < ints_.size(); ++k) {
    const Interaction &it = ints_[k];
    if (it.kind == 'J') continue;
    double a = 0;
    for (int j = 0; j < 3; ++j)
      for (int l = 0; l < 3; ++l) a += M[2][j] * it.pas[j][l] * M[2][l];
    for (size_t i = 0; i < NN; ++i) H[i] += it.op_scale * a * hops_[k][i];
  }
  return H;
}

// ---------------------------------------------------------------- powder sets

Powder powder_zcw(int tstep, int pstep, int gstep) {
  static const int vt[10] = {21, 34, 55, 89, 144, 233, 377, 616, 987, 4184};
  static const int vp[10] = {8, 13, 21, 34, 55, 89, 144, 233, 377, 2584};
  bool gt = false, gp = false;
  for (int i = 0; i < 10; ++i) {
    if (tstep == vt[i]) gt = true;
    if (pstep == vp[i]) gp = true;
  }
  if (!gt || !gp || tstep <= pstep)
    throw Error(1, "ZCW needs Fibonacci theta_step/phi_step with theta_step > phi_step");
  Powder P;
  int gs = gstep <= 0 ? 1 : gstep;
  for (int g = 0; g < gs; ++g) {
    double gnow = gstep == 0 ? 0.0 : double(g) / double(gstep) * kPi;
    for (int k = 1; k < tstep; ++k) {
      double fac = double(k) / double(tstep);
      double f0 = fac - std::floor(fac);
      double f1 = double(fac * pstep);
      f1 = f1 - std::floor(f1);
      P.phi.push_back(2. * kPi * f0);
      P.theta.push_back(kPi * f1);
      P.weight.push_back(1.0 / double(tstep) * std::sin(kPi * f1));
      P.gamma.push_back(gnow);
    }
  }
  double s = 0;
  for (double w : P.weight) s += w;
  for (double &w : P.weight) w /= s;
  return P;
}

Powder powder_read(const std::string &path) {
  std::ifstream in(path);
  if (!in) throw Error(1, "no powder file '" + path + "'");
  Powder P;
  std::string line;
  while (std::getline(in, line)) {
    auto t = split_ws(line);
    if (t.empty() || t[0][0] == '#' || t[0][0] == '%') continue;
    P.phi.push_back(std::atof(t[0].c_str()));
    P.theta.push_back(t.size() >= 2 ? std::atof(t[1].c_str()) : 0.0);
    if (t.size() == 3) {
      P.weight.push_back(std::atof(t[2].c_str()));
      P.gamma.push_back(0.0);
    } else if (t.size() >= 4) {
      P.gamma.push_back(std::atof(t[2].c_str()));
      P.weight.push_back(std::atof(t[3].c_str()));
    } else {
      P.weight.push_back(1.0);
      P.gamma.push_back(0.0);
    }
  }
  return P;
}

// ---------------------------------------------------------------- FID output

namespace {
// Radix-2 transform with the reference's sign (+i) and no normalisation
// (src/container/Vector/Vectoraux.h:113-160).
std::vector<cplx> fft_pos(std::vector<cplx> d) {
  int n = int(d.size());
  for (int j = 0, i = 0; i < n; ++i) {
    if (j > i) std::swap(d[i], d[j]);
    int m = n / 2;
    while (m > 1 && j >= m) j -= m, m /= 2;
    j += m;
  }
  for (int mmax = 1; n > mmax; mmax *= 2) {
    double theta = kPi / mmax, s2 = std::sin(theta * 0.5);
    cplx wp(-2. * s2 * s2, std::sin(theta)), w(1, 0);
    for (int ii = 0; ii < mmax; ++ii) {
      for (int i = ii; i < n; i += 2 * mmax) {
        int j = i + mmax;
        cplx t = w * d[j];
        d[j] = d[i] - t;
        d[i] += t;
      }
      w += w * wp;
    }
  }
  return d;
}
}  // namespace

void write_fid_text(const std::string &path, const cplx *fid, int npts, double dt) {
  int n = 1;
  while (n < npts) n *= 2;
  std::vector<cplx> tf(fid, fid + npts);
  tf.resize(n, cplx(0, 0));
  // The reference zero-fills a length that is not a power of two with
  // Vector::resizeAndPreserve(n, 0) (src/container/Vector/Vector.h:505-513), whose fill loop
  // starts at the old length minus one: the last FID point becomes zero in both the time
  // columns and the spectrum.  Kept, so that the files are the same.
  if (n != npts && npts > 0) tf[size_t(npts) - 1] = cplx(0, 0);
  std::vector<cplx> sp = fft_pos(tf);
  int sh = int(std::ceil(double(n) / 2.0));
  std::vector<cplx> sh_sp(n);
  for (int j = 0; j < n; ++j) sh_sp[j] = sp[(j + sh) % n];
  std::ofstream oo(path);
  if (!oo) throw Error(1, "cannot write '" + path + "'");
  double dw = 1. / dt / n, minw = -1. / dt / 2., t = 0;
  for (int i = 0; i < n; ++i) {
    oo << t << " " << minw << " " << sh_sp[i].real() << " " << sh_sp[i].imag() << " " << tf[i].real() << " "
       << tf[i].imag() << " " << std::abs(sh_sp[i]) << "\n";
    minw += dw;
    t += dt;
  }
}

// ---------------------------------------------------------------- MAT-5 files
namespace {
constexpr uint32_t miINT8 = 1, miUINT16 = 4, miINT32 = 5, miUINT32 = 6, miDOUBLE = 9, miMATRIX = 14;
constexpr uint32_t mxCHAR_CLASS = 4, mxDOUBLE_CLASS = 6, kComplexFlag = 0x0800;
size_t padded8(size_t n) { return (n + 7) / 8 * 8; }
}  // namespace

void Mat5Writer::bytes(const void *p, size_t n) { f_.write(static_cast<const char *>(p), std::streamsize(n)); }
void Mat5Writer::u32(uint32_t v) {  // little endian, whatever the host
  const unsigned char b[4] = {static_cast<unsigned char>(v), static_cast<unsigned char>(v >> 8),
                              static_cast<unsigned char>(v >> 16), static_cast<unsigned char>(v >> 24)};
  bytes(b, 4);
}
void Mat5Writer::pad8(size_t n) {
  static const char z[8] = {0};
  if (padded8(n) != n) bytes(z, padded8(n) - n);
}
void Mat5Writer::name_element(const std::string &name) {
  u32(miINT8), u32(uint32_t(name.size()));
  bytes(name.data(), name.size());
  pad8(name.size());
}

Mat5Writer::Mat5Writer(const std::string &path) : f_(path, std::ios::binary | std::ios::trunc) {
  if (!f_) throw Error(1, "cannot write '" + path + "'");
  std::string txt = "MATLAB 5.0 MAT-file, written by blochlib_gb300";
  txt.resize(116, ' ');
  bytes(txt.data(), 116);
  const char subsys[8] = {0};
  bytes(subsys, 8);
  const unsigned char ver_endian[4] = {0x00, 0x01, 'I', 'M'};  // version 0x0100, "MI" read as int16
  bytes(ver_endian, 4);
}

void Mat5Writer::put_matrix(const std::string &name, const double *re, const double *im, int rows, int cols) {
  if (rows < 0 || cols < 0 || name.empty()) throw Error(1, "bad MAT-5 variable");
  const size_t n = size_t(rows) * size_t(cols), data = 8 * n;
  const size_t body = 16 + 16 + 8 + padded8(name.size()) + 8 + data + (im ? 8 + data : 0);
  u32(miMATRIX), u32(uint32_t(body));
  u32(miUINT32), u32(8), u32(mxDOUBLE_CLASS | (im ? kComplexFlag : 0)), u32(0);  // array flags
  u32(miINT32), u32(8), u32(uint32_t(rows)), u32(uint32_t(cols));                 // dimensions
  name_element(name);
  u32(miDOUBLE), u32(uint32_t(data));
  for (size_t i = 0; i < n; ++i) {
    uint64_t v;
    std::memcpy(&v, re + i, 8);
    u32(uint32_t(v)), u32(uint32_t(v >> 32));
  }
  if (im) {
    u32(miDOUBLE), u32(uint32_t(data));
    for (size_t i = 0; i < n; ++i) {
      uint64_t v;
      std::memcpy(&v, im + i, 8);
      u32(uint32_t(v)), u32(uint32_t(v >> 32));
    }
  }
  f_.flush();
  if (!f_) throw Error(1, "MAT-5 write failed for '" + name + "'");
}

void Mat5Writer::put_string(const std::string &name, const std::string &text) {
  if (name.empty()) throw Error(1, "bad MAT-5 variable");
  const size_t n = text.size(), data = 2 * n;
  const size_t body = 16 + 16 + 8 + padded8(name.size()) + 8 + padded8(data);
  u32(miMATRIX), u32(uint32_t(body));
  u32(miUINT32), u32(8), u32(mxCHAR_CLASS), u32(0);
  u32(miINT32), u32(8), u32(1), u32(uint32_t(n));
  name_element(name);
  u32(miUINT16), u32(uint32_t(data));
  for (unsigned char ch : text) {
    const unsigned char b[2] = {ch, 0};
    bytes(b, 2);
  }
  pad8(data);
  f_.flush();
  if (!f_) throw Error(1, "MAT-5 write failed for '" + name + "'");
}

}  // namespace bl
