// CPU restatement of BlochLib's spinning powder-FID path (gamma-COMPUTE), all FP64.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA product path is
// checked against.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
// leg may load it.  The product never links it and has no CPU fallback.
//
// It is a plain, dense restatement of the reference's arithmetic, written from the
// reference's behaviour and pinned against the reference itself (oracle/ref_harness.cc
// built by oracle/build_ref.sh; golden fixtures in tests/golden/).  Reference files it
// follows (paths inside the BlochLib tree):
//   spin-system text format        src/QMspins/sys.cc:120-204, csa.cc:400-440,
//                                  dip.cc:285-323, j.cc:171-202, qua.cc:511-560
//   single-spin operators          src/QMspins/singlespinop.cc:88-200
//   Kronecker order (spin 0 MSB)   src/QMspins/multispinop.cc:51-74
//   interaction tensors            csa.cc:223-329, dip.cc:136-207, j.cc:129-137,
//                                  qua.cc:169-267, spin_ten.cc:211-236, 285-372, 431-465
//   rotations                      src/QMspins/space_ten.cc:578-652 (3-angle, 2-angle),
//                                  717-805 (powder / rotor angle setters)
//   H(t1,t2,wr)                    src/QMspins/sys.cc:749-770
//   step exponential               src/container/matrix/matexp.h:240-252 (+ chop 1e-12)
//   gamma-COMPUTE                  src/QMspins/driver/compute.h:86-97, 213-235, 257-274,
//                                  294-306, 308-461
//   powder loop                    src/QMspins/driver/oneFID.h:200-208, 339-431
//   static powder FID              src/QMspins/driver/oneFID.h:220-336
//   powder file reader             src/QMspins/driver/powder.cc:333-389
//   point-to-point FID             examples/qmsims/MMMQMAS/propreduce.cc:16-60, 455-521,
//                                  mmmqmas.cc:290-370; examples/solid-2.0/src/
//                                  sequencerun_funcs.cc:624-645, propogation.cc:246-296
//
// Eigen-solvers are this file's own: cyclic complex Jacobi for Hermitian matrices, and
// for the unitary period propagator a Cayley transform K = i(I-W)(I+W)^-1 of the
// phase-shifted W = e^{i a} U (Hermitian, same eigenvectors) solved by the same Jacobi.
// Eigenvalues come from Rayleigh quotients v^H U v.  The reference instead uses
// Householder + QL (matdiagonalize.h:251-483) and corth + comqr3 (matdiagonalize.h:
// 519-1188); the FID is invariant to that choice up to rounding.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

namespace {

typedef std::complex<double> cplx;
const double kPi = 3.14159265358979323846;
const double kPi2 = 2.0 * kPi;
const double kDeg2Rad = kPi / 180.0;

struct CMat {
  int n = 0;
  std::vector<cplx> a;  // row-major
  CMat() {}
  explicit CMat(int n_) : n(n_), a(size_t(n_) * n_, cplx(0, 0)) {}
  cplx &operator()(int r, int c) { return a[size_t(r) * n + c]; }
  const cplx &operator()(int r, int c) const { return a[size_t(r) * n + c]; }
};

CMat identity(int n) {
  CMat m(n);
  for (int i = 0; i < n; ++i) m(i, i) = 1.0;
  return m;
}

CMat mul(const CMat &x, const CMat &y) {
  int n = x.n;
  CMat z(n);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < n; ++k) {
      cplx xik = x(i, k);
      if (xik == cplx(0, 0)) continue;
      for (int j = 0; j < n; ++j) z(i, j) += xik * y(k, j);
    }
  return z;
}

CMat adj(const CMat &x) {
  CMat z(x.n);
  for (int i = 0; i < x.n; ++i)
    for (int j = 0; j < x.n; ++j) z(i, j) = std::conj(x(j, i));
  return z;
}

CMat add(const CMat &x, const CMat &y, double sy = 1.0) {
  CMat z = x;
  for (size_t i = 0; i < z.a.size(); ++i) z.a[i] += sy * y.a[i];
  return z;
}

CMat scale(const CMat &x, double s) {
  CMat z = x;
  for (auto &v : z.a) v *= s;
  return z;
}

// U^H X U  (reference adjprop, src/container/matrix/matmat.h:1049-1066)
CMat adjprop(const CMat &U, const CMat &X) { return mul(adj(U), mul(X, U)); }

CMat kron(const CMat &x, const CMat &y) {
  CMat z(x.n * y.n);
  for (int i = 0; i < x.n; ++i)
    for (int j = 0; j < x.n; ++j)
      for (int k = 0; k < y.n; ++k)
        for (int l = 0; l < y.n; ++l) z(i * y.n + k, j * y.n + l) = x(i, j) * y(k, l);
  return z;
}

// ---------------------------------------------------------------- eigen-solvers

// Cyclic Jacobi for a Hermitian matrix.  On return H holds the eigenvalues on its
// diagonal and V (columns) the orthonormal eigenvectors: H_in = V diag V^H.
void jacobi_herm(CMat H, std::vector<double> &w, CMat &V) {
  int n = H.n;
  V = identity(n);
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, tot = 0;
    for (int p = 0; p < n; ++p)
      for (int q = 0; q < n; ++q) {
        double m = std::norm(H(p, q));
        tot += m;
        if (p != q) off += m;
      }
    if (off <= 1e-34 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        cplx hpq = H(p, q);
        double ab = std::abs(hpq);
        if (ab == 0.0) continue;
        // rotate away |hpq| after removing its phase: hpq = ab e^{i phi}
        cplx ph = hpq / ab;
        double app = H(p, p).real(), aqq = H(q, q).real();
        double theta = 0.5 * (aqq - app) / ab;
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        // G = [[c, s*ph],[-s*conj(ph), c]] acting on columns p,q: H <- G^H H G
        cplx sp = s * ph;
        for (int k = 0; k < n; ++k) {  // columns
          cplx hkp = H(k, p), hkq = H(k, q);
          H(k, p) = c * hkp - std::conj(sp) * hkq;
          H(k, q) = sp * hkp + c * hkq;
        }
        for (int k = 0; k < n; ++k) {  // rows
          cplx hpk = H(p, k), hqk = H(q, k);
          H(p, k) = c * hpk - sp * hqk;
          H(q, k) = std::conj(sp) * hpk + c * hqk;
        }
        H(p, q) = 0;
        H(q, p) = 0;
        H(p, p) = H(p, p).real();
        H(q, q) = H(q, q).real();
        for (int k = 0; k < n; ++k) {
          cplx vkp = V(k, p), vkq = V(k, q);
          V(k, p) = c * vkp - std::conj(sp) * vkq;
          V(k, q) = sp * vkp + c * vkq;
        }
      }
  }
  w.resize(n);
  for (int i = 0; i < n; ++i) w[i] = H(i, i).real();
}

// Solve A X = B (complex, Gaussian elimination with partial pivoting).
CMat solve(CMat A, CMat B) {
  int n = A.n;
  for (int k = 0; k < n; ++k) {
    int piv = k;
    for (int i = k + 1; i < n; ++i)
      if (std::abs(A(i, k)) > std::abs(A(piv, k))) piv = i;
    if (piv != k)
      for (int j = 0; j < n; ++j) {
        std::swap(A(k, j), A(piv, j));
        std::swap(B(k, j), B(piv, j));
      }
    for (int i = k + 1; i < n; ++i) {
      cplx f = A(i, k) / A(k, k);
      if (f == cplx(0, 0)) continue;
      for (int j = k; j < n; ++j) A(i, j) -= f * A(k, j);
      for (int j = 0; j < n; ++j) B(i, j) -= f * B(k, j);
    }
  }
  for (int k = n - 1; k >= 0; --k)
    for (int j = 0; j < n; ++j) {
      cplx s = B(k, j);
      for (int i = k + 1; i < n; ++i) s -= A(k, i) * B(i, j);
      B(k, j) = s / A(k, k);
    }
  return B;
}

// Eigen-decomposition of a unitary matrix U = V diag(lam) V^H via the Cayley transform
// of W = e^{ia}U.  'a' is chosen in a second pass so that -1 sits in the middle of the
// widest gap of the spectrum of W, keeping I+W well conditioned.
void unitary_eig(const CMat &U, std::vector<cplx> &lam, CMat &V) {
  int n = U.n;
  double a = 0.5;
  for (int pass = 0; pass < 2; ++pass) {
    cplx ea = std::polar(1.0, a);
    CMat W = scale(U, 1.0);
    for (auto &v : W.a) v *= ea;
    CMat IpW = identity(n), ImW = identity(n);
    for (size_t i = 0; i < W.a.size(); ++i) {
      IpW.a[i] += W.a[i];
      ImW.a[i] -= W.a[i];
    }
    CMat X = solve(IpW, ImW);
    CMat K(n);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) K(i, j) = cplx(0, 1) * X(i, j);
    CMat Kh = adj(K);
    for (size_t i = 0; i < K.a.size(); ++i) K.a[i] = 0.5 * (K.a[i] + Kh.a[i]);
    std::vector<double> w;
    jacobi_herm(K, w, V);
    CMat UV = mul(U, V);
    lam.assign(n, cplx(0, 0));
    for (int r = 0; r < n; ++r) {
      cplx s = 0;
      for (int k = 0; k < n; ++k) s += std::conj(V(k, r)) * UV(k, r);
      lam[r] = s;
    }
    if (pass == 0) {
      std::vector<double> th(n);
      for (int r = 0; r < n; ++r) th[r] = std::arg(lam[r]);
      std::sort(th.begin(), th.end());
      double best = -1, mid = 0;
      for (int r = 0; r < n; ++r) {
        double lo = th[r], hi = (r + 1 < n) ? th[r + 1] : th[0] + kPi2;
        if (hi - lo > best) {
          best = hi - lo;
          mid = 0.5 * (lo + hi);
        }
      }
      a = kPi - mid;  // W's eigenphases theta + a: the gap midpoint lands on pi
    }
  }
}

// ---------------------------------------------------------------- spin system

// Larmor frequency relative to 1H (src/bloch/Isotope.cc:154-263, 378), quadrupolar nuclei
double isotope_rel_freq(const std::string &iso) {
  static const std::map<std::string, double> t = {
      {"2H", 61.424},   {"6Li", 58.883},  {"7Li", 155.503}, {"9Be", 56.226},   {"10B", 42.99},   {"11B", 128.33},
      {"14N", 28.913},  {"17O", 54.242},  {"21Ne", 31.586}, {"23Na", 105.842}, {"25Mg", 24.496}, {"27Al", 104.262},
      {"33S", 30.714},  {"35Cl", 39.205}, {"37Cl", 32.635}, {"39K", 18.67},    {"43Ca", 26.925}, {"45Sc", 97.2},
      {"47Ti", 22.563}, {"49Ti", 22.557}, {"51V", 105.246}, {"53Cr", 22.615},  {"55Mn", 99.012}, {"59Co", 94.939},
      {"61Ni", 35.756}, {"63Cu", 106.146}, {"65Cu", 113.705}, {"67Zn", 25.036}, {"69Ga", 96.035}, {"71Ga", 122.028},
      {"79Br", 100.249}, {"81Br", 108.063}, {"87Rb", 130.927}, {"93Nb", 97.936}, {"95Mo", 26.076},
      {"115In", 87.68}, {"127I", 80.062}, {"131Xe", 32.811}, {"133Cs", 52.481}};
  auto it = t.find(iso);
  if (it == t.end()) throw std::runtime_error("no relative frequency for isotope " + iso);
  return it->second / 400.13;
}

double isotope_spin(const std::string &iso) {
  // nuclear spin quantum numbers of common NMR isotopes (physical data)
  static const std::map<std::string, double> t = {
      {"1H", 0.5},   {"2H", 1.0},   {"3H", 0.5},   {"3He", 0.5},  {"6Li", 1.0},  {"7Li", 1.5},
      {"9Be", 1.5},  {"10B", 3.0},  {"11B", 1.5},  {"13C", 0.5},  {"14N", 1.0},  {"15N", 0.5},
      {"17O", 2.5},  {"19F", 0.5},  {"21Ne", 1.5}, {"23Na", 1.5}, {"25Mg", 2.5}, {"27Al", 2.5},
      {"29Si", 0.5}, {"31P", 0.5},  {"33S", 1.5},  {"35Cl", 1.5}, {"37Cl", 1.5}, {"39K", 1.5},
      {"43Ca", 3.5}, {"45Sc", 3.5}, {"47Ti", 2.5}, {"49Ti", 3.5}, {"51V", 3.5},  {"53Cr", 1.5},
      {"55Mn", 2.5}, {"57Fe", 0.5}, {"59Co", 3.5}, {"61Ni", 1.5}, {"63Cu", 1.5}, {"65Cu", 1.5},
      {"67Zn", 2.5}, {"69Ga", 1.5}, {"71Ga", 1.5}, {"77Se", 0.5}, {"79Br", 1.5}, {"81Br", 1.5},
      {"87Rb", 1.5}, {"89Y", 0.5},  {"93Nb", 4.5}, {"95Mo", 2.5}, {"103Rh", 0.5}, {"107Ag", 0.5},
      {"109Ag", 0.5}, {"111Cd", 0.5}, {"113Cd", 0.5}, {"115In", 4.5}, {"117Sn", 0.5},
      {"119Sn", 0.5}, {"125Te", 0.5}, {"127I", 2.5}, {"129Xe", 0.5}, {"131Xe", 1.5},
      {"133Cs", 3.5}, {"183W", 0.5}, {"195Pt", 0.5}, {"199Hg", 0.5}, {"205Tl", 0.5},
      {"207Pb", 0.5}, {"e", 0.5}};
  auto it = t.find(iso);
  if (it == t.end()) throw std::runtime_error("unknown isotope " + iso);
  return it->second;
}

struct Interaction {
  char kind;  // 'C' CSA, 'D' dipole, 'J' scalar, 'Q' quadrupole
  double iso = 0, del = 0, eta = 0, a = 0, b = 0, g = 0;
  int s1 = 0, s2 = 0, strong = 0;
  int order = 0;  // quadrupole order column (qua.cc:557-560)
  double PAS[3][3];
};

struct System {
  int nspin = 1;
  std::vector<std::string> iso;
  std::vector<int> dims;
  int N = 1;
  std::vector<CMat> Ix, Iy, Iz, Ip, Im;
  std::vector<Interaction> ints;
  double bfield = 0;  // SolidSys::setBfield (sys.cc:206-210)
  struct Rf {
    std::string iso;
    double amp, phase_deg, offset;
  };
  std::vector<Rf> rf;  // continuous rf during the FID (solid-2.0 PulseData::Pulse)
};

std::vector<std::string> tokens(const std::string &s) {
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

// 3-angle Cartesian rotation (src/QMspins/space_ten.cc:578-618)
void rot3(double a, double b, double g, double R[3][3]) {
  double cg = std::cos(g), cb = std::cos(b), ca = std::cos(a), sg = std::sin(g), sb = std::sin(b),
         sa = std::sin(a);
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

// 2-angle rotor rotation (src/QMspins/space_ten.cc:620-652)
void rot2(double phi, double theta, double R[3][3]) {
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

void mat3mul(const double A[3][3], const double B[3][3], double C[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += A[i][k] * B[k][j];
      C[i][j] = s;
    }
}

// PAS' = rot * diag * rot^T with rot = rot3(alpha,beta,gamma) in degrees
void set_pas(Interaction &it, double d0, double d1, double d2) {
  double R[3][3], D[3][3] = {{d0, 0, 0}, {0, d1, 0}, {0, 0, d2}}, T[3][3], Rt[3][3];
  rot3(it.a * kDeg2Rad, it.b * kDeg2Rad, it.g * kDeg2Rad, R);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Rt[i][j] = R[j][i];
  mat3mul(R, D, T);
  mat3mul(T, Rt, it.PAS);
}

CMat single_op(int hs, char which) {
  CMat m(hs);
  double q = (hs - 1.0) / 2.0, q1 = q * (q + 1.0);
  if (which == 'z') {
    double mm = q;
    for (int k = 0; k < hs; ++k, mm -= 1) m(k, k) = mm;
    return m;
  }
  double mm = q - 1;
  for (int k = 0; k < hs - 1; ++k, mm -= 1) {
    double c = std::sqrt(q1 - mm * (mm + 1));
    switch (which) {
      case 'x': m(k + 1, k) = c / 2; m(k, k + 1) = c / 2; break;
      case 'y': m(k + 1, k) = cplx(0, c / 2); m(k, k + 1) = cplx(0, -c / 2); break;
      case 'p': m(k, k + 1) = c; break;
      case 'm': m(k + 1, k) = c; break;
    }
  }
  return m;
}

CMat expand(const System &S, const CMat &op, int where) {
  CMat out = op;
  for (int i = 0; i < where; ++i) out = kron(identity(S.dims[i]), out);
  for (int i = where + 1; i < S.nspin; ++i) out = kron(out, identity(S.dims[i]));
  return out;
}

System parse_system(const std::vector<std::string> &lines) {
  System S;
  std::vector<std::pair<std::string, int>> types;
  for (auto &l : lines) {
    auto t = tokens(l);
    if (t.size() >= 2 && (t[0] == "numspin" || t[0] == "spins")) S.nspin = std::atoi(t[1].c_str());
    if (t.size() >= 3 && (t[0] == "T" || t[0] == "type" || t[0] == "Type"))
      types.push_back({t[1], std::atoi(t[2].c_str())});
  }
  S.iso.assign(S.nspin, "1H");
  for (auto &p : types)
    if (p.second >= 0 && p.second < S.nspin) S.iso[p.second] = p.first;
  S.dims.resize(S.nspin);
  S.N = 1;
  for (int i = 0; i < S.nspin; ++i) {
    S.dims[i] = int(std::lround(2 * isotope_spin(S.iso[i]) + 1));
    S.N *= S.dims[i];
  }
  for (int i = 0; i < S.nspin; ++i) {
    S.Ix.push_back(expand(S, single_op(S.dims[i], 'x'), i));
    S.Iy.push_back(expand(S, single_op(S.dims[i], 'y'), i));
    S.Iz.push_back(expand(S, single_op(S.dims[i], 'z'), i));
    S.Ip.push_back(expand(S, single_op(S.dims[i], 'p'), i));
    S.Im.push_back(expand(S, single_op(S.dims[i], 'm'), i));
  }
  // interactions in the reference's evaluation order: CSA, dipoles, J, quadrupoles
  // (sys.cc:760-767); the parse order within each kind is file order.
  std::vector<Interaction> csa, dip, jj, qua;
  for (auto &l : lines) {
    auto t = tokens(l);
    if (t.empty() || t[0][0] == '#') continue;
    auto num = [&](size_t i) { return i < t.size() ? std::atof(t[i].c_str()) : 0.0; };
    if ((t[0] == "C" || t[0] == "CSA" || t[0] == "csa") && t.size() >= 5) {
      Interaction it;
      it.kind = 'C';
      it.iso = num(1), it.del = num(2), it.eta = num(3), it.s1 = std::atoi(t[4].c_str());
      it.a = num(5), it.b = num(6), it.g = num(7);
      set_pas(it, it.del * (it.eta - 1.0) / 2.0, -it.del * (it.eta + 1.0) / 2.0, 1.0 * it.del);
      csa.push_back(it);
    } else if ((t[0] == "D" || t[0] == "Dip" || t[0] == "dip" || t[0] == "DIP") && t.size() >= 4) {
      Interaction it;
      it.kind = 'D';
      it.del = num(1), it.s1 = int(num(2)), it.s2 = int(num(3));
      it.a = num(4), it.b = num(5), it.g = num(6);
      double r6 = std::pow(6.0, 0.5);
      set_pas(it, -0.5 * it.del * r6, -0.5 * it.del * r6, 1.0 * it.del * r6);
      dip.push_back(it);
    } else if ((t[0] == "J" || t[0] == "j" || t[0] == "jcop" || t[0] == "Jcop") && t.size() >= 4) {
      Interaction it;
      it.kind = 'J';
      it.iso = num(1), it.s1 = std::atoi(t[2].c_str()), it.s2 = std::atoi(t[3].c_str());
      it.strong = t.size() >= 5 ? std::atoi(t[4].c_str()) : 0;
      jj.push_back(it);
    } else if ((t[0] == "Q" || t[0] == "QUAD" || t[0] == "Quad") && t.size() >= 4) {
      Interaction it;
      it.kind = 'Q';
      it.del = num(1), it.eta = num(2), it.s1 = std::atoi(t[3].c_str());
      it.a = num(4), it.b = num(5), it.g = num(6);
      it.order = t.size() >= 8 ? int(num(7)) : 0;
      set_pas(it, (it.eta - 1.0) / 2.0, -(it.eta + 1.0) / 2.0, 1.0);
      qua.push_back(it);
    }
  }
  for (auto *v : {&csa, &dip, &jj, &qua}) S.ints.insert(S.ints.end(), v->begin(), v->end());
  return S;
}

// H(t1,t2,wr) at rotor phase alpha (sys.cc:749-770) for crystal orientation Rp.
// rf: amp (Ix cos phase + Iy sin phase) + offset Iz on every spin of the isotope, nothing
// when amp == 0 (examples/solid-2.0/src/pulsedata.cc:110-125; phase in degrees, 215)
void add_rf(const System &S, const std::vector<System::Rf> &fields, CMat &H) {
  for (const auto &f : fields) {
    if (f.amp == 0.0) continue;
    const double ph = f.phase_deg * kDeg2Rad;
    for (int sp = 0; sp < S.nspin; ++sp) {
      if (S.iso[sp] != f.iso) continue;
      for (size_t e = 0; e < H.a.size(); ++e)
        H.a[e] += f.amp * (S.Ix[sp].a[e] * std::cos(ph) + S.Iy[sp].a[e] * std::sin(ph)) + f.offset * S.Iz[sp].a[e];
    }
  }
}

CMat hamiltonian(const System &S, const double Rp[3][3], double alpha, double rotb) {
  CMat H(S.N);
  double Rr[3][3], M[3][3];
  rot2(alpha, rotb, Rr);
  mat3mul(Rr, Rp, M);
  const double inv_r3 = 1.0 / std::pow(3., 0.5), r3 = std::pow(3., 0.5);
  for (const auto &it : S.ints) {
    double a = 0;
    if (it.kind != 'J') {
      double T[3][3], Mt[3][3], Rm[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Mt[i][j] = M[j][i];
      mat3mul(M, it.PAS, T);
      mat3mul(T, Mt, Rm);
      a = Rm[2][2];
    }
    if (it.kind == 'C') {
      const CMat &Iz = S.Iz[it.s1];
      if (it.iso != 0) {
        double rot = -r3 * it.iso;
        for (int k = 0; k < S.N; ++k) H(k, k) += (inv_r3 * Iz(k, k).real()) * rot;
      }
      for (int k = 0; k < S.N; ++k) H(k, k) += a * Iz(k, k).real();
    } else if (it.kind == 'D') {
      bool homo = S.iso[it.s1] == S.iso[it.s2];
      CMat T;
      if (homo) {
        CMat t1 = scale(mul(S.Iz[it.s1], S.Iz[it.s2]), 2.0);
        CMat t2 = add(t1, mul(S.Ix[it.s1], S.Ix[it.s2]), -1.0);
        T = scale(add(t2, mul(S.Iy[it.s1], S.Iy[it.s2]), -1.0), std::pow(1. / 6., 0.5));
      } else {
        T = scale(mul(S.Iz[it.s1], S.Iz[it.s2]), std::pow(4. / 6., 0.5));
      }
      H = add(H, T, a);
    } else if (it.kind == 'J') {
      CMat T = mul(S.Iz[it.s1], S.Iz[it.s2]);
      if (it.strong) T = add(add(T, mul(S.Ix[it.s1], S.Ix[it.s2])), mul(S.Iy[it.s1], S.Iy[it.s2]));
      T = scale(T, inv_r3);
      H = add(H, T, it.iso * std::sqrt(3.));
    } else if (it.kind == 'Q') {
      // Qua::get_H (qua.cc:219-267): first order Qp a 3Iz^2; with a field (|B| > 1e-12) and
      // order != 1 the second-order term Qp^2/(B nu_rel) (c4 ((r00-r11)^2/4 + r01^2) -
      // c2 (r02^2 + r12^2)), r = M PAS M^T, c2/c4 = T_QuadTotal (spin_ten.cc:364-375); order 2
      // keeps the second-order term alone
      double spin = isotope_spin(S.iso[it.s1]);
      double Qp = it.del / (4.0 * spin * (2.0 * spin - 1.0));
      const bool first_only = it.order == 1 || std::fabs(S.bfield) <= 1e-12;
      const bool second_only = !first_only && it.order == 2;
      if (!second_only) {
        CMat T = scale(mul(S.Iz[it.s1], S.Iz[it.s1]), 3.0);
        H = add(H, T, Qp * a);
      }
      if (!first_only) {
        double T[3][3], Mt[3][3], Rm[3][3];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) Mt[i][j] = M[j][i];
        mat3mul(M, it.PAS, T);
        mat3mul(T, Mt, Rm);
        const double s2 = Qp * Qp / (S.bfield * isotope_rel_freq(S.iso[it.s1]));
        const double A4 = (Rm[0][0] - Rm[1][1]) * (Rm[0][0] - Rm[1][1]) / 4.0 + Rm[0][1] * Rm[0][1];
        const double A2 = Rm[0][2] * Rm[0][2] + Rm[1][2] * Rm[1][2];
        for (int k = 0; k < S.N; ++k) {
          const double z = S.Iz[it.s1](k, k).real();
          const double c2 = (z * 2.0) * ((-8.0 * (z * z) - 1.0) + 4.0 * spin * (spin + 1));
          const double c4 = (z * 2.0) * ((-2.0 * (z * z) - 1.0) + 2.0 * spin * (spin + 1));
          H(k, k) += s2 * (c4 * A4 - c2 * A2);
        }
      }
    }
  }
  add_rf(S, S.rf, H);
  return H;
}

CMat chop_c(const CMat &x, double eps) {
  CMat z = x;
  for (auto &v : z.a)
    v = cplx(std::fabs(v.real()) < eps ? 0.0 : v.real(), std::fabs(v.imag()) < eps ? 0.0 : v.imag());
  return z;
}

// exp(-i 2 pi tau H) = V chop(exp(mul*lambda)) V^H  (matexp.h:240-252)
CMat step_prop(const CMat &H, double tau) {
  std::vector<double> w;
  CMat V;
  jacobi_herm(H, w, V);
  int n = H.n;
  CMat Ve = V;
  for (int r = 0; r < n; ++r) {
    cplx e = std::exp(cplx(0, -1) * tau * kPi2 * w[r]);
    e = cplx(std::fabs(e.real()) < 1e-12 ? 0.0 : e.real(), std::fabs(e.imag()) < 1e-12 ? 0.0 : e.imag());
    for (int k = 0; k < n; ++k) Ve(k, r) *= e;
  }
  return mul(Ve, adj(V));
}

struct Params {
  int npts = 0;
  double sw = 0, wr = 0, rotb = 0, startT = 0;
};

// compute::calcFID (compute.h:308-461)
std::vector<cplx> calc_fid(const System &S, const std::vector<CMat> &As, int n, double tau, const CMat &ro,
                           const CMat &det, int npts) {
  int N = S.N;
  std::vector<cplx> fid(npts, cplx(0, 0));
  CMat dh = adj(det);
  bool rosym = true;
  for (size_t i = 0; i < ro.a.size(); ++i)
    if (ro.a[i] != 0.5 * (det.a[i] + dh.a[i])) rosym = false;
  std::vector<cplx> lam;
  CMat V;
  unitary_eig(As[n], lam, V);
  std::vector<cplx> ev(N);
  for (int i = 0; i < N; ++i) ev[i] = cplx(std::log(std::abs(lam[i])), std::atan2(lam[i].imag(), lam[i].real()));
  cplx tott(0., double(n) * tau);
  CMat wrs(N);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      cplx v = (ev[i] - ev[j]) / tott;
      wrs(i, j) = cplx(std::fabs(v.real()) < 1e-10 ? 0.0 : v.real(), std::fabs(v.imag()) < 1e-10 ? 0.0 : v.imag());
    }
  std::vector<CMat> Qs(n), Rs(n);
  for (int i = 0; i < n; ++i) {
    Qs[i] = adjprop(V, adjprop(As[i + 1], det));
    if (!rosym) Rs[i] = adjprop(V, adjprop(As[i + 1], ro));
    else Rs[i] = add(Qs[i], adj(Qs[i]));
  }
  // Fave starts from Fz (compute.h:403)
  CMat Fz(N);
  for (int s = 0; s < S.nspin; ++s) Fz = add(Fz, S.Iz[s]);
  std::vector<CMat> Fave(n, Fz);
  for (int i = 0; i < n; ++i)
    for (int p = 0; p < n; ++p) {
      int ind1 = (i + p) % n;
      int ind2 = (i + p) >= n ? p - n : p;
      cplx tmp1(0., -double(ind2) * tau);
      for (int r = 0; r < N; ++r)
        for (int s = 0; s < N; ++s) Fave[p](r, s) += Qs[ind1](r, s) * Rs[i](s, r) * std::exp(tmp1 * wrs(r, s));
    }
  cplx tmp(0., tau);
  CMat step(N), cur(N);
  for (size_t k = 0; k < wrs.a.size(); ++k) step.a[k] = std::exp(tmp * wrs.a[k]);
  cur = step;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) fid[0] += Fave[0](i, j);
  for (int i = 1; i < npts; ++i) {
    int p = i % n;
    for (int r = 0; r < N; ++r)
      for (int s = 0; s < N; ++s) {
        fid[i] += Fave[p](r, s) * cur(r, s);
        cur(r, s) *= step(r, s);
      }
  }
  int ff = rosym ? 2 : 1;
  double sc = double(1. / double(n / ff));
  for (auto &v : fid) v *= sc;
  return fid;
}

// oneFID::singleSpinningFID + compute::FID (oneFID.h:419-431, compute.h:294-306)
std::vector<cplx> single_fid(const System &S, const Params &P, double theta, double phi, double gamma,
                             const CMat &ro, const CMat &det, double &sw_out) {
  int n = int(std::floor(P.sw / P.wr + 0.5));
  int gamma_step = 10, gammaloop = 1;
  if (gamma_step >= n) gammaloop = gamma_step / n;
  if (gammaloop < 1) gammaloop = 1;
  sw_out = double(n * P.wr);
  double tmin = P.startT, tmax = P.startT + 1.0 / P.wr;
  double tau = (tmax - tmin) / n;
  double Rp[3][3];
  rot3(phi, theta, gamma, Rp);  // Rotations::setPowderAngles(phi, theta, gamma)
  double rotb = P.rotb * kDeg2Rad;
  std::vector<cplx> fid(P.npts, cplx(0, 0));
  for (int q = 0; q < gammaloop; ++q) {
    double tadd = kPi2 * double(q) / double(gammaloop * n) / P.wr;
    double t1 = tmin + tadd, t2 = tmin + tadd + tau;
    std::vector<CMat> As(n + 1);
    As[0] = identity(S.N);
    for (int i = 0; i < n; ++i) {
      double tmid = (t2 - t1) / 2.0 + t1;
      CMat H = hamiltonian(S, Rp, tmid * P.wr * kPi2, rotb);
      CMat U = step_prop(H, tau);
      As[i + 1] = mul(U, As[i]);
      t1 += tau;
      t2 += tau;
    }
    auto f = calc_fid(S, As, n, tau, ro, det, P.npts);
    for (int k = 0; k < P.npts; ++k) fid[k] += f[k];
  }
  return fid;
}

std::string trim(const std::string &s) {
  size_t a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  size_t b = s.find_last_not_of(" \t\r\n");
  return s.substr(a, b - a + 1);
}

CMat op_expr(const System &S, const std::string &expr) {
  CMat acc(S.N);
  std::stringstream ss(expr);
  std::string term;
  while (std::getline(ss, term, '+')) {
    term = trim(term);
    double coef = 1.0;
    size_t star = term.find('*');
    if (star != std::string::npos) {
      coef = std::atof(term.substr(0, star).c_str());
      term = trim(term.substr(star + 1));
    }
    std::istringstream is(term);
    std::string name;
    int k = -1;
    is >> name >> k;
    CMat m(S.N);
    auto total = [&](const std::vector<CMat> &v) {
      CMat t(S.N);
      for (auto &x : v) t = add(t, x);
      return t;
    };
    if (name == "Fx") m = total(S.Ix);
    else if (name == "Fy") m = total(S.Iy);
    else if (name == "Fz") m = total(S.Iz);
    else if (name == "Fp") m = total(S.Ip);
    else if (name == "Fm") m = total(S.Im);
    else if (name == "Fe") m = identity(S.N);
    else if (name == "Ix") m = S.Ix.at(k);
    else if (name == "Iy") m = S.Iy.at(k);
    else if (name == "Iz") m = S.Iz.at(k);
    else if (name == "Ip") m = S.Ip.at(k);
    else if (name == "Im") m = S.Im.at(k);
    else throw std::runtime_error("unknown operator " + name);
    acc = add(acc, m, coef);
  }
  return acc;
}

struct Job {
  std::vector<std::string> spin;
  std::string powder;
  Params P;
  std::string rho, det;
  double bfield = 0;
  int p2p_base = 0, p2p_factor = 0;  // point-to-point FID when p2p_base > 0
  double maxtstep = 0;
  std::vector<System::Rf> rf;
  std::vector<std::pair<int, System::Rf>> rfc;  // rf on during one chunk of the period (p2p)
};

Job parse_job(const std::string &text) {
  Job J;
  std::stringstream ss(text);
  std::string line;
  while (std::getline(ss, line)) {
    std::string l = trim(line);
    if (l.empty() || l[0] == '#') continue;
    size_t c = l.find(':');
    if (c == std::string::npos) continue;
    std::string key = trim(l.substr(0, c)), val = trim(l.substr(c + 1));
    if (key == "spin") J.spin.push_back(val);
    else if (key == "powder") J.powder = val;
    else if (key == "npts") J.P.npts = std::atoi(val.c_str());
    else if (key == "sw") J.P.sw = std::atof(val.c_str());
    else if (key == "wr") J.P.wr = std::atof(val.c_str());
    else if (key == "rotb") J.P.rotb = std::atof(val.c_str());
    else if (key == "start") J.P.startT = std::atof(val.c_str());
    else if (key == "rho") J.rho = val;
    else if (key == "det") J.det = val;
    else if (key == "bfield") J.bfield = std::atof(val.c_str());
    else if (key == "p2p") std::sscanf(val.c_str(), "%d %d", &J.p2p_base, &J.p2p_factor);
    else if (key == "maxtstep") J.maxtstep = std::atof(val.c_str());
    else if (key == "rfc") {
      auto t = tokens(val);
      if (t.size() < 3) throw std::runtime_error("rfc: <chunk> <iso> <amp> [phase_deg] [offset]");
      J.rfc.push_back({std::atoi(t[0].c_str()),
                       {t[1], std::atof(t[2].c_str()), t.size() > 3 ? std::atof(t[3].c_str()) : 0.0,
                        t.size() > 4 ? std::atof(t[4].c_str()) : 0.0}});
    } else if (key == "rf") {
      auto t = tokens(val);
      if (t.size() < 2) throw std::runtime_error("rf: <iso> <amp> [phase_deg] [offset]");
      J.rf.push_back({t[0], std::atof(t[1].c_str()), t.size() > 2 ? std::atof(t[2].c_str()) : 0.0,
                      t.size() > 3 ? std::atof(t[3].c_str()) : 0.0});
    }
  }
  return J;
}

// powder::read (powder.cc:333-389): col0 -> phi, col1 -> theta, [col2 -> gamma], last -> weight
void read_powder(const std::string &file, std::vector<double> &th, std::vector<double> &ph, std::vector<double> &ga,
                 std::vector<double> &w) {
  std::ifstream in(file);
  if (!in) throw std::runtime_error("cannot open powder file " + file);
  std::string line;
  while (std::getline(in, line)) {
    auto t = tokens(line);
    if (t.empty() || t[0][0] == '#' || t[0][0] == '%') continue;
    ph.push_back(std::atof(t[0].c_str()));
    th.push_back(t.size() >= 2 ? std::atof(t[1].c_str()) : 0.0);
    if (t.size() == 3) {
      w.push_back(std::atof(t[2].c_str()));
      ga.push_back(0.0);
    } else if (t.size() >= 4) {
      ga.push_back(std::atof(t[2].c_str()));
      w.push_back(std::atof(t[3].c_str()));
    } else {
      w.push_back(1.0);
      ga.push_back(0.0);
    }
  }
}

// oneFID::singleStaticFID (oneFID.h:292-336): H at rotor phase 0 (Hamiltonian(0, dt) with
// wr = 0), one eigen-decomposition, fid[k] = sum A_ij B_ij^k over |A_ij|^2 > 1e-10 with
// A_ij = Do(i,j) sig0(j,i), B_ij = conj(e_i) e_j, e = exp(-2 pi i dt lambda), dt = 1/sw.
std::vector<cplx> single_static_fid(const System &S, const Params &P, double theta, double phi, double gamma,
                                    const CMat &ro, const CMat &det) {
  double dt = 1. / P.sw;
  double Rp[3][3];
  rot3(phi, theta, gamma, Rp);
  CMat H = hamiltonian(S, Rp, 0.0, P.rotb * kDeg2Rad);
  std::vector<double> w;
  CMat V;
  jacobi_herm(H, w, V);
  CMat sig0 = adjprop(V, ro), Do = adjprop(V, det);
  int hs = S.N;
  std::vector<cplx> e(hs), A, B;
  cplx z(0.0, -dt * 2.0 * kPi);
  for (int i = 0; i < hs; ++i) e[i] = std::exp(z * w[i]);
  for (int i = 0; i < hs; ++i)
    for (int j = 0; j < hs; ++j) {
      cplx a = Do(i, j) * sig0(j, i);
      if (std::norm(a) > 1.0e-10) {
        A.push_back(a);
        B.push_back(std::conj(e[i]) * e[j]);
      }
    }
  std::vector<cplx> fid(P.npts);
  for (int k = 0; k < P.npts; ++k) {
    cplx acc = 0;
    for (size_t p = 0; p < A.size(); ++p) {
      acc += A[p];
      A[p] *= B[p];
    }
    fid[k] = acc;
  }
  return fid;
}

// Point-to-point FID of one crystallite, propagated point by point.  A rotor period is cut
// into b chunks (b, f = base, factor over their gcd, as PropReduce::setParams,
// examples/qmsims/MMMQMAS/propreduce.cc:16-33), each the product of ceil(chunk/maxtstep)
// steps exp(-i 2 pi tau H(t)) (propogation.cc:246-296 splitting, compute.h:257-274 step);
// dwell k is the product of chunks (k f + m) mod b, m < f, later chunks on the left (what
// PropReduce::generateProps assembles, propreduce.cc:455-521); rho_{p+1} = W rho_p W^H and
// fid[p] = Tr(rho_p det) / Tr(det det^H) (sequencerun_funcs.cc:624-645).  Static (wr == 0 or
// rotor angle 0): W = exp(-i 2 pi H / sw).
std::vector<cplx> single_p2p_fid(const System &S, const Job &J, double theta, double phi, double gamma,
                                 const CMat &ro, const CMat &det, double &sw_out) {
  const Params &P = J.P;
  int u = J.p2p_base, v = J.p2p_factor;
  if (u <= 0 || v <= 0) throw std::runtime_error("p2p base and factor must be positive");
  while (v) {
    int t = u % v;
    u = v, v = t;
  }
  int b = J.p2p_base / u, f = J.p2p_factor / u;
  if (!J.rfc.empty()) b = J.p2p_base, f = J.p2p_factor;  // the schedule's own chunks
  double Rp[3][3];
  rot3(phi, theta, gamma, Rp);
  const double rotb = P.rotb * kDeg2Rad;
  std::vector<CMat> W;
  if (P.wr == 0.0 || P.rotb == 0.0) {
    CMat H = hamiltonian(S, Rp, 0.0, rotb);
    W.push_back(step_prop(H, 1.0 / P.sw));
    b = f = 1;
    sw_out = P.sw;
  } else {
    const double chunk = 1.0 / (P.wr * b);
    int sub = J.maxtstep > 0 ? int(std::ceil(chunk / J.maxtstep)) : 1;
    if (sub < 1) sub = 1;
    const double tau = chunk / sub;
    std::vector<CMat> U(b);
    for (int k = 0; k < b; ++k) {
      U[k] = identity(S.N);
      for (int j = 0; j < sub; ++j) {
        double t1 = P.startT + double(k * sub + j) * tau;
        double tmid = t1 + tau / 2.0;
        CMat H = hamiltonian(S, Rp, tmid * P.wr * kPi2, rotb);
        for (const auto &rc : J.rfc)
          if (rc.first == k) add_rf(S, {rc.second}, H);
        U[k] = mul(step_prop(H, tau), U[k]);
      }
    }
    for (int k = 0; k < b; ++k) {
      CMat w = identity(S.N);
      for (int m = 0; m < f; ++m) w = mul(U[(k * f + m) % b], w);
      W.push_back(w);
    }
    sw_out = P.wr * b / f;
  }
  double dd = 0;
  for (const auto &x : det.a) dd += std::norm(x);
  std::vector<cplx> fid(P.npts);
  CMat rho = ro;
  for (int p = 0; p < P.npts; ++p) {
    cplx tr = 0;
    for (int r = 0; r < S.N; ++r)
      for (int c = 0; c < S.N; ++c) tr += rho(r, c) * det(c, r);
    fid[p] = tr / dd;
    const CMat &w = W[p % b];
    rho = mul(w, mul(rho, adj(w)));
  }
  return fid;
}

int run(const Job &J, const double *pw, int C, double *out, double *sw_out) {
  System S = parse_system(J.spin);
  S.bfield = J.bfield;
  S.rf = J.rf;
  CMat ro = op_expr(S, J.rho), det = op_expr(S, J.det);
  std::vector<cplx> acc(J.P.npts, cplx(0, 0));
  double sw = J.P.sw;
  const bool stat = J.P.wr == 0.0 || J.P.rotb == 0.0;  // oneFID::FID dispatch (oneFID.h:206)
  for (int c = 0; c < C; ++c) {
    double phi = pw[4 * c + 0], theta = pw[4 * c + 1], gamma = pw[4 * c + 2], w = pw[4 * c + 3];
    std::vector<cplx> f = J.p2p_base > 0 ? single_p2p_fid(S, J, theta, phi, gamma, ro, det, sw)
                          : stat          ? single_static_fid(S, J.P, theta, phi, gamma, ro, det)
                                          : single_fid(S, J.P, theta, phi, gamma, ro, det, sw);
    for (int k = 0; k < J.P.npts; ++k) acc[k] += w * f[k];
  }
  for (int k = 0; k < J.P.npts; ++k) {
    out[2 * k] = acc[k].real();
    out[2 * k + 1] = acc[k].imag();
  }
  if (sw_out) *sw_out = sw;
  return 0;
}

}  // namespace

extern "C" {

// Oracle entry: job text in the ref_harness format (its 'powder:' line is ignored);
// crystallites as C rows of (phi, theta, gamma, weight); out = 2*npts doubles.
// Returns 0 on success, 1 on a parse/math error (message on stderr).
int oracle_powder_fid(const char *job_text, const double *powder4, int C, double *out, double *sw_out) {
  try {
    Job J = parse_job(job_text);
    return run(J, powder4, C, out, sw_out);
  } catch (const std::exception &e) {
    std::fprintf(stderr, "oracle_powder_fid: %s\n", e.what());
    return 1;
  }
}

}  // extern "C"

#ifdef ORACLE_MAIN
// Same command line as oracle/ref_harness.cc: <job file> <output file>
int main(int argc, char **argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: gcompute_ref <job file> <output file>\n");
    return 2;
  }
  std::ifstream in(argv[1]);
  std::stringstream ss;
  ss << in.rdbuf();
  Job J = parse_job(ss.str());
  std::vector<double> th, ph, ga, w;
  read_powder(J.powder, th, ph, ga, w);
  int C = int(th.size());
  std::vector<double> pw(4 * C);
  for (int c = 0; c < C; ++c) pw[4 * c] = ph[c], pw[4 * c + 1] = th[c], pw[4 * c + 2] = ga[c], pw[4 * c + 3] = w[c];
  std::vector<double> out(2 * J.P.npts);
  double sw = 0;
  if (run(J, pw.data(), C, out.data(), &sw) != 0) return 1;
  FILE *f = std::fopen(argv[2], "wb");
  std::fwrite(&sw, sizeof(double), 1, f);
  std::fwrite(out.data(), sizeof(double), out.size(), f);
  std::fclose(f);
  return 0;
}
#endif
