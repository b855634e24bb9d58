// blochlib_gb300 C++ host API: the BlochLib classes a powder-FID program uses, with the
// reference's names and argument meaning, over the C ABI of blochlib_gb300.h.  Header only;
// link with -lblochlib_gb300.  Errors throw bl_error (the reference raises SIGINT or
// throws BL_exception, src/utils/blassert.h:66-78).
//
//   SolidSys(Vector<string>)           src/QMspins/sys.cc:40-42, read 120-204
//   SolidSys::Fx() ... Imi(k)          src/QMspins/spinsys.h:143-162
//   Rotations (Cartesian)              src/QMspins/space_ten.h:60-111, space_ten.cc:578-805
//   powder(powder::zcw, t, p, g)       src/QMspins/driver/powder.cc:94-113, 248-280
//   powder(file)                       src/QMspins/driver/powder.cc:333-389
//   oneFID<SolidSys>(sys, npts, sw, wr, rotb, startT), FID(powder, ro, det)
//                                      src/QMspins/driver/oneFID.h:103-108, 200-208
//   plotterFID(fid, file, dt)          src/utils/plotter.cc:49-135
//   matstream / Matlab5 put(name, x)   src/utils/matlab5.h:603-792
#ifndef BLOCHLIB_GB300_HPP
#define BLOCHLIB_GB300_HPP

#include <complex>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "blochlib_gb300.h"

namespace blochlib_gb300 {

typedef std::complex<double> complex;

struct bl_error : std::runtime_error {
  bl_status status;
  bl_error(bl_status s, const std::string &m) : std::runtime_error(m), status(s) {}
};

inline void check(bl_status s) {
  if (s != BL_OK) throw bl_error(s, bl_last_error());
}

// Dense complex N x N operator, row-major (the ABI layout).
struct matrix {
  int n = 0;
  std::vector<complex> a;
  matrix() {}
  explicit matrix(int n_) : n(n_), a(size_t(n_) * n_) {}
  complex &operator()(int r, int c) { return a[size_t(r) * n + c]; }
  const complex &operator()(int r, int c) const { return a[size_t(r) * n + c]; }
  int rows() const { return n; }
  int cols() const { return n; }
  const double *data() const { return reinterpret_cast<const double *>(a.data()); }
};

inline matrix operator+(const matrix &x, const matrix &y) {
  matrix z = x;
  for (size_t i = 0; i < z.a.size(); ++i) z.a[i] += y.a[i];
  return z;
}
inline matrix operator*(double s, const matrix &x) {
  matrix z = x;
  for (auto &v : z.a) v *= s;
  return z;
}

// One CUDA device and stream shared by the objects below (created on first use).
class Context {
 public:
  static bl_ctx *get(int device = 0, size_t hbm_budget = 0) {
    static Context c(device, hbm_budget);
    return c.h_;
  }
  ~Context() { bl_ctx_destroy(h_); }

 private:
  Context(int device, size_t budget) { check(bl_ctx_create(device, budget, &h_)); }
  bl_ctx *h_ = nullptr;
};

class SolidSys {
 public:
  explicit SolidSys(const std::vector<std::string> &lines) {
    std::string text;
    for (const auto &l : lines) text += l + "\n";
    check(bl_system_create(text.c_str(), &h_));
  }
  SolidSys(const SolidSys &) = delete;
  SolidSys &operator=(const SolidSys &) = delete;
  ~SolidSys() { bl_system_destroy(h_); }
  int HS() const { return bl_system_dim(h_); }
  int spins() const { return bl_system_spins(h_); }
  // sys.cc:206-210: second-order quadrupolar terms (qua.cc:219-267) with a field
  void setBfield(double Bf) { check(bl_system_set_bfield(h_, Bf)); }
  // continuous rf during the FID (solid-2.0 PulseData::Pulse, pulsedata.cc:110-125)
  void addRf(const std::string &iso, double amp, double phase_deg = 0, double offset = 0) {
    check(bl_system_add_rf(h_, iso.c_str(), amp, phase_deg, offset));
  }
  matrix op(const std::string &expr) const {
    matrix m(HS());
    check(bl_system_operator(h_, expr.c_str(), reinterpret_cast<double *>(m.a.data())));
    return m;
  }
  matrix Fx() const { return op("Fx"); }
  matrix Fy() const { return op("Fy"); }
  matrix Fz() const { return op("Fz"); }
  matrix Fp() const { return op("Fp"); }
  matrix Fmi() const { return op("Fm"); }
  matrix Fe() const { return op("Fe"); }
  matrix Ix(int k) const { return op("Ix " + std::to_string(k)); }
  matrix Iy(int k) const { return op("Iy " + std::to_string(k)); }
  matrix Iz(int k) const { return op("Iz " + std::to_string(k)); }
  matrix Ip(int k) const { return op("Ip " + std::to_string(k)); }
  matrix Imi(int k) const { return op("Im " + std::to_string(k)); }
  const bl_system *handle() const { return h_; }

 private:
  bl_system *h_ = nullptr;
};

// Cartesian rotations of the reference: R(alpha, beta, gamma) for the crystallite and
// R(phi, theta) for the rotor; rotor phase and powder angles in radians.
class Rotations {
 public:
  double alpha = 0, beta = 0, theta = 0, phi = 0, gamma = 0;
  double cartPowder[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  double cartSpin[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  void setPowderAngles(double phi_, double theta_, double gamma_) {
    phi = phi_, theta = theta_, gamma = gamma_;
    check(bl_rotation3(phi, theta, gamma, cartPowder));
  }
  void setRotorAngles(double alpha_, double beta_) {
    alpha = alpha_, beta = beta_;
    check(bl_rotation2(alpha, beta, cartSpin));
  }
};

class powder {
 public:
  enum pTypes { zcw };
  powder(pTypes, int tstep, int pstep, int gstep = 0) { check(bl_powder_zcw(tstep, pstep, gstep, &h_)); }
  explicit powder(const std::string &file) { check(bl_powder_read(file.c_str(), &h_)); }
  powder(const std::vector<double> &theta, const std::vector<double> &phi, const std::vector<double> &gamma,
         const std::vector<double> &weight) {
    check(bl_powder_from_arrays(theta.data(), phi.data(), gamma.data(), weight.data(), int(theta.size()), &h_));
  }
  powder(const powder &) = delete;
  powder &operator=(const powder &) = delete;
  ~powder() { bl_powder_destroy(h_); }
  int size() const { return bl_powder_size(h_); }
  void angles(std::vector<double> &theta, std::vector<double> &phi, std::vector<double> &gamma,
              std::vector<double> &weight) const {
    int n = size();
    theta.resize(n), phi.resize(n), gamma.resize(n), weight.resize(n);
    check(bl_powder_get(h_, theta.data(), phi.data(), gamma.data(), weight.data()));
  }
  const bl_powder *handle() const { return h_; }

 private:
  bl_powder *h_ = nullptr;
};

// HamiltonianGen (src/QMspins/driver/ham_gen.h): "Ix_0 + complexi*Iy_1", "T2m1_0,1*A21", ...
// evaluated for a system at powder angles (theta, phi); see bl_hamgen for the grammar.
class HamiltonianGen {
 public:
  void addVar(const std::string &name, complex v) { vars_.push_back({name, v}); }
  matrix Hamiltonian(const SolidSys &sys, const std::string &expr, double theta = 0, double phi = 0,
                     double gamma = 0) const {
    std::vector<const char *> names;
    std::vector<double> vals;
    for (const auto &v : vars_) names.push_back(v.first.c_str()), vals.push_back(v.second.real()),
        vals.push_back(v.second.imag());
    matrix m(sys.HS());
    check(bl_hamgen(sys.handle(), expr.c_str(), theta, phi, gamma, names.data(), vals.data(), int(vars_.size()),
                    reinterpret_cast<double *>(m.a.data())));
    return m;
  }

 private:
  std::vector<std::pair<std::string, complex>> vars_;
};

// PropReduce(base, factor) (examples/qmsims/MMMQMAS/propreduce.cc:16-60): a rotor period in
// 'base' chunks, a dwell of 'factor' chunks, both divided by their gcd.  The dwell propagators
// it would assemble are never formed here: oneFID::p2pFID takes the pair.
class PropReduce {
 public:
  int base = 1, factor = 1;
  PropReduce() {}
  PropReduce(int bas, int fac) { setParams(bas, fac); }
  void setParams(int bas, int fac) {
    if (bas <= 0 || fac <= 0) throw std::invalid_argument("PropReduce: base and factor must be positive");
    int u = bas, v = fac;
    while (v) {
      int t = u % v;
      u = v, v = t;
    }
    base = bas / u, factor = fac / u;
  }
};

template <class Func_T = SolidSys>
class oneFID {
 public:
  oneFID(Func_T &sys, int npts, double sw = 20000, double wr = 0, double rotb = 0, double startT = 0)
      : sys_(&sys), npts_(npts), sw_(sw), wr_(wr), rotb_(rotb), startT_(startT) {}
  std::vector<complex> FID(powder &pw, const matrix &ro, const matrix &det) {
    bl_fid_params p = {npts_, sw_, wr_, rotb_, startT_, 0, /*Taylor step*/ 1, 0};
    std::vector<complex> fid(static_cast<size_t>(npts_));
    double sw_used = sw_;
    check(bl_powder_fid(Context::get(), sys_->handle(), pw.handle(), ro.data(), det.data(), &p,
                        reinterpret_cast<double *>(fid.data()), &sw_used));
    sw_ = sw_used;  // as the reference, sw becomes n * wr (oneFID.h:429)
    fid_ = fid;
    return fid;
  }
  // Point-to-point FID every red.factor/red.base rotor periods, steps of at most maxtstep
  // (bl_p2p_fid); sw becomes base*wr/factor.
  // rf fields on during one chunk of every rotor period (base and factor then as given)
  struct RfChunk {
    int chunk;
    std::string iso;
    double amp, phase_deg, offset;
  };
  std::vector<complex> p2pFID(powder &pw, const matrix &ro, const matrix &det, const PropReduce &red,
                              double maxtstep = 0, const std::vector<RfChunk> &rf = {}) {
    std::vector<bl_rf_chunk> sched;
    for (const auto &r : rf) sched.push_back({r.chunk, r.iso.c_str(), r.amp, r.phase_deg, r.offset});
    bl_p2p_params p = {npts_, sw_, wr_, rotb_, startT_, 0, /*Taylor step*/ 1, red.base, red.factor, maxtstep,
                       sched.empty() ? nullptr : sched.data(), int(sched.size())};
    std::vector<complex> fid(static_cast<size_t>(npts_));
    double sw_used = sw_;
    check(bl_p2p_fid(Context::get(), sys_->handle(), pw.handle(), ro.data(), det.data(), &p,
                     reinterpret_cast<double *>(fid.data()), &sw_used));
    sw_ = sw_used;
    fid_ = fid;
    return fid;
  }
  double sw() const { return sw_; }
  double wr() const { return wr_; }
  double rotorAngle() const { return rotb_; }
  int npts() const { return npts_; }
  void setSw(double v) { sw_ = v; }
  void setWr(double v) { wr_ = v; }
  void setRotorAngle(double v) { rotb_ = v; }
  const std::vector<complex> &fid() const { return fid_; }

 private:
  Func_T *sys_;
  int npts_;
  double sw_, wr_, rotb_, startT_;
  std::vector<complex> fid_;
};

inline std::string plotterFID(const std::vector<complex> &fid, const std::string &datasave = "fid", double dt = 1) {
  check(bl_plotter_fid(reinterpret_cast<const double *>(fid.data()), int(fid.size()), datasave.c_str(), dt));
  return datasave;
}

// MAT-5 output (src/utils/matlab5.h:603-792, `typedef Matlab5 matstream`): put(name, x)
// appends a scalar, a vector (column), a matrix or a string.
class matstream {
 public:
  explicit matstream(const std::string &fname) { check(bl_mat5_open(fname.c_str(), &h_)); }
  ~matstream() { bl_mat5_close(h_); }
  matstream(const matstream &) = delete;
  matstream &operator=(const matstream &) = delete;
  void put(const std::string &name, double x) { check(bl_mat5_put(h_, name.c_str(), &x, 1, 1, 0)); }
  void put(const std::string &name, complex x) {
    check(bl_mat5_put(h_, name.c_str(), reinterpret_cast<const double *>(&x), 1, 1, 1));
  }
  void put(const std::string &name, const std::vector<double> &v) {
    check(bl_mat5_put(h_, name.c_str(), v.data(), int(v.size()), 1, 0));
  }
  void put(const std::string &name, const std::vector<complex> &v) {
    check(bl_mat5_put(h_, name.c_str(), reinterpret_cast<const double *>(v.data()), int(v.size()), 1, 1));
  }
  void put(const std::string &name, const matrix &m) { check(bl_mat5_put(h_, name.c_str(), m.data(), m.n, m.n, 1)); }
  void put(const std::string &name, const std::string &text) {
    check(bl_mat5_put_string(h_, name.c_str(), text.c_str()));
  }
  void put(const std::string &name, const char *text) { put(name, std::string(text)); }

 private:
  bl_mat5 *h_ = nullptr;
};
typedef matstream Matlab5;

}  // namespace blochlib_gb300

#endif  // BLOCHLIB_GB300_HPP
