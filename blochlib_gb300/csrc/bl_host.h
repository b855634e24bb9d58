// Host-side model of a BlochLib solid-state spin system (the SolidSys / SpinSys /
// Rotations / powder surface), prepared for the GPU engine.
//
// Reference behaviour mirrored here (paths inside the BlochLib tree):
//   SolidSys::read                    src/QMspins/sys.cc:120-204
//   read_csa / read_dip / read_js /   src/QMspins/csa.cc:400-440, dip.cc:285-323,
//     read_qua                          j.cc:171-202, qua.cc:511-560
//   single-spin and expanded ops      src/QMspins/singlespinop.cc:88-200,
//                                     src/QMspins/multispinop.cc:51-74
//   interaction PAS tensors           csa.cc:223-286, dip.cc:136-169, qua.cc:169-217
//   spin tensors T20/T00/T_Dip/T_J    src/QMspins/spin_ten.cc:211-236, 285-372, 431-465
//   Hamiltonian(t1,t2,wr)             src/QMspins/sys.cc:749-770
//   powder generation / file reader   src/QMspins/driver/powder.cc:179-311, 333-389
//   plotterFID text output            src/utils/plotter.cc:49-135
//   Matlab5 / matstream MAT-5 files   src/utils/matlab5.h:603-792
#pragma once

#include <complex>
#include <cstdint>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace bl {

typedef std::complex<double> cplx;

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// Dense complex N x N matrix, row-major.
struct CMatrix {
  int n = 0;
  std::vector<cplx> a;
  CMatrix() {}
  explicit CMatrix(int n_) : n(n_), a(size_t(n_) * n_) {}
  cplx &operator()(int r, int c) { return a[size_t(r) * n + c]; }
  const cplx &operator()(int r, int c) const { return a[size_t(r) * n + c]; }
};

// One interaction line of the spin-system file.
struct Interaction {
  char kind = 'C';  // 'C' CSA, 'D' dipole, 'J' scalar coupling, 'Q' quadrupole
  double iso = 0, del = 0, eta = 0;
  double alpha = 0, beta = 0, gamma = 0;  // PAS Euler angles, degrees
  int s1 = 0, s2 = 0, strong = 0;
  int order = 0;  // quadrupole: 1 first order, 2 second order only, else both (with a field)
  double pas[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // crystal-frame tensor
  double op_scale = 0;  // H term = op_scale * (R pas R^T)_22 * T
};

// Block structure of every Hamiltonian the system can produce: connected components of
// the union of the non-zero patterns of its operator terms.  All SolidSys terms commute
// with total Fz, so blocks sit inside magnetisation sectors (or finer).
struct BlockLayout {
  int N = 0;
  std::vector<int> size, off, poff;  // per block: dimension, first permuted index, packed offset
  std::vector<int> perm;             // permuted index -> Zeeman index
  std::vector<int> inv;              // Zeeman index -> permuted index
  std::vector<int> block_of;         // permuted index -> block
  int S2 = 0;                        // sum of size^2
  int max_block = 0;
};

// Continuous rf on every spin of one isotope during the whole FID: the pulse Hamiltonian of
// solid-2.0's PulseData::Pulse (examples/solid-2.0/src/pulsedata.cc:110-125),
// amp (Ix cos phase + Iy sin phase) + offset Iz per spin, in Hz and degrees; a field with
// amp == 0 adds nothing (its offset included), as there.
struct RfField {
  std::string iso;
  double amp = 0, phase_deg = 0, offset = 0;
};

class SpinSystem {
 public:
  explicit SpinSystem(const std::vector<std::string> &lines);
  static SpinSystem from_text(const std::string &text);

  int spins() const { return nspin_; }
  int dim() const { return N_; }
  const std::vector<std::string> &isotopes() const { return iso_; }
  const std::vector<Interaction> &interactions() const { return ints_; }

  // Operator from an expression: '+'-separated terms "[coef*]NAME [spin]" with NAME in
  // Fx Fy Fz Fp Fm Fe Ix Iy Iz Ip Im.
  CMatrix op(const std::string &expr) const;
  CMatrix single(char which, int spin) const;  // x y z p m e
  template <class F>
  void pair_terms(int s1, int s2, F f) const;  // two-spin operator products, element by element
  std::vector<double> iz_diag(int s) const;    // diagonal of Iz of spin s

  // Constant part of H (isotropic CSA, J couplings) and the operator multiplying each
  // orientation-dependent interaction (index matches interactions(); zero for J).
  const std::vector<double> &h_const() const { return hc_; }  // N*N real, row-major
  const std::vector<std::vector<double>> &h_ops() const { return hops_; }
  // second-order quadrupolar spin operators of each quadrupole (empty for other kinds):
  // T_QuadTotal(rank 4) and (rank 2) of spin_ten.cc:364-375, both diagonal
  const std::vector<std::vector<double>> &h_ops_q4() const { return hq4_; }
  const std::vector<std::vector<double>> &h_ops_q2() const { return hq2_; }
  // SolidSys::setBfield (sys.cc:206-210): with a field, quadrupoles add their second-order
  // term Qp^2 / (B nu_rel) (c4 ((r00-r11)^2/4 + r01^2) - c2 (r02^2 + r12^2)) (qua.cc:219-267)
  double bfield() const { return bfield_; }
  void set_bfield(double b) { bfield_ = b; }
  // rf fields (rebuilds the operators and the block layout).  The x part of each isotope's
  // summed field is a real constant term of h_const(); a phase off the x axis is carried by
  // the frame R = diag(frame()) = exp(-i phase Fz_iso): the engine propagates the real H'
  // with rho and det taken as R^H X R, exact when the rest of H commutes with Fz_iso (every
  // SolidSys term but a strong J coupling to another isotope; add_rf refuses otherwise).
  void add_rf(const RfField &f);
  const std::vector<RfField> &rf() const { return rf_; }
  const std::vector<cplx> &frame() const { return frame_; }  // empty: no phase frame
  CMatrix to_frame(const CMatrix &X) const;                  // R^H X R
  const BlockLayout &layout() const { return layout_; }

  // Reference-order dense H at rotor phase 'alpha_rot' for powder rotation Rp (for tests).
  std::vector<double> hamiltonian(const double Rp[3][3], double alpha_rot, double rotb_rad) const;

 private:
  void build();
  int nspin_ = 1, N_ = 1;
  std::vector<std::string> iso_;
  std::vector<int> dims_;
  std::vector<Interaction> ints_;
  std::vector<double> hc_;
  std::vector<std::vector<double>> hops_, hq4_, hq2_;
  double bfield_ = 0;
  std::vector<RfField> rf_;
  std::vector<cplx> frame_;
  BlockLayout layout_;
};

double isotope_spin(const std::string &iso);
// Larmor frequency relative to 1H (src/bloch/Isotope.cc:378), quadrupolar isotopes
double isotope_rel_freq(const std::string &iso);

// Cartesian rotations of the reference (src/QMspins/space_ten.cc:578-652)
void rotation3(double a, double b, double g, double R[3][3]);
void rotation2(double phi, double theta, double R[3][3]);

// Powder angle sets (src/QMspins/driver/powder.cc)
struct Powder {
  std::vector<double> theta, phi, gamma, weight;
  int size() const { return int(theta.size()); }
};
Powder powder_zcw(int tstep, int pstep, int gstep);  // powder.cc:248-280 + normalisation
Powder powder_read(const std::string &path);        // powder.cc:333-389 (no renormalisation)

// plotterFID-style 7-column text output (src/utils/plotter.cc:49-135)
void write_fid_text(const std::string &path, const cplx *fid, int npts, double dt);

// MAT-file level 5 writer, the file format of the reference's Matlab5 / matstream
// (src/utils/matlab5.h:603-792): a 128-byte header, then one uncompressed miMATRIX element per
// variable (double matrices, real or complex, and character strings), little endian.
class Mat5Writer {
 public:
  explicit Mat5Writer(const std::string &path);
  // rows x cols in MATLAB (column-major) order; im may be null for a real matrix
  void put_matrix(const std::string &name, const double *re, const double *im, int rows, int cols);
  void put_string(const std::string &name, const std::string &text);

 private:
  std::ofstream f_;
  void bytes(const void *p, size_t n);
  void u32(uint32_t v);
  void pad8(size_t n);
  void name_element(const std::string &name);
};

}  // namespace bl
