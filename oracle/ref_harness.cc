// Runs the BlochLib reference's own spinning powder-FID path on one job file.
//
// Test infrastructure only: this program is compiled against a scratch, build-fixed
// copy of the reference (oracle/build_ref.sh) and is the oracle that pins this
// repository's CPU restatement (oracle/gcompute.cc) and the golden FID fixtures.  It
// is never linked into the product.
//
// Call path exercised (reference files):
//   SolidSys(Vector<string>)            QMspins/sys.cc:40-42, read() 120-204
//   powder::read(file)                  QMspins/driver/powder.cc:333-389
//   oneFID<SolidSys>(sys,npts,sw,wr,rotb)  QMspins/driver/oneFID.h:103-108
//   oneFID::FID(powder, ro, det)        QMspins/driver/oneFID.h:200-208 -> spinningFID 339-410
//
// Job file format (one "key: value" per line, '#' comments):
//   spin: <one line of the reference's spin-system format>   (repeatable, in order)
//   powder: <path of a powder file in the reference's format>
//   powder_zcw: <theta_steps> <phi_steps>      (instead of 'powder:'; powder.cc:248-280)
//   dump_powder: <path>   (writes the powder as C rows of theta phi gamma weight doubles)
//   npts: <int>   sw: <Hz>   wr: <Hz>   rotb: <degrees>   start: <s>
//   bfield: <value passed to SolidSys::setBfield>  (sys.cc:206-210; 0 when absent: a system
//           read from text leaves its field unset, so the harness always sets it)
//   rho: <operator expression>   det: <operator expression>
//   hamgen: <expression>   (repeatable; instead of a FID, writes the matrix the reference's
//           HamiltonianGen (QMspins/driver/ham_gen.cc) evaluates for each expression, at the
//           angles of 'hamgen_angles: <theta> <phi> <gamma>' (radians, default 0 0 0))
//   rf: <iso> <amp Hz> [phase deg] [offset Hz]   (repeatable: continuous rf during the FID,
//           added to SolidSys::Hamiltonian by RfSys below, as solid-2.0's PulseData::Pulse)
//   rfc: <chunk> <iso> <amp Hz> [phase deg] [offset Hz]   (p2p only, repeatable: rf on during
//           one chunk of every rotor period; base and factor are then used as given)
//   writers: <fid binary> <npts> <dt> <text out> <mat out>   (instead of a FID: reads npts
//           (re, im) doubles and writes them with the reference's own writers, plotterFID
//           (utils/plotter.cc:49-135) to <text out> and Matlab5/matstream
//           (utils/matlab5.h:700-721, matlab5.cc) to <mat out> as the complex column vector
//           'vdat' and the real scalar 'dt'; the output file argument is then unused)
//   p2p: <base> <factor>   maxtstep: <s>   (point-to-point FID instead of oneFID::FID: see
//           p2p_fid below; a rotor period in 'base' chunks of ceil(chunk/maxtstep) steps,
//           a point every 'factor' chunks)
// An operator expression is a '+'-separated sum of terms "[coef*]NAME [spin]" with NAME
// one of Fx Fy Fz Fp Fm Fe Ix Iy Iz Ip Im (single-spin names take a spin index).
//
// Output (argv[2]): little-endian doubles: sw_out, then npts (re, im) pairs.
#include "mpi/mpi_controller.h"
#include "QMspins/sys.h"
#include "QMspins/driver/oneFID.h"
#include "propreduce.h"  // examples/qmsims/MMMQMAS (scratch copy, built by oracle/ref.mk)
#include "QMspins/driver/ham_gen.h"
#include "utils/plotter.h"
#include "utils/matlab5.h"

#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

using namespace BlochLib;

static std::string trim(const std::string &s) {
  size_t a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  size_t b = s.find_last_not_of(" \t\r\n");
  return s.substr(a, b - a + 1);
}

static matrix op_term(SolidSys &sys, const std::string &term_in) {
  std::string term = trim(term_in);
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
  matrix m;
  if (name == "Fx") m = sys.Fx();
  else if (name == "Fy") m = sys.Fy();
  else if (name == "Fz") m = sys.Fz();
  else if (name == "Fp") m = sys.Fp();
  else if (name == "Fm") m = sys.Fmi();
  else if (name == "Fe") m = sys.Fe();
  else if (name == "Ix") m = sys.Ix(k);
  else if (name == "Iy") m = sys.Iy(k);
  else if (name == "Iz") m = sys.Iz(k);
  else if (name == "Ip") m = sys.Ip(k);
  else if (name == "Im") m = sys.Imi(k);
  else {
    std::cerr << "ref_harness: unknown operator '" << name << "'\n";
    std::exit(2);
  }
  if (coef != 1.0) m = coef * m;
  return m;
}

static matrix op_expr(SolidSys &sys, const std::string &expr) {
  matrix acc;
  bool first = true;
  size_t pos = 0;
  while (pos <= expr.size()) {
    size_t plus = expr.find('+', pos);
    std::string t = expr.substr(pos, plus == std::string::npos ? std::string::npos : plus - pos);
    matrix m = op_term(sys, t);
    if (first) { acc = m; first = false; }
    else acc = acc + m;
    if (plus == std::string::npos) break;
    pos = plus + 1;
  }
  return acc;
}

struct RfSpec {
  std::string iso;
  double amp, phase_deg, offset;
};

// SolidSys with continuous rf: the Func_T that oneFID and compute are templated on (they call
// setRotorAngles, setPowderAngles, Hamiltonian, Fe, Fz: oneFID.h:299-301, compute.h:206,
// 265, 403), with the rf term built as PulseData::Pulse builds it
// (examples/solid-2.0/src/pulsedata.cc:110-125; phase in degrees, pulsedata.cc:215).
class RfSys {
 public:
  RfSys(SolidSys &s, const std::vector<RfSpec> &rf) : s_(&s) {
    matrix tm = s.F0();
    for (size_t j = 0; j < rf.size(); ++j) {
      if (rf[j].amp == 0) continue;
      const double ph = rf[j].phase_deg * DEG2RAD;
      for (int i = 0; i < s.size(); ++i)
        if (s.symbol(i) == rf[j].iso)
          tm += rf[j].amp * (s.Ix(i) * cos(ph) + s.Iy(i) * sin(ph)) + rf[j].offset * s.Iz(i);
    }
    P_ = tm;
  }
  void setRotorAngles(double a, double b) { s_->setRotorAngles(a, b); }
  void setPowderAngles(double t, double p, double g) { s_->setPowderAngles(t, p, g); }
  hmatrix &Hamiltonian(double t1, double t2, double wr = 0.0) {
    H_ = s_->Hamiltonian(t1, t2, wr);
    H_ += P_;
    return H_;
  }
  rimatrix &Fe() { return s_->Fe(); }
  rdmatrix &Fz() { return s_->Fz(); }

 private:
  SolidSys *s_;
  hmatrix P_, H_;
};

// Point-to-point powder FID assembled from the reference's own pieces: chunk propagators as
// products of Mexp(SolidSys::Hamiltonian(t1,t2,wr), -i tau 2pi) with later steps on the left
// (compute.h:257-274 convention; chunk loop of mmmqmas.cc:315-330), the forward and back
// products that PropReduce documents (propreduce.h:88-97), the dwell propagators from
// PropReduce::reduce + generateProps (propreduce.cc:455-521) where reduce terminates (base <
// factor; otherwise the direct products of the same chunks), rho stepped as A rho A^H
// and trace(rho, det)/trace(det, adjoint(det)) summed per point with the powder weight
// (sequencerun_funcs.cc:624-645).  Static (wr == 0 or rotor angle 0): one Mexp of 1/sw.
static Vector<complex> p2p_fid(SolidSys &sys, RfSys &hs, const std::vector<RfSpec> &rf,
                               const std::vector<std::pair<int, RfSpec> > &rfc, powder &pw, matrix &ro, matrix &det,
                               int npts, double sw, double wr, double rotb, double start, int base, int factor,
                               double maxtstep, double &sw_out) {
  PropReduce red(base, factor);  // divides base and factor by their gcd (propreduce.cc:16-33)
  const int b = rfc.empty() ? red.base : base, f = rfc.empty() ? red.factor : factor;
  // per chunk: the continuous fields plus the chunk's own (solid-2.0's pulse list, one pulse
  // per chunk, propogation.cc:246-296)
  std::vector<RfSys *> hk;
  if (!rfc.empty())
    for (int k = 0; k < b; ++k) {
      std::vector<RfSpec> fk = rf;
      for (size_t j = 0; j < rfc.size(); ++j)
        if (rfc[j].first == k) fk.push_back(rfc[j].second);
      hk.push_back(new RfSys(sys, fk));
    }
  // PropReduce::reduce terminates only for base < factor: setParams sizes BackRed to base-1
  // but fills min(base, factor)-1 entries, and an empty entry matches every sequence in
  // iteration(), so backReduce's while loop never ends when base > factor.  There (and for
  // base == 1) the dwell products are formed directly, in the same order.
  const bool use_red = b > 1 && b < f && rfc.empty();
  if (use_red) red.reduce();
  const bool stat = wr == 0.0 || rotb == 0.0;
  Vector<complex> fid(npts, complex(0, 0));
  complex nrm = trace(det, adjoint(det));
  powder::iterator it(pw);
  while (it) {
    sys.setRotorAngles(0.0, rotb * DEG2RAD);
    sys.setPowderAngles(it.theta(), it.phi(), it.gamma());
    Vector<matrix> W;
    int nb = b;
    if (stat) {
      double dt = 1.0 / sw;
      nb = 1;
      W.resize(1);
      W[0] = Mexp(hs.Hamiltonian(0.0, dt, 0.0), -complexi * dt * PI2);
      sw_out = sw;
    } else {
      const double chunk = 1.0 / (wr * b);
      int sub = maxtstep > 0 ? int(std::ceil(chunk / maxtstep)) : 1;
      if (sub < 1) sub = 1;
      const double tau = chunk / sub;
      Vector<matrix> U(b);
      for (int k = 0; k < b; ++k) {
        U[k] = sys.Fe();
        for (int j = 0; j < sub; ++j) {
          double t1 = start + double(k * sub + j) * tau;
          RfSys &h = rfc.empty() ? hs : *hk[k];
          U[k] = Mexp(h.Hamiltonian(t1, t1 + tau, wr), -complexi * tau * PI2) * U[k];
        }
      }
      W.resize(b);
      if (!use_red) {
        for (int k = 0; k < b; ++k) {
          W[k] = U[(k * f) % b];
          for (int m = 1; m < f; ++m) W[k] = U[(k * f + m) % b] * W[k];
        }
      } else {
        Vector<matrix> Fow(b - 1), Back(red.maxBackReduce());
        Fow[0] = U[1] * U[0];  // "0*1", "0*1*2", ...
        for (int i = 2; i < b; ++i) Fow[i - 1] = U[i] * Fow[i - 2];
        if (Back.size() > 0) Back[0] = U[b - 1] * U[b - 2];  // "b-2 b-1", "b-3 b-2 b-1", ...
        for (int i = 1; i < Back.size(); ++i) Back[i] = Back[i - 1] * U[b - 2 - i];
        red.generateProps(U, Fow, Back, W);
      }
      sw_out = wr * b / f;
    }
    matrix r = ro;
    for (int p = 0; p < npts; ++p) {
      fid[p] += it.weight() * trace(r, det) / nrm;
      r = W[p % nb] * r * adjoint(W[p % nb]);  // prop (A rho A^H); the member form does not
                                               // compile (its own adjoint() hides the free one)
    }
    ++it;
  }
  for (size_t k = 0; k < hk.size(); ++k) delete hk[k];
  return fid;
}

int main(int argc, char **argv) {
  if (argc < 3) {
    std::cerr << "usage: ref_harness <job file> <output file>\n";
    return 2;
  }
  std::ifstream in(argv[1]);
  if (!in) { std::cerr << "ref_harness: cannot open " << argv[1] << "\n"; return 2; }
  Vector<std::string> spin_lines;
  std::string powder_file, rho_s, det_s, dump_file;
  int npts = 0, zcw_t = 0, zcw_p = 0;
  double sw = 0, wr = 0, rotb = 0, start = 0, bfield = 0, maxtstep = 0;
  std::vector<RfSpec> rf;
  std::vector<std::pair<int, RfSpec> > rfc;
  int p2p_base = 0, p2p_factor = 0;
  std::vector<std::string> hamgen;
  double hg_theta = 0, hg_phi = 0, hg_gamma = 0;
  std::string line;
  while (std::getline(in, line)) {
    std::string l = trim(line);
    if (l.empty() || l[0] == '#') continue;
    size_t c = l.find(':');
    if (c == std::string::npos) continue;
    std::string key = trim(l.substr(0, c)), val = trim(l.substr(c + 1));
    if (key == "spin") spin_lines.push_back(val + "\n");
    else if (key == "powder") powder_file = val;
    else if (key == "powder_zcw") std::sscanf(val.c_str(), "%d %d", &zcw_t, &zcw_p);
    else if (key == "dump_powder") dump_file = val;
    else if (key == "start") start = std::atof(val.c_str());
    else if (key == "npts") npts = std::atoi(val.c_str());
    else if (key == "sw") sw = std::atof(val.c_str());
    else if (key == "wr") wr = std::atof(val.c_str());
    else if (key == "rotb") rotb = std::atof(val.c_str());
    else if (key == "bfield") bfield = std::atof(val.c_str());
    else if (key == "rho") rho_s = val;
    else if (key == "det") det_s = val;
    else if (key == "p2p") std::sscanf(val.c_str(), "%d %d", &p2p_base, &p2p_factor);
    else if (key == "maxtstep") maxtstep = std::atof(val.c_str());
    else if (key == "hamgen") hamgen.push_back(val);
    else if (key == "rfc") {
      RfSpec r = {"", 0, 0, 0};
      char iso[32] = {0};
      int ch = -1;
      std::sscanf(val.c_str(), "%d %31s %lf %lf %lf", &ch, iso, &r.amp, &r.phase_deg, &r.offset);
      r.iso = iso;
      rfc.push_back(std::make_pair(ch, r));
    } else if (key == "rf") {
      RfSpec r = {"", 0, 0, 0};
      char iso[32] = {0};
      std::sscanf(val.c_str(), "%31s %lf %lf %lf", iso, &r.amp, &r.phase_deg, &r.offset);
      r.iso = iso;
      rf.push_back(r);
    }
    else if (key == "hamgen_angles") std::sscanf(val.c_str(), "%lf %lf %lf", &hg_theta, &hg_phi, &hg_gamma);
    else if (key == "writers") {
      char fin[512] = {0}, ftxt[512] = {0}, fmat[512] = {0};
      int n = 0;
      double dt = 1;
      std::sscanf(val.c_str(), "%511s %d %lf %511s %511s", fin, &n, &dt, ftxt, fmat);
      FILE *fi = std::fopen(fin, "rb");
      if (!fi || n <= 0) { std::cerr << "ref_harness: bad writers line\n"; return 2; }
      Vector<complex> v(n, complex(0, 0));
      for (int k = 0; k < n; ++k) {
        double re = 0, im = 0;
        if (std::fread(&re, sizeof(double), 1, fi) != 1 || std::fread(&im, sizeof(double), 1, fi) != 1) {
          std::cerr << "ref_harness: short FID file\n";
          return 2;
        }
        v(k) = complex(re, im);
      }
      std::fclose(fi);
      plotterFID(v, std::string(ftxt), dt);
      matstream ms(fmat, std::ios::binary | std::ios::out);
      ms.put("vdat", v);
      ms.put("dt", dt);
      ms.close();
      return 0;
    }
  }
  SolidSys sys(spin_lines);
  sys.setBfield(bfield);
  if (!hamgen.empty()) {  // output: per expression, N then N*N (re, im) row-major
    FILE *f = std::fopen(argv[2], "wb");
    if (!f) { std::cerr << "ref_harness: cannot write " << argv[2] << "\n"; return 2; }
    for (size_t k = 0; k < hamgen.size(); ++k) {
      HamiltonianGen gen;
      matrix m = gen.Hamiltonian(sys, hamgen[k], hg_theta, hg_phi, hg_gamma);
      double nd = m.rows();
      std::fwrite(&nd, sizeof(double), 1, f);
      for (int r = 0; r < m.rows(); ++r)
        for (int c = 0; c < m.cols(); ++c) {
          double re = Re(m(r, c)), im = Im(m(r, c));
          std::fwrite(&re, sizeof(double), 1, f);
          std::fwrite(&im, sizeof(double), 1, f);
        }
    }
    std::fclose(f);
    return 0;
  }
  powder pw;
  if (zcw_t > 0) pw = powder(powder::zcw, zcw_t, zcw_p);
  else pw.read(powder_file);
  if (!dump_file.empty()) {
    FILE *fp = std::fopen(dump_file.c_str(), "wb");
    powder::iterator it(pw);
    while (it) {
      double row[4] = {it.theta(), it.phi(), it.gamma(), it.weight()};
      std::fwrite(row, sizeof(double), 4, fp);
      ++it;
    }
    std::fclose(fp);
  }
  matrix ro = op_expr(sys, rho_s);
  matrix det = op_expr(sys, det_s);
  Vector<complex> fid;
  double sw_out = sw;
  RfSys hs(sys, rf);
  if (p2p_base > 0) {
    fid = p2p_fid(sys, hs, rf, rfc, pw, ro, det, npts, sw, wr, rotb, start, p2p_base, p2p_factor, maxtstep, sw_out);
  } else if (!rf.empty()) {
    oneFID<RfSys> driver(hs, npts, sw, wr, rotb, start);
    fid = driver.FID(pw, ro, det);
    sw_out = driver.sw();
  } else {
    oneFID<SolidSys> driver(sys, npts, sw, wr, rotb, start);
    fid = driver.FID(pw, ro, det);
    sw_out = driver.sw();
  }
  FILE *f = std::fopen(argv[2], "wb");
  if (!f) { std::cerr << "ref_harness: cannot write " << argv[2] << "\n"; return 2; }
  std::fwrite(&sw_out, sizeof(double), 1, f);
  for (int i = 0; i < fid.size(); ++i) {
    double re = Re(fid[i]), im = Im(fid[i]);
    std::fwrite(&re, sizeof(double), 1, f);
    std::fwrite(&im, sizeof(double), 1, f);
  }
  std::fclose(f);
  return 0;
}
