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
// An operator expression is a '+'-separated sum of terms "[coef*]NAME [spin]" with NAME
// one of Fx Fy Fz Fp Fm Fe Ix Iy Iz Ip Im (single-spin names take a spin index).
//
// Output (argv[2]): little-endian doubles: sw_out, then npts (re, im) pairs.
#include "mpi/mpi_controller.h"
#include "QMspins/sys.h"
#include "QMspins/driver/oneFID.h"

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
  double sw = 0, wr = 0, rotb = 0, start = 0, bfield = 0;
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
  }
  SolidSys sys(spin_lines);
  sys.setBfield(bfield);
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
  oneFID<SolidSys> driver(sys, npts, sw, wr, rotb, start);
  Vector<complex> fid = driver.FID(pw, ro, det);
  FILE *f = std::fopen(argv[2], "wb");
  if (!f) { std::cerr << "ref_harness: cannot write " << argv[2] << "\n"; return 2; }
  double sw_out = driver.sw();
  std::fwrite(&sw_out, sizeof(double), 1, f);
  for (int i = 0; i < fid.size(); ++i) {
    double re = Re(fid[i]), im = Im(fid[i]);
    std::fwrite(&re, sizeof(double), 1, f);
    std::fwrite(&im, sizeof(double), 1, f);
  }
  std::fclose(f);
  return 0;
}
