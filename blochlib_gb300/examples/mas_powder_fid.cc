// A BlochLib-style powder FID program on the GB300 engine: the same steps as the
// reference's canonical caller (examples/qmsims/simple90.cc:12-49) through the C++ host
// API of blochlib_gb300.hpp.
//
//   mas_powder_fid <npts> <sw Hz> <wr Hz> <rotor angle deg> <zcw theta steps> <zcw phi steps> <out file>
#include <cstdio>
#include <cstdlib>
#include <iostream>

#include "blochlib_gb300.hpp"

using namespace blochlib_gb300;

int main(int argc, char **argv) {
  if (argc < 8) {
    std::cerr << "usage: mas_powder_fid npts sw wr rotb zcw_t zcw_p out\n";
    return 2;
  }
  int npts = std::atoi(argv[1]);
  double sw = std::atof(argv[2]), wr = std::atof(argv[3]), beta = std::atof(argv[4]);
  int thd = std::atoi(argv[5]), phs = std::atoi(argv[6]);
  std::vector<std::string> spinl = {
      "numspin 3", "T 1H 0", "T 1H 1", "T 1H 2",
      "C 1243 1548 0.3 0 10 20 30", "C -4561 3215 0.5 1 40 50 60", "C 200 2500 0.1 2 70 80 90",
      "D -12000 0 1 0 30 0", "D -7000 1 2 45 60 0", "D -5000 0 2 90 100 0", "J 120 0 1"};
  try {
    SolidSys mysys(spinl);
    powder zcw(powder::zcw, thd, phs);
    matrix detect = mysys.Fp();
    matrix roeq = mysys.Fx() + mysys.Fz();
    oneFID<SolidSys> myfid(mysys, npts, sw, wr, beta);
    std::vector<complex> fid = myfid.FID(zcw, roeq, detect);
    plotterFID(fid, argv[7], 1.0 / myfid.sw());
    matstream matout(std::string(argv[7]) + ".mat");  // as solid-2.0 saves its FIDs
    matout.put("vdat", fid);
    matout.put("sw1", myfid.sw());
    std::printf("%d crystallites, dim %d, sw %.6g Hz, fid[0] = %.15g %+.15gi\n", zcw.size(), mysys.HS(),
                myfid.sw(), fid[0].real(), fid[0].imag());
  } catch (const bl_error &e) {
    std::cerr << "error " << e.status << ": " << e.what() << "\n";
    return 1;
  }
  return 0;
}
