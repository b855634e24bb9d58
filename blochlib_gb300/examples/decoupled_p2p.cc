// A 13C spectrum under 1H decoupling, through the C++ host API of blochlib_gb300.hpp:
// operators from HamiltonianGen strings (as solid-2.0 reads 'ro' and 'detect'), continuous
// rf on 1H (solid-2.0's pulse term), the gamma-COMPUTE FID and the point-to-point FID
// sampled every 7/9 of a rotor period (PropReduce(9, 7) of the MMMQMAS example), both saved
// with matstream.
//
//   decoupled_p2p <npts> <wr Hz> <decoupling amp Hz> <decoupling phase deg> <zcw theta> <zcw phi> <out.mat>
#include <cstdio>
#include <cstdlib>
#include <iostream>

#include "blochlib_gb300.hpp"

using namespace blochlib_gb300;

int main(int argc, char **argv) {
  if (argc < 8) {
    std::cerr << "usage: decoupled_p2p npts wr amp phase zcw_t zcw_p out.mat\n";
    return 2;
  }
  const int npts = std::atoi(argv[1]);
  const double wr = std::atof(argv[2]), amp = std::atof(argv[3]), phase = std::atof(argv[4]);
  const int thd = std::atoi(argv[5]), phs = std::atoi(argv[6]);
  std::vector<std::string> spinl = {"numspin 3",
                                    "T 13C 0",
                                    "T 1H 1",
                                    "T 1H 2",
                                    "C 1500 6000 0.5 0 10 70 30",
                                    "D 8000 0 1 20 30 40",
                                    "D 5000 0 2 60 10 0",
                                    "D -18000 1 2 70 80 0"};
  try {
    SolidSys mysys(spinl);
    mysys.addRf("1H", amp, phase);
    HamiltonianGen gen;
    matrix roeq = gen.Hamiltonian(mysys, "Ix_0");
    matrix detect = gen.Hamiltonian(mysys, "Ip_0");
    powder zcw(powder::zcw, thd, phs);
    oneFID<SolidSys> myfid(mysys, npts, 40 * wr, wr, 54.7356);
    std::vector<complex> fid = myfid.FID(zcw, roeq, detect);
    const double sw = myfid.sw();
    std::vector<complex> p2p = myfid.p2pFID(zcw, roeq, detect, PropReduce(18, 14), 2e-6);
    matstream matout(argv[7]);
    matout.put("fid", fid);
    matout.put("sw", sw);
    matout.put("p2p", p2p);
    matout.put("sw_p2p", myfid.sw());
    matout.put("ro", roeq);
    std::printf("%d crystallites, dim %d, fid[0] = %.15g, p2p[0] = %.15g\n", zcw.size(), mysys.HS(),
                fid[0].real(), p2p[0].real());
  } catch (const bl_error &e) {
    std::cerr << "error " << e.status << ": " << e.what() << "\n";
    return 1;
  }
  return 0;
}
