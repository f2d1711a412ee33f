// extern "C" shim over the reference's configuration planting (DumpConfig),
// compiled from the reference sources where they lie (oracle/build_ref.sh).
// Test infrastructure only: it runs the unmodified dump() of the reference's
// DumpConfig classes with a fixed seed of the reference's random generator
// (MyUtility::setseed, DumpConfig/utilityb.cpp), so the golden-fixture script
// can record the configurations the reference plants.
//
// Dispatch mirrors DumpConfig/main.cpp:57-120 (model, axialdir -> class, with
// multieigs passed as extend_cond).
#include <cstdint>
#include <memory>
#include <string>

#include "../TMat/commondef.hpp"
#include "dumpconfig.hpp"
#include "dumpreduce.hpp"
#include "utilityb.hpp"

extern "C" int ref_dump(char model, int axialdir, int extend_cond, double betaJ, double kappa, double kappa2,
                        double h, int size, const char* vecfile, const char* veclfile, int nconfig, int length,
                        unsigned seed, const char* prefix) {
  const MParameter mpara{betaJ, kappa, kappa2, h, size};
  std::unique_ptr<DumpMat::DumpConfig_Base> bs;
  try {
    if (model == 'A' && axialdir == 1)
      bs.reset(new DumpMat::XAT2DDumpConfig(mpara, vecfile));
    else if (model == 'A' && axialdir == 2)
      bs.reset(new DumpMat::YAT2DDumpConfig(mpara, vecfile, veclfile ? veclfile : ""));
    else if (model == 'A' && axialdir == 5)
      bs.reset(new DumpMat::XAM2DDumpConfig(mpara, vecfile, extend_cond));
    else if (model == 'A' && axialdir == 6)
      bs.reset(new DumpMat::YAM2DDumpConfig(mpara, vecfile, veclfile ? veclfile : "", extend_cond));
    else if (model == 'B' && axialdir == 6)
      bs.reset(new DumpMat::YBM2DDumpConfig(mpara, vecfile, veclfile ? veclfile : "", extend_cond));
    else if (model == 'D' && axialdir == 5)
      bs.reset(new DumpMat::XDM2DDumpConfig(mpara, vecfile, extend_cond));
    else
      return 2;
    MyUtility::setseed(seed);
    bs->dump(nconfig, length, prefix);
  } catch (...) {
    return 1;
  }
  return 0;
}
