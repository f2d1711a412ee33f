// dumpconfig -- GB300 drop-in for the reference's `DumpConfig` driver
// (DumpConfig/main.cpp:30-143): plants equilibrium configurations from the
// leading eigenvector(s) a tmat run saved.
//
//   dumpconfig [input.dat] [ndump] [length] [--seed S]
//
// Arguments as the reference's (defaults input.dat, 1, 100).  Reads the same
// input file as tmat, loads <out>_vec.dat (and <out>_vecl.dat for the
// two-layer parallel TMs, model A axialdir 2 and 6, model B axialdir 6),
// plants on the GPU through tm_dump_configs / tm_dump_configs_lr and writes
// <out>_config_<k>.dat, one layer per line, L digits, site 0 first.
// The reference seeds its mt19937 from time(NULL) (MyUtility::setseed,
// DumpConfig/utilityb.cpp:19-22); so does this driver unless --seed is given,
// and a given seed plants the configurations the reference's generator would
// with that seed.
#include <sys/stat.h>

#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "latttmat.h"
#include "read_input.hpp"

using latttmat::ReadInput;

// The reference's vector reader (DumpConfig/dumpconfig.hpp:55-76): the first
// n coefficients' absolute values; for a two-layer (complex-scalar) dumper a
// file of at least 16 n bytes is read as interleaved (re, im) and the real
// parts kept.
static std::vector<double> read_vector(const std::string& fname, int64_t n, bool complex_scalar) {
  struct stat sb;
  if (stat(fname.c_str(), &sb)) throw std::runtime_error("Open \"" + fname + "\" failed");
  if ((uint64_t)sb.st_size < sizeof(double) * (uint64_t)n)
    throw std::runtime_error("File \"" + fname + "\" size incorrect");
  const bool interleaved = complex_scalar && (uint64_t)sb.st_size >= 2 * sizeof(double) * (uint64_t)n;
  std::ifstream f(fname, std::ios::binary);
  std::vector<double> v((size_t)n);
  double t;
  for (int64_t i = 0; i < n; ++i) {
    f.read(reinterpret_cast<char*>(&t), sizeof(double));
    v[(size_t)i] = std::fabs(t);
    if (interleaved) f.read(reinterpret_cast<char*>(&t), sizeof(double));
  }
  if (!f) throw std::runtime_error("Read from \"" + fname + "\" failed");
  return v;
}

// One line per layer, site 0 first (DumpConfig_Base::output,
// DumpConfig/dumpconfig.hpp:31-39).
static void write_config(const std::string& path, const uint64_t* states, int nlayer, int L) {
  std::ofstream f(path);
  std::string line((size_t)L + 1, '\n');
  for (int s = 0; s < nlayer; ++s) {
    uint64_t st = states[s];
    for (int i = 0; i < L; ++i, st >>= 1) line[(size_t)i] = (st & 1) ? '1' : '0';
    f << line;
  }
}

// The dispatch of DumpConfig/main.cpp:57-131.  Returns 0 with the
// reference's message for a combination it has no dumper for.
static int dump(const ReadInput& in, int ndump, int length, uint32_t seed) {
  const int multieigs = in.neigs > 1 ? 2 : 0;
  bool two_layer = false, reduced_sym = false, known = false;
  if (in.dim != 2) {
    std::cerr << "Error: dimension not supported yet" << std::endl;
    return 0;
  }
  if (in.model == 'A') {
    known = in.axialdir == 1 || in.axialdir == 2 || in.axialdir == 5 || in.axialdir == 6;
    two_layer = in.axialdir == 2 || in.axialdir == 6;
    reduced_sym = in.axialdir == 5;
  } else if (in.model == 'B') {
    if (in.axialdir == 7) {
      // the reference's ZBM2DDumpConfig::dump is an unfinished stub
      // (DumpConfig/dumpreduce.cpp:409, marked TODO); nothing is planted
      std::cerr << "Error: planting for the reduced z-BNNNI TM is not implemented" << std::endl;
      return 1;
    }
    known = two_layer = in.axialdir == 6;
  } else if (in.model == 'D') {
    known = reduced_sym = in.axialdir == 5;
  } else {
    std::cerr << "Error: model not supported yet" << std::endl;
    return 0;
  }
  if (!known) {
    std::cerr << "Error: axial direction not supported yet" << std::endl;
    return 0;
  }
  // the dumpers build their operators with extend_cond = multieigs for the
  // reduced symmetric ones and the default 0 otherwise
  tm_params p{in.betaJ, in.kappa, in.kappa2, in.h, in.size};
  tm_op* op = nullptr;
  if (tm_create(&p, in.model, in.dim, in.axialdir, reduced_sym ? multieigs : 0, &op) != TM_OK) {
    std::cerr << tm_last_error() << std::endl;
    return 1;
  }
  const int64_t n = tm_rows(op);
  const int nlayer = (in.model == 'A' && in.axialdir == 2) ? length + 1 : length;
  std::vector<uint64_t> states((size_t)ndump * (size_t)nlayer);
  tm_status st;
  try {
    std::vector<double> vr = read_vector(in.outprefix + "_vec.dat", n, two_layer);
    std::vector<double> vl;
    if (two_layer) vl = read_vector(in.outprefix + "_vecl.dat", n, true);
    if (ndump < 1) {  // the reference reads its vectors, then plants nothing
      tm_destroy(op);
      return 0;
    }
    if (two_layer) {
      st = tm_dump_configs_lr(op, vr.data(), vl.data(), ndump, length, seed, states.data());
    } else {
      st = tm_dump_configs(op, vr.data(), ndump, length, seed, states.data());
    }
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    tm_destroy(op);
    return 1;
  }
  tm_destroy(op);
  if (st != TM_OK) {
    std::cerr << tm_last_error() << std::endl;
    return 1;
  }
  for (int k = 0; k < ndump; ++k)
    write_config(in.outprefix + "_config_" + std::to_string(k) + ".dat", states.data() + (size_t)k * nlayer, nlayer,
                 in.size);
  return 0;
}

int main(int argc, char** argv) {
  std::vector<const char*> pos;
  bool seeded = false;
  uint32_t seed = 0;
  for (int i = 1; i < argc; ++i) {
    if (!std::strcmp(argv[i], "--seed") && i + 1 < argc) {
      seed = (uint32_t)std::strtoul(argv[++i], nullptr, 10);
      seeded = true;
    } else {
      pos.push_back(argv[i]);
    }
  }
  const char* infile = pos.size() > 0 ? pos[0] : "input.dat";
  const int ndump = pos.size() > 1 ? std::atoi(pos[1]) : 1;
  const int length = pos.size() > 2 ? std::atoi(pos[2]) : 100;
  if (!seeded) seed = (uint32_t)std::time(nullptr);
  ReadInput input;
  int err = input.read(infile);
  if (err) return err;
  auto t1 = std::chrono::steady_clock::now();
  int rc = dump(input, ndump, length, seed);
  auto t2 = std::chrono::steady_clock::now();
  double tc = std::chrono::duration<double>(t2 - t1).count();
  if (tc >= 1.0) std::cout << "Time consumed: " << tc << " s" << std::endl;
  return rc;
}
