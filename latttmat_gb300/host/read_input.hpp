// Positional input-file reader, restating Read_Input::read
// (TMat/read_input.hpp:15-28, TMat/read_input.cpp:14-92): values are taken
// after successive '=' signs in fixed order (model, dim, axialdir, neigs,
// savevec[2], outfile, size (two ints when dim=3), J, kappa [kappa2], h);
// keys and comments are ignored.  Return codes 2 (cannot open), 3 (read
// failure), 4 (invalid dim / model / size), as the reference.
#pragma once
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>

namespace latttmat {

struct ReadInput {
  char model = 'A';
  int dim = 2, axialdir = 1, neigs = 1;
  int savevec[2] = {0, 0};
  std::string outprefix;
  int size = 0;
  double betaJ = 0, kappa = 0, kappa2 = 0, h = 0;

  int read(const char* inputf, std::ostream& log = std::cout) {
    int size1 = 0, size2 = 0;
    std::ifstream in(inputf);
    if (!in) {
      log << "Can't open " << inputf << " for input." << std::endl;
      return 2;
    }
    log << "Reading input from file " << inputf << std::endl;
    char buf[300], c;
    auto next = [&]() {
      in.get(buf, 300, '=');
      in.get(c);
    };
    next();
    in >> model;
    next();
    in >> dim;
    next();
    in >> axialdir;
    next();
    in >> neigs;
    next();
    in >> savevec[0] >> savevec[1];
    next();
    in >> outprefix;
    next();
    if (dim == 2) {
      in >> size;
    } else if (dim == 3) {
      in >> size1 >> size2;
      size = size1 << 16 | size2;
    } else {
      log << "Invalid dim " << dim << std::endl;
      return 4;
    }
    next();
    in >> betaJ;
    in.get(buf, 300, '=');
    std::string kline;
    std::getline(in, kline);
    std::istringstream ks(kline);
    ks.get(c);
    ks >> kappa;
    ks >> kappa2;
    if (!ks) kappa2 = 0.;
    next();
    in >> h;
    int error = 0;
    if (in.fail()) {
      log << "Error reading input file " << inputf << std::endl;
      error = 3;
    }
    log << "     MODEL : " << dim << "D_" << model << axialdir << "\n";
    log << "Save & flg : " << outprefix << " " << savevec[0] << " " << savevec[1] << "\n";
    if (dim == 2)
      log << "      size : " << size << "\n";
    else
      log << "      size : " << size1 << " " << size2 << "\n";
    log << "     betaJ : " << betaJ << "\n";
    log << "     kappa : " << kappa << std::endl;
    if ('B' == model) log << "    kappa2 : " << kappa2 << std::endl;
    log << "         h : " << h << std::endl;
    if (model != 'A' && model != 'B' && model != 'D') {
      log << "Invalid model " << model << std::endl;
      error = 4;
    } else if (size < 4) {
      log << "Invalid size (<4) " << size << std::endl;
      error = 4;
    }
    return error;
  }
};

}  // namespace latttmat
