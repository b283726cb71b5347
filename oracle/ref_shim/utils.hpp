/*
 * Stand-in for the reference's src/olivier/utils.hpp, used only to compile
 * the reference's kNN.cpp, sampler.cpp, glPack.cpp, glVQ.cpp, geneticMap.cpp
 * and hmmLike.cpp in place (oracle/Makefile -> oracle/_ref, and the C++
 * drop-in test).  The original pulls in Boost (program_options, iostreams,
 * uuid), which is not installed here.  Of it, those files use only the
 * standard headers below and the file classes ofile/ifile: ofile only in
 * Save() members, which nothing here calls, and ifile in GeneticMap's
 * reader, for which a plain (uncompressed) file stream stands in.  This file
 * is test infrastructure.
 */
#ifndef GLP_REF_SHIM_UTILS_HPP
#define GLP_REF_SHIM_UTILS_HPP

#include <cassert>
#include <climits>
#include <cmath>
#include <cstdint>
#include <fstream>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

struct ofile : std::ofstream {
  explicit ofile(const std::string &path) : std::ofstream(path) {}
};

struct ifile : std::ifstream {
  explicit ifile(const std::string &path) : std::ifstream(path) {}
  bool isGood() const { return good(); }
};

#endif
