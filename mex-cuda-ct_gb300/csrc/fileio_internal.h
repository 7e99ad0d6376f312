// fileio_internal.h -- shared pieces of the MAT-file readers (fileio.cpp,
// mat73.cpp); host code only.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/mexct.h"

namespace mexct {

// zlib stream (RFC 1950) -> bytes, with the DEFLATE decoder of fileio.cpp;
// false on malformed or truncated input or a wrong Adler-32.
bool zlib_inflate_bytes(const uint8_t* p, size_t n, std::vector<uint8_t>& out);

// One variable of a -v7.3 MAT-file (an object in the HDF5 root group).
struct Mat73Var {
  std::string name;
  std::string mclass;           // the MATLAB_class attribute ("double", "single", ...)
  bool numeric = false;         // a numeric or logical array this reader converts
  std::vector<long long> dims;  // MATLAB order (the HDF5 dimensions reversed)
  uint64_t header = 0;          // file offset of the dataset's object header
  const char* unsupported = nullptr;  // an HDF5 feature of it that is not read, if any
};

// True when the file holds an HDF5 superblock where MATLAB puts it (after a
// 512-byte user block) or at the start.
bool mat73_is_hdf5(const std::vector<uint8_t>& f);

// The root group's variables, in name order (MATLAB's own #refs# and
// #subsystem# groups left out).
mexct_status mat73_list(const std::vector<uint8_t>& f, const char* path,
                        std::vector<Mat73Var>& vars);

// The real part of a numeric variable as float32, column-major; count must be
// the product of its dimensions.
mexct_status mat73_read(const std::vector<uint8_t>& f, const char* path, const Mat73Var& v,
                        float* out, long long count);

// Writes one single-precision variable (dims in MATLAB order) as a -v7.3
// MAT-file: a new file, or (append) one more variable of an existing one with
// a version 0/1 superblock, its root group relinked at the end of the file.
mexct_status mat73_write(const char* path, const char* name, const float* data, int ndims,
                         const long long* dims, bool append);

}  // namespace mexct
