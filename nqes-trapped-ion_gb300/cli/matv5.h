// MATLAB Level-5 MAT-file reading and writing for the drop-in executable.
//
// Covers what the reference exchanges through libmatio (code/rbm.cc:272-471,
// 828-889): numeric arrays, real or complex, any rank, stored column-major,
// uncompressed. Reading accepts every numeric storage type MAT v5 allows
// (files written by MATLAB store integer-valued doubles compactly) and the
// "small data element" tag form; compressed elements are reported as
// unsupported.
#pragma once
#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace nqes_cli {

struct MatArray {
    std::vector<size_t> dims;  // MATLAB dimensions (column-major storage)
    bool is_complex = false;
    bool is_double = true;     // class mxDOUBLE_CLASS (vs other numeric classes)
    std::vector<double> re, im;
    size_t numel() const {
        size_t n = 1;
        for (auto d : dims) n *= d;
        return n;
    }
};

// Reads every numeric variable of a MAT v5 file. Returns false and sets err
// on failure (missing file, not MAT v5, big-endian, compressed element).
bool mat_read(const std::string &path, std::map<std::string, MatArray> &vars, std::string &err);

// Writes the variables in order, uncompressed, as double (complex when
// is_complex). Returns false and sets err on I/O failure.
bool mat_write(const std::string &path, const std::vector<std::pair<std::string, MatArray>> &vars, std::string &err);

}  // namespace nqes_cli
