// gb300_ntt_io.hpp -- the reference harness's quarter-file format in C++
// (header-only, standard library only).
//
// The reference streams every polynomial through four PLIOs, one quarter of
// the coefficients each (src/project.cpp:111-132, src/kernels/io_kernels.cc):
// <folder>/input_data_q{0..3}.txt are four independent streams of integers,
// one 128-bit PLIO word per line (8 int16 or 4 int32 values); polynomial i is
// coefficients [i n/4, (i+1) n/4) of q0, q1, q2, q3 in that order.  Results go
// to output_data_q{0..3}.txt the same way.  Lines starting with 'T' (the
// cycle-accurate simulator's timestamps) are skipped when reading.
#pragma once

#include <cstdint>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace gb300ntt {

inline std::vector<long long> read_quarter_stream(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::vector<long long> v;
    std::string line;
    while (std::getline(f, line)) {
        size_t i = line.find_first_not_of(" \t\r");
        if (i == std::string::npos || line[i] == 'T') continue;
        std::istringstream s(line);
        long long x;
        while (s >> x) v.push_back(x);
    }
    return v;
}

// `count` polynomials of n coefficients (n a multiple of 4), back to back.
// Values are stored like the PLIO lanes (two's-complement wrap to T).
template <typename T>
std::vector<T> read_quarters(const std::string& folder, unsigned n, size_t count,
                             const std::string& prefix = "input_data") {
    if (n % 4) throw std::invalid_argument("n must be a multiple of 4");
    const size_t qn = n / 4;
    std::vector<T> out((size_t)n * count);
    for (int k = 0; k < 4; ++k) {
        const std::vector<long long> s = read_quarter_stream(folder + "/" + prefix + "_q" + std::to_string(k) + ".txt");
        if (s.size() < qn * count) throw std::runtime_error("quarter file too short for the requested polynomials");
        for (size_t p = 0; p < count; ++p)
            for (size_t j = 0; j < qn; ++j)
                out[p * n + k * qn + j] = (T)(uint64_t)s[p * qn + j];
    }
    return out;
}

// Writes `count` polynomials as four quarter files, 16 bytes of values per line.
template <typename T>
void write_quarters(const std::string& folder, const T* polys, unsigned n, size_t count,
                    const std::string& prefix = "output_data") {
    if (n % 4) throw std::invalid_argument("n must be a multiple of 4");
    const size_t qn = n / 4, per_line = 16 / sizeof(T);
    for (int k = 0; k < 4; ++k) {
        std::ofstream f(folder + "/" + prefix + "_q" + std::to_string(k) + ".txt");
        if (!f) throw std::runtime_error("cannot write to " + folder);
        size_t col = 0;
        for (size_t p = 0; p < count; ++p)
            for (size_t j = 0; j < qn; ++j) {
                f << (long long)polys[p * n + k * qn + j];
                f << (++col % per_line == 0 ? '\n' : ' ');
            }
        if (col % per_line) f << '\n';
    }
}

}  // namespace gb300ntt
