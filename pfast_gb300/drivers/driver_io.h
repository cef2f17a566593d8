// driver_io.h -- the reference drivers' input/output conventions, for the drop-in
// executables built on the pfast_gb300 C ABI.
//   * .inp: every line not starting with '#' is a parameter line, read by position
//     (src/RT_PFAST2D.cpp:137-172, src/T_PFAST3D.cpp:105-134).
//   * binary files: raw native-endian doubles, row-major (readmod / writemod,
//     src/T_pfsm3d.h:39-57).
//   * coordinates in metres become node indices with (int)ceil(x/h)-1
//     (src/T_PFAST3D.cpp:250-252, src/RT_PFAST2D.cpp:300-301).
//   * output prefix <p> = the initial-model path minus its last 3 characters
//     (src/RT_PFAST2D.cpp:242-243, src/T_PFAST3D.cpp:322-328).
#pragma once

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "pfast_gb300.h"

namespace drv {

inline std::vector<std::string> param_lines(const char* path) {
    std::vector<std::string> out;
    FILE* f = std::fopen(path, "r");
    if (!f) {
        std::printf("The file %s was not opened\n", path);
        std::exit(1);
    }
    char line[1024];
    while (std::fgets(line, sizeof line, f))
        if (line[0] != '#') out.emplace_back(line);
    std::fclose(f);
    return out;
}

// whitespace-separated tokens of parameter line `k`
inline std::vector<std::string> tokens(const std::vector<std::string>& L, size_t k) {
    std::vector<std::string> t;
    if (k >= L.size()) {
        std::printf("The input file has too few parameter lines (need line %zu)\n", k + 1);
        std::exit(1);
    }
    char buf[1024];
    std::strncpy(buf, L[k].c_str(), sizeof buf - 1);
    buf[sizeof buf - 1] = 0;
    for (char* p = std::strtok(buf, " \t\r\n"); p; p = std::strtok(nullptr, " \t\r\n")) t.emplace_back(p);
    if (t.empty()) {
        std::printf("Parameter line %zu is empty\n", k + 1);
        std::exit(1);
    }
    return t;
}

inline std::vector<double> readmod(const std::string& path, size_t count) {
    std::vector<double> v(count);
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        std::printf(" The file %s cannot be opened\n", path.c_str());
        std::exit(1);
    }
    const size_t got = std::fread(v.data(), sizeof(double), count, f);
    std::fclose(f);
    if (got != count) {
        std::printf(" The file %s holds %zu doubles, %zu expected\n", path.c_str(), got, count);
        std::exit(1);
    }
    return v;
}

inline void writemod(const std::string& path, const double* a, size_t count) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) {
        std::printf(" The file %s cannot be opened\n", path.c_str());
        std::exit(1);
    }
    std::fwrite(a, sizeof(double), count, f);
    std::fclose(f);
}

inline int to_index(double metres, double h) { return (int)std::ceil(metres / h) - 1; }

inline std::string prefix_of(const std::string& vp0, int drop = 3) {
    return vp0.size() > (size_t)drop ? vp0.substr(0, vp0.size() - drop) : std::string();
}

inline void check(pfast_status s, const char* where) {
    if (s != PFAST_OK) {
        std::printf("%s: %s (%s)\n", where, pfast_status_string(s), pfast_last_error());
        std::exit(1);
    }
}

// PFAST_PRECISION=mixed selects the FP32-bulk + FP64-polish sweeps; the default is the
// plain FP64 arithmetic of the reference.
inline int precision_from_env() {
    const char* p = std::getenv("PFAST_PRECISION");
    return (p && std::strcmp(p, "mixed") == 0) ? PFAST_MIXED : PFAST_PLAIN_FP64;
}

}  // namespace drv
