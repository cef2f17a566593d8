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

// writemod with the reference's message (src/RT_pfsm2d.h:49-57)
inline void writemod_logged(const std::string& path, const double* a, size_t count) {
    std::printf(" \n...writing file:\n\t %s\n", path.c_str());
    writemod(path, a, count);
}

inline std::vector<double> readmod_logged(const std::string& path, size_t count) {
    std::printf(" \n...reading file:\n\t %s\n", path.c_str());
    return readmod(path, count);
}

inline int to_index(double metres, double h) { return (int)std::ceil(metres / h) - 1; }

// The line-search messages of one iteration, as the drivers print them
// (src/RT_PFAST2D.cpp:561-815, src/T_PFAST3D.cpp:505-645).  `secs`: the search's wall time.
inline void print_linesearch(const pfast_invert_report& r, int lsrc, int schemetag, int dim) {
    const double secs = r.ms_linesearch / 1000.0;
    auto trials = [&]() {
        for (int t = 0; t < r.ntrials; ++t)
            std::printf("(alpha0,alpha1,phi0,phi1,dphi0,dphi1)=(%g %g %g %g %g %g\n", r.trial[t][0], r.trial[t][1],
                        r.trial[t][2], r.trial[t][3], r.trial[t][4], r.trial[t][5]);
    };
    auto wolfe_end = [&]() {
        if (r.stopped)
            std::printf("Line Search Stopped, takes %g seconds, Stepsize=%f\n ...Updating velocity now...\n", secs,
                        r.stepsize);
        else
            std::printf("Wolfe condition satisfied After %d Iterations, takes %g seconds, Stepsize=%f\n...Updating "
                        "velocity now...\n", r.count, secs, r.stepsize);
    };
    switch (lsrc) {
        case PFAST_LS_SECANT_EXACT:
            std::printf("Secant Method Line Search for 'exact' condition (alpha1=%g)...\n", r.alpha_start);
            if (r.stopped)
                std::printf("Line Search Stopped, takes %g seconds, Stepsize=%f\n ...Updating velocity now...\n", secs,
                            r.stepsize);
            else
                std::printf("Line Search Completed After %d Iterations, takes %g seconds, Stepsize=%f\n...Updating "
                            "velocity now...\n", r.count, secs, r.stepsize);
            break;
        case PFAST_LS_SECANT_WOLFE:
            std::printf(dim == 2 ? "Secant Method Line Search with Strong Wolfe Condition (alpha1=%g)...\n"
                                 : "Secant Method Line Search for Strong Wolfe Condition (alpha1=%g)...\n",
                        r.alpha_start);
            trials();
            wolfe_end();
            break;
        case PFAST_LS_CUBIC:
            if (dim == 3)
                std::printf("Cubic Interpolation Line Searching (alpha1=%g)...\n", r.alpha_start);
            else if (schemetag == PFAST_SCHEME_LBFGS)
                std::printf("Cubic Interpolation Line Search with Strong Wolfe Condition (alpha1=%g)...\n", r.alpha_start);
            else
                std::printf("Cubic Interpolation Line Search (alpha1=%g)...\n", r.alpha_start);
            trials();
            if (dim == 3 || schemetag == PFAST_SCHEME_LBFGS) wolfe_end();
            break;
        default:
            std::printf("No Line Searching, Stepsize=%f\n", r.stepsize);
            break;
    }
}

// Iteration cap: the drivers' MAXIter unless PFAST_MAXITER is set (a cap for test runs).
inline int max_iter_from_env(int dflt) {
    const char* p = std::getenv("PFAST_MAXITER");
    return (p && std::atoi(p) > 0) ? std::atoi(p) : dflt;
}

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
