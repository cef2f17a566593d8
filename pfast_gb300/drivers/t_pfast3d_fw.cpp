// t_pfast3d_fw.cpp -- drop-in for the forward build of T_PFAST3D (T_PFAST3D_FW,
// src/T_Compile3D.sh).
//
//   T_PFAST3D_FW file.inp
//
// Reads the .inp and the binary files as src/T_PFAST3D.cpp:100-319 does (including
// the check that sources and receivers lie where vp >= 400, :253-256 and :294-297),
// computes first-arrival traveltimes for every source on the GPU, and writes
// <p>_Tr3D.bin: the traveltime at each receiver row, [sum(srnum) x 1]
// (src/T_PFAST3D.cpp:672-697 with one rank).
#include <chrono>
#include "driver_io.h"

int main(int argc, char** argv) {
    if (argc < 2) {
        std::printf("usage: %s input_file.inp\n", argv[0]);
        return 1;
    }
    const auto t0 = std::chrono::steady_clock::now();
    const auto L = drv::param_lines(argv[1]);
    const std::string vp0 = drv::tokens(L, 0)[0], srcfile = drv::tokens(L, 1)[0], recfile = drv::tokens(L, 3)[0];
    const int sNX = std::atoi(drv::tokens(L, 2)[0].c_str()), sNY = std::atoi(drv::tokens(L, 2)[1].c_str());
    const int rNX = std::atoi(drv::tokens(L, 4)[0].c_str()), rNY = std::atoi(drv::tokens(L, 4)[1].c_str());
    const auto g = drv::tokens(L, 5);
    const int NX = std::atoi(g[0].c_str()), NY = std::atoi(g[1].c_str()), NZ = std::atoi(g[2].c_str());
    const double dx = std::atof(g[3].c_str()), dy = std::atof(g[4].c_str()), dz = std::atof(g[5].c_str());
    const int MAXSwp = 100;   // src/T_PFAST3D.cpp:69
    // output prefix: a model name ending in a digit is a resume (src/T_PFAST3D.cpp:140-147, 322-328)
    const char last = vp0.empty() ? 'p' : vp0.back();
    const int resume = (last == 'p') ? 0 : last - '0';
    const std::string p = drv::prefix_of(vp0, resume == 0 ? 3 : (resume <= 9 ? 4 : 5));

    const auto vp = drv::readmod(vp0, (size_t)NX * NY * NZ);
    const auto srcA = drv::readmod(srcfile, (size_t)sNX * sNY);
    const auto recA = drv::readmod(recfile, (size_t)rNX * rNY);
    const int nsrc = sNX;
    std::vector<int> src(3 * nsrc), srnum(nsrc), rec(3 * (size_t)rNX);
    auto at = [&](int i, int j, int k) { return vp[(size_t)k * NX * NY + (size_t)i * NY + j]; };
    auto inside = [&](int i, int j, int k) { return i >= 0 && i < NX && j >= 0 && j < NY && k >= 0 && k < NZ; };
    long long ch1 = 0;
    for (int s = 0; s < nsrc; ++s) {
        src[3 * s] = drv::to_index(srcA[(size_t)s * sNY + 0], dy);
        src[3 * s + 1] = drv::to_index(srcA[(size_t)s * sNY + 1], dx);
        src[3 * s + 2] = drv::to_index(srcA[(size_t)s * sNY + 2], dz);
        if (!inside(src[3 * s], src[3 * s + 1], src[3 * s + 2]) || at(src[3 * s], src[3 * s + 1], src[3 * s + 2]) < 400) {
            std::printf("Source %d:\t%d\t%d\t%d is not in the model volume, please check...\n", s, src[3 * s] + 1,
                        src[3 * s + 1] + 1, src[3 * s + 2] + 1);
            return 1;
        }
        srnum[s] = (int)std::ceil(srcA[(size_t)s * sNY + 3]);
        ch1 += srnum[s];
    }
    for (int r = 0; r < rNX; ++r) {
        rec[3 * r] = drv::to_index(recA[(size_t)r * rNY + 0], dy);
        rec[3 * r + 1] = drv::to_index(recA[(size_t)r * rNY + 1], dx);
        rec[3 * r + 2] = drv::to_index(recA[(size_t)r * rNY + 2], dz);
        if (!inside(rec[3 * r], rec[3 * r + 1], rec[3 * r + 2]) || at(rec[3 * r], rec[3 * r + 1], rec[3 * r + 2]) < 400) {
            std::printf("Receiver %d:\t%d\t%d\t%d is not in the model volume, please check...\n", r, rec[3 * r] + 1,
                        rec[3 * r + 1] + 1, rec[3 * r + 2] + 1);
            return 1;
        }
    }
    if (ch1 > rNX) {
        std::printf("the sources list %lld receiver rows, the receiver file holds %d\n", ch1, rNX);
        return 1;
    }
    std::printf("T_PFAST3D forward: %d x %d x %d grid, %d sources, %lld traces\n", NX, NY, NZ, nsrc, ch1);
    pfast_ctx* ctx = nullptr;
    drv::check(pfast_ctx_create(0, &ctx), "context");
    pfast_options opt;
    pfast_default_options(&opt);
    opt.precision = drv::precision_from_env();
    opt.maxswp = MAXSwp;
    std::vector<double> picks((size_t)std::max<long long>(ch1, 1));
    drv::check(pfast_forward3d(ctx, vp.data(), NX, NY, NZ, dx, dy, dz, nsrc, src.data(), srnum.data(), rec.data(),
                               &opt, picks.data(), nullptr),
               "forward3d");
    drv::writemod(p + "_Tr3D.bin", picks.data(), (size_t)ch1);
    pfast_ctx_destroy(ctx);
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("wrote %s_Tr3D.bin\nTotal Elapse Time: %10.4f seconds (%8.4f hours) \n", p.c_str(), sec, sec / 3600.0);
    return 0;
}
