// rt_pfast2d_fw.cpp -- drop-in for the forward builds of RT_PFAST2D
// (RT_PFAST2D_FW and, with -DNoShotGather, RT_PFAST2D_FW_NoS; src/RT_Compile2D.sh).
//
//   RT_PFAST2D_FW file.inp
//
// Reads the .inp and the binary model / source / receiver / reflector files as
// src/RT_PFAST2D.cpp:137-343 does, computes transmission and reflection traveltimes
// for every source on the GPU, and writes what the reference writes with one rank:
//   <p>_Tr2D.bin            [sum(srnum) x (NumofR+1)]: TT, then TTu of each reflector
//                           at the receivers (src/RT_PFAST2D.cpp:837-852, 858-868)
//   <p>_Src<id>_TTd.2d/_TTu.2d  the down-/up-going fields of each source (NumofR x NX*NY),
//                           unless built with -DNoShotGather (src/RT_PFAST2D.cpp:853-856).
#include <chrono>
#include "driver_io.h"

int main(int argc, char** argv) {
    if (argc < 2) {
        std::printf("usage: %s input_file.inp\n", argv[0]);
        return 1;
    }
    const auto t0 = std::chrono::steady_clock::now();
    const auto L = drv::param_lines(argv[1]);
    const std::string vp0 = drv::tokens(L, 0)[0], srcfile = drv::tokens(L, 1)[0], recfile = drv::tokens(L, 3)[0],
                      refgeom = drv::tokens(L, 5)[0];
    const int sNX = std::atoi(drv::tokens(L, 2)[0].c_str()), sNY = std::atoi(drv::tokens(L, 2)[1].c_str());
    const int rNX = std::atoi(drv::tokens(L, 4)[0].c_str()), rNY = std::atoi(drv::tokens(L, 4)[1].c_str());
    const int gmNX = std::atoi(drv::tokens(L, 6)[0].c_str()), gmNY = std::atoi(drv::tokens(L, 6)[1].c_str());
    const auto g = drv::tokens(L, 7);
    const int NX = std::atoi(g[0].c_str()), NY = std::atoi(g[1].c_str());
    const double dx = std::atof(g[2].c_str()), dz = std::atof(g[3].c_str());
    const int NumofR = (int)std::ceil((double)gmNX / NY);   // src/RT_PFAST2D.cpp:230
    const int MAXSwp = 500;                                  // src/RT_PFAST2D.cpp:75
    const std::string p = drv::prefix_of(vp0);

    const auto vp = drv::readmod(vp0, (size_t)NX * NY);
    const auto srcA = drv::readmod(srcfile, (size_t)sNX * sNY);
    const auto recA = drv::readmod(recfile, (size_t)rNX * rNY);
    std::vector<double> Z;
    if (gmNX > 0) Z = drv::readmod(refgeom, (size_t)gmNX * gmNY);
    const int nsrc = sNX;
    std::vector<int> src(2 * nsrc), srnum(nsrc), rec(2 * (size_t)rNX);
    long long ch1 = 0;
    for (int s = 0; s < nsrc; ++s) {
        src[2 * s] = drv::to_index(srcA[(size_t)s * sNY + 0], dz);
        src[2 * s + 1] = drv::to_index(srcA[(size_t)s * sNY + 1], dx);
        srnum[s] = (int)srcA[(size_t)s * sNY + 2];
        ch1 += srnum[s];
    }
    for (int r = 0; r < rNX; ++r) {
        rec[2 * r] = drv::to_index(recA[(size_t)r * rNY + 0], dz);
        rec[2 * r + 1] = drv::to_index(recA[(size_t)r * rNY + 1], dx);
    }
    if (ch1 > rNX) {
        std::printf("the sources list %lld receiver rows, the receiver file holds %d\n", ch1, rNX);
        return 1;
    }
    std::printf("RT_PFAST2D forward: %d x %d grid, %d sources, %lld traces, %d reflector(s)\n", NX, NY, nsrc, ch1,
                NumofR);
    pfast_ctx* ctx = nullptr;
    drv::check(pfast_ctx_create(0, &ctx), "context");
    pfast_options opt;
    pfast_default_options(&opt);
    opt.precision = drv::precision_from_env();
    opt.maxswp = MAXSwp;
    std::vector<double> Tr((size_t)std::max<long long>(ch1, 1) * (NumofR + 1));
#ifdef NoShotGather
    drv::check(pfast_forward2d(ctx, vp.data(), NX, NY, dx, dz, nsrc, src.data(), srnum.data(), (int)ch1, rec.data(),
                               NumofR, NumofR ? Z.data() : nullptr, &opt, Tr.data(), nullptr),
               "forward2d");
#else
    {
        const size_t N = (size_t)NX * NY;
        std::vector<double> U(N), TTd(N * std::max(NumofR, 1)), TTu(N * std::max(NumofR, 1));
        std::vector<double> vpc(vp);
        long long chr = 0;
        for (int s = 0; s < nsrc; ++s) {
            drv::check(pfast_RT_fsm2d(vpc.data(), U.data(), TTd.data(), TTu.data(), NumofR ? Z.data() : nullptr,
                                      src.data(), rec.data(), srnum.data(), s, NumofR, MAXSwp, dx, dz, NX, NY, 0),
                       "RT_fsm2d");
            for (int idx = 0; idx < srnum[s]; ++idx) {
                const long long row = chr + idx;
                const size_t o = (size_t)rec[2 * row] * NY + rec[2 * row + 1];
                Tr[row * (NumofR + 1)] = U[o];
                for (int ir = 0; ir < NumofR; ++ir) Tr[row * (NumofR + 1) + ir + 1] = TTu[ir * N + o];
            }
            char name[64];
            std::snprintf(name, sizeof name, "_Src%d_TTd.2d", s);
            drv::writemod(p + name, TTd.data(), N * NumofR);
            std::snprintf(name, sizeof name, "_Src%d_TTu.2d", s);
            drv::writemod(p + name, TTu.data(), N * NumofR);
            chr += srnum[s];
        }
    }
#endif
    drv::writemod(p + "_Tr2D.bin", Tr.data(), (size_t)ch1 * (NumofR + 1));
    pfast_ctx_destroy(ctx);
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("wrote %s_Tr2D.bin\nTotal Elapse Time: %10.4f seconds (%8.4f hours) \n", p.c_str(), sec, sec / 3600.0);
    return 0;
}
