// t_pfast3d.cpp -- drop-in for the inverse build of T_PFAST3D (src/T_Compile3D.sh):
// 3D first-arrival traveltime inversion.
//
//   T_PFAST3D file.inp [LM]      LM: L-BFGS memory (5)
//
// Reads the .inp and the binary files as src/T_PFAST3D.cpp:86-319 does (sources and
// receivers must lie where vp >= 400) and runs the outer loop of
// src/T_PFAST3D.cpp:346-656 on the GPU (pfast_inversion3d_*).  Writes, under the prefix
// <p> (the initial model's path minus ".vp"):
//   <p>_bf_regu_<k>.vp, <p>_af_regu_<k>.vp   gradient of iteration k before / after regu3d
//   <p>_GlobalErr.txt                        misfit per iteration
//   alpha1.tmp                               last step length (secant line search)
//   <p>.vp<k>                                model after iteration k
//   the .inp's output model and <p>_AveRes_T.txt (residuals in ms) at the end.
// Resume: an initial model named <p>.vp<k> (last character a digit) restarts iteration
// k+1 from <p>_bf_regu_<k>.vp, <p>_bf_regu_<k+1>.vp, global_E.tmp and alpha1.tmp, as
// the reference does (src/T_PFAST3D.cpp:140-147, 346-385).
// PFAST_PRECISION=mixed evaluates gradients with the FP32-bulk sweeps; PFAST_MAXITER caps
// the iteration count (the reference's MAXIter is 100).
#include <chrono>
#include "driver_io.h"

namespace {

double wall_s(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// first number of every line of a text file (global_E.tmp, alpha1.tmp)
std::vector<double> read_column(const char* path) {
    std::vector<double> v;
    FILE* f = std::fopen(path, "r");
    if (!f) {
        std::printf(" The file %s cannot be opened\n", path);
        std::exit(1);
    }
    char line[128];
    while (std::fgets(line, sizeof line, f)) {
        char tok[128];
        if (std::sscanf(line, "%127s", tok) == 1) v.push_back(std::atof(tok));
    }
    std::fclose(f);
    return v;
}

}  // namespace

int main(int argc, char** argv) {
    const auto t0 = std::chrono::steady_clock::now();
    if (argc < 2 || argc > 3) {
        std::printf("usage: %s input_file.inp [LM]\n", argv[0]);
        return 1;
    }
    const int LM = argc == 3 ? std::atoi(argv[2]) : 5;
    std::printf("Only Applicable to Optimization Method: L-BFGS\n\t...%s Memory Number m=%d\n",
                argc == 2 ? "Default" : "Specified", LM);
    const auto L = drv::param_lines(argv[1]);
    std::printf("Read input parameters from file %s\nUser Parameters are as follows:\n", argv[1]);
    const std::string vp0 = drv::tokens(L, 0)[0], srcfile = drv::tokens(L, 1)[0], recfile = drv::tokens(L, 3)[0],
                      vpfile = drv::tokens(L, 6)[0];
    const int sNX = std::atoi(drv::tokens(L, 2)[0].c_str()), sNY = std::atoi(drv::tokens(L, 2)[1].c_str());
    const int rNX = std::atoi(drv::tokens(L, 4)[0].c_str()), rNY = std::atoi(drv::tokens(L, 4)[1].c_str());
    const auto g = drv::tokens(L, 5);
    const int NX = std::atoi(g[0].c_str()), NY = std::atoi(g[1].c_str()), NZ = std::atoi(g[2].c_str());
    const double dx = std::atof(g[3].c_str()), dy = std::atof(g[4].c_str()), dz = std::atof(g[5].c_str());
    const auto nu = drv::tokens(L, 7);
    const double nux = std::atof(nu[0].c_str()), nuy = std::atof(nu[1].c_str()), nuz = std::atof(nu[2].c_str());
    const auto sl = drv::tokens(L, 8);
    const int lsrc = std::atoi(sl[1].c_str());
    const char last = vp0.empty() ? 'p' : vp0.back();
    const int resume = (last == 'p') ? 0 : last - '0';
    std::printf("\nThe initial velocity file... %s\n", vp0.c_str());
    std::printf(resume ? "|==========This is a RESUME run===========|\n" : "|==========This is a NEW run===========|\n");
    std::printf("The source location file... %s\n", srcfile.c_str());
    std::printf("The source binary file dimension... %d x %d\n", sNX, sNY);
    std::printf("The receiver location file... %s\n", recfile.c_str());
    std::printf("The receiver binary file dimension... %d x %d\n", rNX, rNY);
    std::printf("The size of the model... %d X %d X %d\nSample Interval... %.2lfm x %.2lfm x %.2lfm\n", NX, NY, NZ, dx,
                dy, dz);
    std::printf("Final Velocity Model Output to %s\n", vpfile.c_str());
    std::printf("Regularization Parameters, (nux, nuy, nuz)=(%f, %f, %f)\n", nux, nuy, nuz);
    std::printf("L-BFGS quasi-newton method IN USE\n");   // the loop runs L-BFGS (src/T_PFAST3D.cpp:428)
    static const char* kLs[] = {"No Line Search, i.e. Steepest Decent", "Secant method with exact Conditions",
                                "Secant method with Strong Wolfe Conditions",
                                "Cubic Interpolation method with Strong Wolfe Conditions"};
    if (lsrc >= 0 && lsrc <= 3) std::printf("Line Search Method: %s\n", kLs[lsrc]);
    if (rNY < 7) {
        std::printf("the receiver file has %d columns; 7 are needed (position, normal, first arrival)\n", rNY);
        return 1;
    }
    const std::string p = drv::prefix_of(vp0, resume == 0 ? 3 : (resume <= 9 ? 4 : 5));
    const size_t N = (size_t)NX * NY * NZ;
    const auto vp = drv::readmod_logged(vp0, N);
    const auto srcA = drv::readmod_logged(srcfile, (size_t)sNX * sNY);
    const auto recA = drv::readmod_logged(recfile, (size_t)rNX * rNY);
    const int nsrc = sNX;
    std::vector<int> src(3 * nsrc), srnum(nsrc), rec(3 * (size_t)rNX);
    std::vector<double> nxyz(3 * (size_t)rNX), Tobs(rNX);
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
        const double* row = &recA[(size_t)r * rNY];
        rec[3 * r] = drv::to_index(row[0], dy);
        rec[3 * r + 1] = drv::to_index(row[1], dx);
        rec[3 * r + 2] = drv::to_index(row[2], dz);
        if (!inside(rec[3 * r], rec[3 * r + 1], rec[3 * r + 2]) || at(rec[3 * r], rec[3 * r + 1], rec[3 * r + 2]) < 400) {
            std::printf("Receiver %d:\t%d\t%d\t%d is not in the model volume, please check...\n", r, rec[3 * r] + 1,
                        rec[3 * r + 1] + 1, rec[3 * r + 2] + 1);
            return 1;
        }
        nxyz[3 * r] = row[3];
        nxyz[3 * r + 1] = row[4];
        nxyz[3 * r + 2] = row[5];
        Tobs[r] = row[6];
    }
    if (ch1 > rNX) {
        std::printf("the sources list %lld receiver rows, the receiver file holds %d\n", ch1, rNX);
        return 1;
    }

    pfast_ctx* ctx = nullptr;
    drv::check(pfast_ctx_create(0, &ctx), "context");
    pfast_survey3d* sv = nullptr;
    drv::check(pfast_survey3d_create(ctx, NX, NY, NZ, dx, dy, dz, nsrc, src.data(), srnum.data(), rec.data(),
                                     nxyz.data(), Tobs.data(), &sv),
               "survey3d_create");
    pfast_invert_options o;
    pfast_invert_default_options(3, &o);
    o.eval.precision = drv::precision_from_env();
    o.lsrc = lsrc;
    o.LM = LM;
    o.nux = nux;
    o.nuy = nuy;
    o.nuz = nuz;
    pfast_inversion* inv = nullptr;
    drv::check(pfast_inversion3d_create(ctx, sv, vp.data(), &o, &inv), "inversion3d_create");

    std::vector<double> gE, buf(N);
    int Iterk = 0;
    char name[96];
    if (resume) {
        std::snprintf(name, sizeof name, "_bf_regu_%d.vp", resume);
        const auto gprev = drv::readmod_logged(p + name, N);
        std::snprintf(name, sizeof name, "_bf_regu_%d.vp", resume + 1);
        const auto gcur = drv::readmod_logged(p + name, N);
        gE = read_column("global_E.tmp");
        const auto a1 = read_column("alpha1.tmp");
        if (a1.empty() || (int)gE.size() < resume + 1) {
            std::printf("global_E.tmp needs %d misfits and alpha1.tmp a step length to resume\n", resume + 1);
            return 1;
        }
        drv::check(pfast_inversion_resume(inv, resume, gprev.data(), gcur.data(), gE.data(), (int)gE.size(), a1.back()),
                   "inversion_resume");
        gE.resize(resume);
        Iterk = resume;
        std::printf("Iterating No. %d resumed: (nux,nuy,nuz)=(%f,%f,%f)\n", Iterk, nux, nuy, nuz);
    }
    const int MAXIter = drv::max_iter_from_env(100);   // src/T_PFAST3D.cpp:69
    bool conv = false;
    bool resumed_step = resume != 0;
    while (!conv && Iterk++ < MAXIter) {
        const auto tic = std::chrono::steady_clock::now();
        std::printf("Iterating No. %d started: (nux,nuy,nuz)=(%f,%f,%f)\n", Iterk, nux, nuy, nuz);
        pfast_invert_report r;
        const pfast_status st = pfast_inversion_step(inv, &r);
        if (st != PFAST_OK && st != PFAST_ERR_OVER_CORRECTED) drv::check(st, "inversion_step");
        gE.push_back(r.E);
        std::printf("Average Time Residual: %g ms\n", 1000 * std::sqrt(2 * r.E / rNX));
        if (!resumed_step) {
            drv::check(pfast_inversion_get(inv, PFAST_INV_GRAD_RAW, buf.data()), "inversion_get");
            std::snprintf(name, sizeof name, "_bf_regu_%d.vp", Iterk);
            drv::writemod_logged(p + name, buf.data(), N);
            drv::check(pfast_inversion_get(inv, PFAST_INV_GRAD, buf.data()), "inversion_get");
            std::snprintf(name, sizeof name, "_af_regu_%d.vp", Iterk);
            drv::writemod_logged(p + name, buf.data(), N);
            if (FILE* fe = std::fopen((p + "_GlobalErr.txt").c_str(), "w")) {
                for (double e : gE) std::fprintf(fe, "%g\n", e);
                std::fclose(fe);
            }
        }
        resumed_step = false;
        drv::print_linesearch(r, lsrc, PFAST_SCHEME_LBFGS, 3);
        if (lsrc == PFAST_LS_SECANT_WOLFE) {
            if (FILE* fa = std::fopen("alpha1.tmp", "w")) {
                std::fprintf(fa, "%g\n", r.stepsize);
                std::fclose(fa);
            }
        }
        drv::check(pfast_inversion_get(inv, PFAST_INV_VP, buf.data()), "inversion_get");
        std::snprintf(name, sizeof name, ".vp%d", Iterk);
        drv::writemod_logged(p + name, buf.data(), N);
        if (st == PFAST_ERR_OVER_CORRECTED) {
            std::printf("Over corrected..abort...\n");
            return 1;
        }
        conv = r.converged != 0;
        std::printf("--------Interating No. %d takes %10.4f seconds---------------\n\n", Iterk, wall_s(tic));
    }
    drv::check(pfast_inversion_get(inv, PFAST_INV_VP, buf.data()), "inversion_get");
    drv::writemod_logged(vpfile, buf.data(), N);
    if (FILE* fe = std::fopen((p + "_AveRes_T.txt").c_str(), "w")) {
        for (double e : gE) std::fprintf(fe, "%g\n", 1000 * std::sqrt(2 * e / rNX));
        std::fclose(fe);
    }
    pfast_inversion_destroy(inv);
    pfast_survey3d_destroy(sv);
    pfast_ctx_destroy(ctx);
    const double sec = wall_s(t0);
    std::printf("Total Elapse Time: %10.4f seconds (%8.4f hours) \n", sec, sec / 3600.0);
    return 0;
}
