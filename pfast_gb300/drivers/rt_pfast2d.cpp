// rt_pfast2d.cpp -- drop-in for the inverse build of RT_PFAST2D (src/RT_Compile2D.sh):
// joint (or transmission-only / reflection-only) 2D traveltime inversion.
//
//   RT_PFAST2D file.inp [LM [RTtag]]      LM: L-BFGS memory (5); RTtag: 3 joint, 1 T, 2 R
//
// Reads the .inp and the binary files as src/RT_PFAST2D.cpp:92-343 does and runs the
// outer loop of src/RT_PFAST2D.cpp:412-816 on the GPU (pfast_inversion2d_*).  Writes
// what the reference writes with one rank, under the prefix <p> (the initial model's
// path minus ".vp"):
//   <p>_bf_regu_RT<k>, <p>_af_regu_RT<k>   gradient of iteration k before / after the
//   <p>_bf_regu_R<k>,  <p>_af_regu_R<k>    regularisation (joint, reflection, transmission)
//   <p>_bf_regu_T<k>,  <p>_af_regu_T<k>
//   <p>_GlobalErr_TR_T_R.txt               misfits E, Et, Er per iteration
//   <p>_<k>                                model after iteration k
//   the .inp's output model and <p>_AveRes_TR_T_R.txt (residuals in ms) at the end.
// PFAST_PRECISION=mixed evaluates gradients with the FP32-bulk sweeps; PFAST_MAXITER caps
// the iteration count (the reference's MAXIter is 500).
#include <chrono>
#include "driver_io.h"

namespace {

double wall_s(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

int main(int argc, char** argv) {
    const auto t0 = std::chrono::steady_clock::now();
    if (argc < 2 || argc > 4) {
        std::printf("usage: %s input_file.inp [LM [RTtag]]\n", argv[0]);
        return 1;
    }
    const int LM = argc >= 3 ? std::atoi(argv[2]) : 5;
    const int RTtag = argc == 4 ? std::atoi(argv[3]) : 3;
    std::printf("Optimization Method: L-BFGS\n%s Memory Number m=%d (Ignore if L-BFGS is not used)\n",
                argc == 2 ? "Default" : "Specified", LM);
    std::printf(" *****************************************************************\n");
    if (RTtag == 3) std::printf("Joint Inversion of Reflection and Transmission\n");
    else if (RTtag == 1) std::printf("Inversion of Transmission ONLY\n");
    else if (RTtag == 2) std::printf("Inversion of Reflection ONLY\n");
    std::printf(" *****************************************************************\n");
    if (RTtag < 1 || RTtag > 3) {
        std::printf("RTtag is unrecognized!...abort...\n");
        return 1;
    }

    const auto L = drv::param_lines(argv[1]);
    std::printf("Read input parameters from file %s\nUser Parameters are as follows:\n", argv[1]);
    const std::string vp0 = drv::tokens(L, 0)[0], srcfile = drv::tokens(L, 1)[0], recfile = drv::tokens(L, 3)[0],
                      refgeom = drv::tokens(L, 5)[0], vpfile = drv::tokens(L, 8)[0], twfile = drv::tokens(L, 10)[0];
    const int sNX = std::atoi(drv::tokens(L, 2)[0].c_str()), sNY = std::atoi(drv::tokens(L, 2)[1].c_str());
    const int rNX = std::atoi(drv::tokens(L, 4)[0].c_str()), rNY = std::atoi(drv::tokens(L, 4)[1].c_str());
    const int gmNX = std::atoi(drv::tokens(L, 6)[0].c_str()), gmNY = std::atoi(drv::tokens(L, 6)[1].c_str());
    const auto g = drv::tokens(L, 7);
    const int NX = std::atoi(g[0].c_str()), NY = std::atoi(g[1].c_str());
    const double dx = std::atof(g[2].c_str()), dz = std::atof(g[3].c_str());
    const auto nu = drv::tokens(L, 9);
    const double nux = std::atof(nu[0].c_str()), nuy = std::atof(nu[1].c_str());
    const auto sl = drv::tokens(L, 11);
    const int schemetag = std::atoi(sl[0].c_str()), lsrc = std::atoi(sl[1].c_str());
    std::printf("\nThe initial velocity file... %s\n", vp0.c_str());
    std::printf("The source location file... %s\n", srcfile.c_str());
    std::printf("The receiver location file... %s\n", recfile.c_str());
    std::printf("The source binary file dimension... %d x %d\n", sNX, sNY);
    std::printf("The receiver binary file dimension... %d x %d\n", rNX, rNY);
    std::printf("The reflector geometry file... %s\n", refgeom.c_str());
    std::printf("The reflector geometry binary file dimension... %d x %d\n", gmNX, gmNY);
    std::printf("The size of the model... %d X %d\nSample Interval... %.2lfm x %.2lfm\n", NX, NY, dx, dz);
    std::printf("Final Velocity Model Output to %s\n", vpfile.c_str());
    std::printf("The weighting factor matrix file... %s\n\n", twfile.c_str());
    static const char* kScheme[] = {"Steepest Decent Method In Use", "HS Nonlinear Conjugate Method In Use",
                                    "CGDESCENT Nonlinear Conjugate Method In Use", "L-BFGS quasi-newton method In Use"};
    static const char* kLs[] = {"No Line Search for steepest decent only", "Secant method with exact Conditions",
                                "Line Search with Strong Wolfe Conditions",
                                "Cubic Interpolation method with Strong Wolfe Conditions"};
    if (schemetag >= 0 && schemetag <= 3) std::printf("%s\n", kScheme[schemetag]);
    if (lsrc >= 0 && lsrc <= 3) std::printf("%s\n", kLs[lsrc]);

    const int NumofR = (int)std::ceil((double)gmNX / NY);   // src/RT_PFAST2D.cpp:230
    const size_t N = (size_t)NX * NY;
    const std::string p = drv::prefix_of(vp0);
    const auto vp = drv::readmod_logged(vp0, N);
    const auto srcA = drv::readmod_logged(srcfile, (size_t)sNX * sNY);
    const auto recA = drv::readmod_logged(recfile, (size_t)rNX * rNY);
    std::vector<double> Z;
    if (gmNX > 0) Z = drv::readmod_logged(refgeom, (size_t)gmNX * gmNY);
    if (rNY < 5 + NumofR) {
        std::printf("the receiver file has %d columns; row, column, two normal components, TT and %d reflection "
                    "times are needed\n", rNY, NumofR);
        return 1;
    }
    const int nsrc = sNX;
    std::vector<int> src(2 * nsrc), srnum(nsrc), rec(2 * (size_t)rNX);
    std::vector<double> nxy(2 * (size_t)rNX), TT(rNX), TR((size_t)rNX * std::max(NumofR, 1));
    long long ch1 = 0;
    for (int s = 0; s < nsrc; ++s) {
        src[2 * s] = drv::to_index(srcA[(size_t)s * sNY + 0], dz);
        src[2 * s + 1] = drv::to_index(srcA[(size_t)s * sNY + 1], dx);
        srnum[s] = (int)srcA[(size_t)s * sNY + 2];
        ch1 += srnum[s];
    }
    for (int r = 0; r < rNX; ++r) {
        const double* row = &recA[(size_t)r * rNY];
        rec[2 * r] = drv::to_index(row[0], dz);
        rec[2 * r + 1] = drv::to_index(row[1], dx);
        nxy[2 * r] = row[2];
        nxy[2 * r + 1] = row[3];
        TT[r] = row[4];
        for (int ir = 0; ir < NumofR; ++ir) TR[(size_t)r * NumofR + ir] = row[5 + ir];
    }
    if (ch1 > rNX) {
        std::printf("the sources list %lld receiver rows, the receiver file holds %d\n", ch1, rNX);
        return 1;
    }
    const auto WR = drv::readmod_logged(twfile, N);

    pfast_ctx* ctx = nullptr;
    drv::check(pfast_ctx_create(0, &ctx), "context");
    pfast_survey2d* sv = nullptr;
    drv::check(pfast_survey2d_create(ctx, NX, NY, dx, dz, nsrc, src.data(), srnum.data(), (int)ch1, rec.data(),
                                     nxy.data(), TT.data(), NumofR, NumofR ? TR.data() : nullptr,
                                     NumofR ? Z.data() : nullptr, &sv),
               "survey2d_create");
    pfast_invert_options o;
    pfast_invert_default_options(2, &o);
    o.eval.precision = drv::precision_from_env();
    o.schemetag = schemetag;
    o.lsrc = lsrc;
    o.LM = LM;
    o.rttag = RTtag;
    o.nux = nux;
    o.nuz = nuy;                 // the .inp's second value weights the rows (regu2d's nuz)
    o.keep_components = 1;
    pfast_inversion* inv = nullptr;
    drv::check(pfast_inversion2d_create(ctx, sv, vp.data(), WR.data(), &o, &inv), "inversion2d_create");

    const int MAXIter = drv::max_iter_from_env(500);   // src/RT_PFAST2D.cpp:75
    std::vector<double> gE, gEt, gEr, buf(N);
    int Iterk = 0;
    bool conv = false;
    char name[64];
    while (!conv && Iterk++ < MAXIter) {
        const auto tic = std::chrono::steady_clock::now();
        std::printf("Iterating No. %d: (nux,nuy)=(%f,%f)\n", Iterk, nux, nuy);
        pfast_invert_report r;
        const pfast_status st = pfast_inversion_step(inv, &r);
        if (st != PFAST_OK && st != PFAST_ERR_OVER_CORRECTED) drv::check(st, "inversion_step");
        gE.push_back(r.E);
        gEt.push_back(r.Et);
        gEr.push_back(r.Er);
        std::printf("Average Time Residual (TR): %g ms\t", 1000 * std::sqrt(2 * r.E / rNX));
        std::printf("(T): %g ms\t", 1000 * std::sqrt(2 * r.Et / rNX));
        std::printf("(R): %g ms\n", 1000 * std::sqrt(2 * r.Er / rNX));
        const struct { const char* tag; int raw, reg; } parts[] = {
            {"RT", PFAST_INV_GRAD_RAW, PFAST_INV_GRAD}, {"R", PFAST_INV_GR_RAW, PFAST_INV_GR},
            {"T", PFAST_INV_GT_RAW, PFAST_INV_GT}};
        for (const auto& q : parts) {
            drv::check(pfast_inversion_get(inv, q.raw, buf.data()), "inversion_get");
            std::snprintf(name, sizeof name, "_bf_regu_%s%d", q.tag, Iterk);
            drv::writemod_logged(p + name, buf.data(), N);
            drv::check(pfast_inversion_get(inv, q.reg, buf.data()), "inversion_get");
            std::snprintf(name, sizeof name, "_af_regu_%s%d", q.tag, Iterk);
            drv::writemod_logged(p + name, buf.data(), N);
        }
        if (FILE* fe = std::fopen((p + "_GlobalErr_TR_T_R.txt").c_str(), "w")) {
            for (size_t i = 0; i < gE.size(); ++i) std::fprintf(fe, "%g\t%g\t%g\n", gE[i], gEt[i], gEr[i]);
            std::fclose(fe);
        }
        drv::print_linesearch(r, lsrc, schemetag, 2);
        drv::check(pfast_inversion_get(inv, PFAST_INV_VP, buf.data()), "inversion_get");
        std::snprintf(name, sizeof name, "_%d", Iterk);
        drv::writemod_logged(p + name, buf.data(), N);
        if (st == PFAST_ERR_OVER_CORRECTED) {
            std::printf("Over corrected..abort...\n");
            return 1;
        }
        conv = r.converged != 0;
        std::printf("--------Interating No. %d takes %10.4f seconds---------------\n\n", Iterk, wall_s(tic));
    }
    if (Iterk > MAXIter) Iterk = MAXIter;
    drv::check(pfast_inversion_get(inv, PFAST_INV_VP, buf.data()), "inversion_get");
    drv::writemod_logged(vpfile, buf.data(), N);
    if (FILE* fe = std::fopen((p + "_AveRes_TR_T_R.txt").c_str(), "w")) {
        for (size_t i = 0; i < gE.size(); ++i)
            std::fprintf(fe, "%g\t%g\t%g\n", 1000 * std::sqrt(2 * gE[i] / rNX), 1000 * std::sqrt(2 * gEt[i] / rNX),
                         1000 * std::sqrt(2 * gEr[i] / rNX));
        std::fclose(fe);
    }
    pfast_inversion_destroy(inv);
    pfast_survey2d_destroy(sv);
    pfast_ctx_destroy(ctx);
    const double sec = wall_s(t0);
    std::printf("Total Elapse Time: %10.4f seconds (%8.4f hours) \n", sec, sec / 3600.0);
    return 0;
}
