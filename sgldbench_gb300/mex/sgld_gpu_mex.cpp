/*
 * sgld_gpu_mex.cpp -- MATLAB MEX gateway of the GB300 solver.
 *
 * One mexFunction, first argument a command string; the solver context
 * persists between calls (one per MATLAB session).  Each command replaces one
 * function of SGLDBench's solve path and keeps its argument meaning:
 *
 *   sgld_gpu_mex('create', voxelizedVolume, numLevels, nonDyadic, poissonRatio, cellSize, omega)
 *        FEA_VoxelBasedDiscretization.m + Solving_BuildingMeshHierarchy.m (padded grid)
 *   sgld_gpu_mex('fixed', fixedDOFs)            FEA_SetupVoxelBased.m:13-26 (logical numDOFs)
 *   sgld_gpu_mex('modulus', eleModulus)         meshHierarchy_(1).eleModulus
 *   nLev = sgld_gpu_mex('hierarchy', numLevels[, nonDyadic])
 *                                               Solving_BuildingMeshHierarchy.m (rebuild)
 *   sgld_gpu_mex('assemble')                    Solving_AssembleFEAstencil.m
 *   y = sgld_gpu_mex('kbyu', u[, precision])    Solving_KbyU_MatrixFree.m
 *   z = sgld_gpu_mex('vcycle', r[, precision])  Solving_Vcycle.m
 *       precision as for pcg: the operator that solve mode applies
 *   [U, its] = sgld_gpu_mex('pcg', F, tol, maxIT[, U0[, 'fp64' | 'mixed' | 'mixed64']])
 *       'mixed' = SGLD_PREC_MIXED_DF, 'mixed64' = SGLD_PREC_MIXED
 *                                               Solving_PreconditionedConjugateGradientSolver.m
 *   ce = sgld_gpu_mex('compliance', U)          TopOpti_ComputeUnitCompliance.m
 *   [s, vm, vmE] = sgld_gpu_mex('stress', U)    FEA_StressAnalysis.m, FEA_ComputePerElementVonMisesStress.m
 *   y = sgld_gpu_mex('filter', x, rMin)         TopOpti_PerformDensityFiltering_mex
 *   sgld_gpu_mex('destroy')
 *
 * Errors become mexErrMsgIdAndTxt (the reference's error behaviour); a PCG
 * that reaches maxIT warns, as Solving_PreconditionedConjugateGradientSolver.m:32-35.
 * Build with MATLAB:  mex -R2018a sgld_gpu_mex.cpp -I<repo>/include -L<lib dir> -lsgld_gb300
 */
#include <stdint.h>
#include <string.h>

#include <vector>

#include "mex.h"
#include "sgld_gpu.h"

static sgld_ctx *g_ctx = nullptr;

// MATLAB calls this when the MEX file is cleared (clear mex, clear all) or
// exits, so that the context's device memory goes with it
static void release_ctx(void) {
    if (g_ctx) sgld_destroy(g_ctx);
    g_ctx = nullptr;
}

static void check(int rc) {
    if (rc != SGLD_OK) mexErrMsgIdAndTxt("sgld:gpu", "%s", g_ctx ? sgld_last_error(g_ctx) : "no context");
}

// 'fp64' (the reference form), 'mixed' (FP32 inner operators with the
// double-float outer K*u) or 'mixed64' (FP32 inner, FP64 outer) -> SGLD_PREC_*
static int precision_arg(const mxArray *a) {
    char mode[16] = {0};
    mxGetString(a, mode, sizeof mode);
    if (!strcmp(mode, "fp64")) return SGLD_PREC_FP64;
    if (!strcmp(mode, "mixed")) return SGLD_PREC_MIXED_DF;
    if (!strcmp(mode, "mixed64")) return SGLD_PREC_MIXED;
    mexErrMsgIdAndTxt("sgld:arg", "precision must be 'fp64', 'mixed' or 'mixed64'");
    return SGLD_PREC_FP64;
}

static void need_ctx() {
    if (!g_ctx) mexErrMsgIdAndTxt("sgld:state", "call sgld_gpu_mex('create', ...) first");
}

static const double *dvec(const mxArray *a, size_t n, const char *what) {
    if (!mxIsDouble(a) || mxGetNumberOfElements(a) != n)
        mexErrMsgIdAndTxt("sgld:arg", "%s must be a double vector of %zu entries", what, n);
    return mxGetPr(a);
}

static int64_t level_count(int what) {
    int64_t ne = 0, nn = 0;
    int res[3], span;
    check(sgld_level_info(g_ctx, 1, res, &span, &ne, &nn));
    return what == 0 ? ne : 3 * nn;
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
    char cmd[32] = {0};
    if (nrhs < 1 || mxGetString(prhs[0], cmd, sizeof cmd) != 0)
        mexErrMsgIdAndTxt("sgld:arg", "first argument must be a command string");
    if (!strcmp(cmd, "create")) {
        if (nrhs < 2) mexErrMsgIdAndTxt("sgld:arg", "create needs the voxel grid");
        const mxArray *v = prhs[1];
        if (mxGetNumberOfDimensions(v) != 3) mexErrMsgIdAndTxt("sgld:arg", "voxel grid must be 3-D");
        const mwSize *d = mxGetDimensions(v);
        const size_t n = d[0] * d[1] * d[2];
        std::vector<uint8_t> solid(n);
        if (mxIsLogical(v) || mxGetClassID(v) == mxUINT8_CLASS) {
            const uint8_t *p = (const uint8_t *)mxGetData(v);
            for (size_t i = 0; i < n; ++i) solid[i] = p[i] ? 1 : 0;
        } else if (mxIsDouble(v)) {
            const double *p = mxGetPr(v);
            for (size_t i = 0; i < n; ++i) solid[i] = p[i] != 0.0;
        } else {
            mexErrMsgIdAndTxt("sgld:arg", "voxel grid must be logical, uint8 or double");
        }
        sgld_options o;
        sgld_default_options(&o);
        if (nrhs > 2) o.num_levels = (int)mxGetScalar(prhs[2]);
        if (nrhs > 3) o.non_dyadic = (int)mxGetScalar(prhs[3]);
        if (nrhs > 4) o.poisson_ratio = mxGetScalar(prhs[4]);
        if (nrhs > 5) o.cell_size = mxGetScalar(prhs[5]);
        if (nrhs > 6) o.omega = mxGetScalar(prhs[6]);
        release_ctx();
        mexAtExit(release_ctx);
        const int rc = sgld_create((int)d[0], (int)d[1], (int)d[2], solid.data(), &o, &g_ctx);
        if (rc != SGLD_OK) {
            const char *m = g_ctx ? sgld_last_error(g_ctx) : "create failed";
            char buf[512];
            strncpy(buf, m, sizeof buf - 1);
            buf[sizeof buf - 1] = 0;
            if (g_ctx) sgld_destroy(g_ctx);
            g_ctx = nullptr;
            mexErrMsgIdAndTxt("sgld:gpu", "%s", buf);
        }
        if (nlhs > 0) plhs[0] = mxCreateDoubleScalar(sgld_num_levels(g_ctx));
        return;
    }
    if (!strcmp(cmd, "destroy")) {
        release_ctx();
        return;
    }
    need_ctx();
    const size_t ndof = (size_t)level_count(1), nel = (size_t)level_count(0);
    if (!strcmp(cmd, "fixed")) {
        if (nrhs < 2 || mxGetNumberOfElements(prhs[1]) != ndof)
            mexErrMsgIdAndTxt("sgld:arg", "fixedDOFs must have numDOFs entries");
        std::vector<uint8_t> f(ndof);
        if (mxIsLogical(prhs[1])) {
            const uint8_t *p = (const uint8_t *)mxGetData(prhs[1]);
            for (size_t i = 0; i < ndof; ++i) f[i] = p[i] ? 1 : 0;
        } else {
            const double *p = dvec(prhs[1], ndof, "fixedDOFs");
            for (size_t i = 0; i < ndof; ++i) f[i] = p[i] != 0.0;
        }
        check(sgld_set_fixed_dofs(g_ctx, f.data()));
    } else if (!strcmp(cmd, "modulus")) {
        check(sgld_set_modulus(g_ctx, dvec(prhs[1], nel, "eleModulus")));
    } else if (!strcmp(cmd, "assemble")) {
        check(sgld_assemble(g_ctx));
    } else if (!strcmp(cmd, "hierarchy")) {
        // Solving_BuildingMeshHierarchy() for numLevels_ / nonDyadic_; fixed DOFs
        // and moduli are set again afterwards
        if (nrhs < 2) mexErrMsgIdAndTxt("sgld:arg", "hierarchy needs numLevels [, nonDyadic]");
        check(sgld_build_hierarchy(g_ctx, (int)mxGetScalar(prhs[1]), nrhs > 2 ? (int)mxGetScalar(prhs[2]) : 0));
        if (nlhs > 0) plhs[0] = mxCreateDoubleScalar(sgld_num_levels(g_ctx));
    } else if (!strcmp(cmd, "kbyu") || !strcmp(cmd, "vcycle")) {
        // optional third argument: the operator of a solve mode (precision_arg)
        const double *u = dvec(prhs[1], ndof, "vector");
        const int prec = nrhs > 2 ? precision_arg(prhs[2]) : SGLD_PREC_FP64;
        plhs[0] = mxCreateDoubleMatrix(ndof, 1, mxREAL);
        check(cmd[0] == 'k' ? sgld_kbyu_prec(g_ctx, u, mxGetPr(plhs[0]), prec)
                            : sgld_vcycle_prec(g_ctx, u, mxGetPr(plhs[0]), prec));
    } else if (!strcmp(cmd, "pcg")) {
        if (nrhs < 4) mexErrMsgIdAndTxt("sgld:arg", "pcg needs F, tol, maxIT");
        const double *F = dvec(prhs[1], ndof, "F");
        sgld_solve_opts o;
        memset(&o, 0, sizeof o);
        o.tol = mxGetScalar(prhs[2]);
        o.maxit = (int)mxGetScalar(prhs[3]);
        o.precision = SGLD_PREC_FP64;
        plhs[0] = mxCreateDoubleMatrix(ndof, 1, mxREAL);
        if (nrhs > 4 && mxGetNumberOfElements(prhs[4]) == ndof) {
            memcpy(mxGetPr(plhs[0]), dvec(prhs[4], ndof, "U0"), ndof * sizeof(double));
            o.use_x0 = 1;
        }
        if (nrhs > 5) o.precision = precision_arg(prhs[5]);
        sgld_solve_info info;
        check(sgld_pcg(g_ctx, F, mxGetPr(plhs[0]), &o, &info));
        if (nlhs > 1) plhs[1] = mxCreateDoubleScalar(info.iterations);
        if (!info.converged) {
            mexWarnMsgIdAndTxt("sgld:maxit", "Exceed the maximum iterate numbers");
            mexPrintf("The iterative process stops at residual = %10.4f\n", info.relres);
        }
    } else if (!strcmp(cmd, "compliance")) {
        plhs[0] = mxCreateDoubleMatrix(nel, 1, mxREAL);
        double c = 0.0;
        check(sgld_compliance(g_ctx, dvec(prhs[1], ndof, "U"), mxGetPr(plhs[0]), &c));
        if (nlhs > 1) plhs[1] = mxCreateDoubleScalar(c);
    } else if (!strcmp(cmd, "stress")) {
        const size_t nn = ndof / 3;
        plhs[0] = mxCreateDoubleMatrix(nn, 6, mxREAL);
        std::vector<double> rowmajor(6 * nn), vm(nn);
        mxArray *vme = mxCreateDoubleMatrix(nel, 1, mxREAL);
        check(sgld_stress(g_ctx, dvec(prhs[1], ndof, "U"), rowmajor.data(), vm.data(), mxGetPr(vme)));
        double *s = mxGetPr(plhs[0]);   // MATLAB numNodes x 6, column-major
        for (size_t i = 0; i < nn; ++i)
            for (int k = 0; k < 6; ++k) s[i + nn * k] = rowmajor[6 * i + k];
        if (nlhs > 1) {
            plhs[1] = mxCreateDoubleMatrix(nn, 1, mxREAL);
            memcpy(mxGetPr(plhs[1]), vm.data(), nn * sizeof(double));
        }
        if (nlhs > 2)
            plhs[2] = vme;
        else
            mxDestroyArray(vme);
    } else if (!strcmp(cmd, "filter")) {
        plhs[0] = mxCreateDoubleMatrix(nel, 1, mxREAL);
        check(sgld_density_filter(g_ctx, mxGetScalar(prhs[2]), dvec(prhs[1], nel, "x"), mxGetPr(plhs[0])));
    } else if (!strcmp(cmd, "principal")) {
        // [ps, dir] = ('principal', U): FEA_ComputePrincipalStress.m per node (numNodes x 12),
        // Common_ExtractDominantDirectionsFromPrincipalStressDirections.m per element (numElements x 3)
        const size_t nn = ndof / 3;
        std::vector<double> ps(12 * nn), dir(3 * nel);
        check(sgld_principal_stress(g_ctx, dvec(prhs[1], ndof, "U"), ps.data(), dir.data()));
        plhs[0] = mxCreateDoubleMatrix(nn, 12, mxREAL);
        for (size_t i = 0; i < nn; ++i)
            for (int k = 0; k < 12; ++k) mxGetPr(plhs[0])[i + nn * k] = ps[12 * i + k];
        if (nlhs > 1) {
            plhs[1] = mxCreateDoubleMatrix(nel, 3, mxREAL);
            for (size_t i = 0; i < nel; ++i)
                for (int k = 0; k < 3; ++k) mxGetPr(plhs[1])[i + nel * k] = dir[3 * i + k];
        }
    } else if (!strcmp(cmd, "pdefilter")) {
        // [y, its] = ('pdefilter', x, rHatMin, tol, maxIT): TopOpti_PDEFiltering_matrixFree.m
        if (nrhs < 5) mexErrMsgIdAndTxt("sgld:arg", "pdefilter needs x, rHatMin, tol, maxIT");
        plhs[0] = mxCreateDoubleMatrix(nel, 1, mxREAL);
        int its = 0;
        check(sgld_pde_filter(g_ctx, mxGetScalar(prhs[2]), dvec(prhs[1], nel, "x"), mxGetPr(plhs[0]),
                              mxGetScalar(prhs[3]), (int)mxGetScalar(prhs[4]), &its));
        if (nlhs > 1) plhs[1] = mxCreateDoubleScalar(its);
    } else if (!strcmp(cmd, "passive")) {
        // ('passive', passiveElements_): 1-based element indices, as MATLAB holds them
        const size_t np = mxGetNumberOfElements(prhs[1]);
        const double *p = np ? mxGetPr(prhs[1]) : nullptr;
        std::vector<int64_t> e(np);
        for (size_t i = 0; i < np; ++i) {
            if (!(p[i] >= 1.0 && p[i] <= (double)nel)) mexErrMsgIdAndTxt("sgld:arg", "passive element out of range");
            e[i] = (int64_t)p[i] - 1;
        }
        check(sgld_set_passive(g_ctx, (int64_t)np, e.data()));
    } else if (!strcmp(cmd, "mma")) {
        // [xmma, xold1, xold2] = ('mma', m, n, xval, xmin, xmax, xold1, xold2, df0dx, fval, dfdx): MMA_mex.cpp
        if (nrhs < 11) mexErrMsgIdAndTxt("sgld:arg", "mma needs m, n, xval, xmin, xmax, xold1, xold2, df0dx, fval, dfdx");
        const int mm = (int)mxGetScalar(prhs[1]), n = (int)mxGetScalar(prhs[2]);
        if (mm < 1 || n < 1) mexErrMsgIdAndTxt("sgld:arg", "m and n must be positive");
        const size_t un = (size_t)n;
        plhs[0] = mxCreateDoubleMatrix(un, 1, mxREAL);
        mxArray *o1 = mxCreateDoubleMatrix(un, 1, mxREAL), *o2 = mxCreateDoubleMatrix(un, 1, mxREAL);
        check(sgld_mma_update(g_ctx, mm, n, dvec(prhs[3], un, "xval"), dvec(prhs[4], un, "xmin"),
                              dvec(prhs[5], un, "xmax"), dvec(prhs[6], un, "xold1"), dvec(prhs[7], un, "xold2"),
                              dvec(prhs[8], un, "df0dx"), dvec(prhs[9], (size_t)mm, "fval"),
                              dvec(prhs[10], un * mm, "dfdx"), mxGetPr(plhs[0]), mxGetPr(o1), mxGetPr(o2)));
        if (nlhs > 1) plhs[1] = o1; else mxDestroyArray(o1);
        if (nlhs > 2) plhs[2] = o2; else mxDestroyArray(o2);
    } else if (!strcmp(cmd, "topopt") || !strcmp(cmd, "topopt_local")) {
        // [xPhys, hist] = ('topopt', F, V, rMin, nLoop, tol, maxIT[, 'OC'|'MMA'])
        //   TopOpti_GlobalVolumeConstraint_Tmp.m;
        // [xPhys, hist] = ('topopt_local', F, alphaMin, rMin, rHatMin, p, nLoop, tol, maxIT)
        //   TopOpti_LocalVolumeConstraint.m.
        // hist: one row per iteration [compliance volume sharpness change constraint iterations]
        const bool local = cmd[6] == '_';
        if (nrhs < (local ? 9 : 7)) mexErrMsgIdAndTxt("sgld:arg", "too few arguments for %s", cmd);
        const double *F = dvec(prhs[1], ndof, "F");
        sgld_solve_opts so;
        memset(&so, 0, sizeof so);
        so.precision = SGLD_PREC_FP64;
        int nloop = 0, nit = 0;
        std::vector<sgld_topopt_iter> hist;
        plhs[0] = mxCreateDoubleMatrix(nel, 1, mxREAL);
        if (local) {
            sgld_topopt_projected_opts o;
            memset(&o, 0, sizeof o);
            o.constraint = SGLD_CONS_LOCAL;
            o.alpha = mxGetScalar(prhs[2]);
            o.rmin = mxGetScalar(prhs[3]);
            o.rhat = mxGetScalar(prhs[4]);
            o.pnorm = mxGetScalar(prhs[5]);
            nloop = o.n_loop = (int)mxGetScalar(prhs[6]);
            so.tol = mxGetScalar(prhs[7]);
            so.maxit = (int)mxGetScalar(prhs[8]);
            o.penalty_increment = 0.2;    // penaltyIncrement_ (Data_GlobalVariables.m:73)
            o.penalty_interval = 30;      // penaltyUpdateIterations_ (:74)
            o.solve = so;
            if (nloop < 1) mexErrMsgIdAndTxt("sgld:arg", "nLoop must be positive");
            hist.resize((size_t)nloop);
            check(sgld_topopt_projected(g_ctx, &o, F, mxGetPr(plhs[0]), hist.data(), &nit));
        } else {
            sgld_topopt_opts o;
            memset(&o, 0, sizeof o);
            o.volfrac = mxGetScalar(prhs[2]);
            o.rmin = mxGetScalar(prhs[3]);
            nloop = o.n_loop = (int)mxGetScalar(prhs[4]);
            so.tol = mxGetScalar(prhs[5]);
            so.maxit = (int)mxGetScalar(prhs[6]);
            o.solve = so;
            if (nrhs > 7) {
                char opt[8] = {0};
                mxGetString(prhs[7], opt, sizeof opt);
                if (!strcmp(opt, "MMA")) o.optimizer = SGLD_OPT_MMA;
                else if (strcmp(opt, "OC")) mexErrMsgIdAndTxt("sgld:arg", "optimizer must be 'OC' or 'MMA'");
            }
            if (nloop < 1) mexErrMsgIdAndTxt("sgld:arg", "nLoop must be positive");
            hist.resize((size_t)nloop);
            check(sgld_topopt(g_ctx, &o, F, nullptr, mxGetPr(plhs[0]), hist.data(), &nit));
        }
        if (nlhs > 1) {
            plhs[1] = mxCreateDoubleMatrix((size_t)nit, 6, mxREAL);
            double *h = mxGetPr(plhs[1]);
            for (int i = 0; i < nit; ++i) {
                const sgld_topopt_iter &r = hist[(size_t)i];
                const double row[6] = {r.compliance, r.volume, r.sharpness, r.change, r.constraint,
                                       (double)r.cg_iterations};
                for (int k = 0; k < 6; ++k) h[i + (size_t)nit * k] = row[k];
            }
        }
    } else {
        mexErrMsgIdAndTxt("sgld:arg", "unknown command '%s'", cmd);
    }
}
