// C ABI of the SIMP loop and the density filter (include/sgld_gpu.h):
// TopOpti_GlobalVolumeConstraint_Tmp.m:26-120 driven from the host, every
// field operation on the device.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <utility>

#include "../../include/sgld_gpu.h"
#include "sgld_internal.cuh"

using namespace sgld;

namespace {

int tfail(sgld_ctx *ctx, int code, const std::string &m) {
    ctx->c.err = m;
    return code;
}

#define TCK(x)                                                                                  \
    do {                                                                                        \
        cudaError_t e_ = (x);                                                                   \
        if (e_ != cudaSuccess) return tfail(ctx, SGLD_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

enum { OC_MID = 2, OC_G = 3, OC_DONE = 4, OC_STEPS = 5, T_SHARP = 8, T_C = 9, T_CHANGE = 10, T_VOL = 11 };

int ensure_topo(sgld_ctx *ctx) {
    Ctx &c = ctx->c;
    if (c.t_x) return SGLD_OK;
    const size_t n = (size_t)c.lv[0].nel;
    for (double **p : {&c.t_x, &c.t_xp, &c.t_hs, &c.t_ce, &c.t_dcs, &c.t_dvs, &c.t_dc, &c.t_dv, &c.t_q, &c.t_tmp}) {
        cudaError_t e = cudaMalloc((void **)p, n * sizeof(double));
        if (e != cudaSuccess) return tfail(ctx, SGLD_ERR_NOMEM, "SIMP-loop buffers: out of device memory");
    }
    TCK(cudaMalloc((void **)&c.t_st, 16 * sizeof(double)));
    return SGLD_OK;
}

// weights for this rmin and the weight sums Hs in t_hs
int setup_filter(sgld_ctx *ctx, double rmin, int *radius) {
    Ctx &c = ctx->c;
    if (!(rmin > 0.0) || (int)ceil(rmin) - 1 > 3) return tfail(ctx, SGLD_ERR_ARG, "rmin must be in (0, 4]");
    int r = 0;
    if (!c.t_fw) TCK(cudaMalloc((void **)&c.t_fw, sizeof(double) * 7 * 7 * 7));
    upload_filter_weights(rmin, &r, c.t_fw, c.stream);
    if (c.t_rmin != rmin) {
        launch_density_filter(c.lv[0], nullptr, r, c.t_fw, c.t_hs, c.stream);
        c.t_rmin = rmin;
    }
    *radius = r;
    return SGLD_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

}  // namespace

extern "C" int sgld_density_filter(sgld_ctx *ctx, double rmin, const double *x, double *y) {
    if (!ctx || !y) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    Ctx &c = ctx->c;
    int rc = ensure_topo(ctx);
    if (rc) return rc;
    int r = 0;
    if ((rc = setup_filter(ctx, rmin, &r))) return rc;
    const int64_t ne = (int64_t)c.h_elemap.size();
    const Level &l0 = c.lv[0];
    if (x) {
        TCK(cudaMemcpyAsync(c.d_tmp, x, sizeof(double) * ne, cudaMemcpyHostToDevice, c.stream));
        TCK(cudaMemsetAsync(c.t_tmp, 0, sizeof(double) * l0.nel, c.stream));
        launch_scatter_elems(c.d_elemap, ne, c.d_tmp, c.t_tmp, c.stream);
        launch_density_filter(l0, c.t_tmp, r, c.t_fw, c.t_q, c.stream);
        launch_gather_elems(c.d_elemap, ne, c.t_q, c.d_tmp, c.stream);
    } else {
        launch_gather_elems(c.d_elemap, ne, c.t_hs, c.d_tmp, c.stream);
    }
    TCK(cudaGetLastError());
    TCK(cudaMemcpyAsync(y, c.d_tmp, sizeof(double) * ne, cudaMemcpyDeviceToHost, c.stream));
    TCK(cudaStreamSynchronize(c.stream));
    return SGLD_OK;
}

namespace {

// K_pde = r^2 dN'dN + N' diag(w detJ) N (TopOpti_BuildPDEfilter_matrixFree.m:9-20):
// dN = shape-function derivatives in natural coordinates at the 8 Gauss
// points (FEA_DeShapeFunction.m), unit cell (detJ = 1/8, weights 1),
// r = rHatMin / (2 sqrt(3)); row-major 8 x 8 in the reference's node order
void pde_element_matrix(double rhat, double K[64]) {
    const double g = 0.577350269189626;   // FEA_GaussianIntegral.m:10-15
    const double gs[8] = {-g, g, g, -g, -g, g, g, -g}, gt[8] = {-g, -g, g, g, -g, -g, g, g},
                 gp[8] = {-g, -g, -g, -g, g, g, g, g};
    const double ns[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, nt[8] = {-1, -1, 1, 1, -1, -1, 1, 1},
                 np[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
    double dN[24][8], N[8][8];
    for (int q = 0; q < 8; ++q)
        for (int n = 0; n < 8; ++n) {
            dN[3 * q][n] = 0.125 * ns[n] * (1 + nt[n] * gt[q]) * (1 + np[n] * gp[q]);
            dN[3 * q + 1][n] = 0.125 * nt[n] * (1 + ns[n] * gs[q]) * (1 + np[n] * gp[q]);
            dN[3 * q + 2][n] = 0.125 * np[n] * (1 + ns[n] * gs[q]) * (1 + nt[n] * gt[q]);
            N[q][n] = 0.125 * (1 + ns[n] * gs[q]) * (1 + nt[n] * gt[q]) * (1 + np[n] * gp[q]);
        }
    const double ir = rhat / 2.0 / sqrt(3.0);
    for (int a = 0; a < 8; ++a)
        for (int b = 0; b < 8; ++b) {
            double k0 = 0.0, k1 = 0.0;
            for (int r = 0; r < 24; ++r) k0 += dN[r][a] * dN[r][b];
            for (int q = 0; q < 8; ++q) k1 += N[q][a] * (1.0 / 8.0) * N[q][b];
            K[8 * a + b] = ir * ir * k0 + k1;
        }
}

}  // namespace

namespace {

// the scalar part of MMAseq::SolveDIP (MMAseq.cpp:191-245) for m = 1,
// a = 0, c = 100, d = 0; every evaluation of x(lambda) and its two sums is a
// device pass over the n variables (launch_mma_eval)
int mma_solve_device(sgld_ctx *ctx, int64_t n, const double *xv, const double *xmin, const double *xmax,
                     const double *df0, const double *dg, double gval, double *xout, double *part1, double *part2,
                     double *d_sums, int *newton_steps) {
    Ctx &c = ctx->c;
    double h[2];
    auto eval = [&](double lam) -> int {
        launch_mma_eval(xv, xmin, xmax, df0, dg, n, lam, xout, part1, part2, d_sums, c.stream);
        TCK(cudaGetLastError());
        TCK(cudaMemcpyAsync(h, d_sums, sizeof h, cudaMemcpyDeviceToHost, c.stream));
        TCK(cudaStreamSynchronize(c.stream));
        return SGLD_OK;
    };
    int rc;
    if ((rc = eval(-1.0))) return rc;
    const double b = -gval + h[0];
    const double cc = 100.0;
    double lam = cc / 2.0, mu = 1.0;
    const double tol = 1.0e-9 * sqrt(1.0 + (double)n);
    double epsi = 1.0, err = 1.0;
    int steps = 0;
    lam = fmax(lam, 0.0);
    if ((rc = eval(lam))) return rc;
    while (epsi > tol) {
        int loop = 0;
        while (err > 0.9 * epsi && loop < 100) {
            ++loop;
            ++steps;
            lam = fmax(lam, 0.0);
            const double y = fmax(0.0, lam - cc);
            double grad = -b - y + h[0];
            grad = -grad - epsi / lam;
            double H = h[1];
            if (lam > cc) H += -1.0;
            H += -mu / lam;
            double corr = 1e-4 * H;
            if (-corr < 1.0e-7) corr = -1.0e-7;
            H += corr;
            const double s0 = grad / H;
            const double s1 = -mu + epsi / lam - s0 * mu / lam;
            double theta = 1.005;
            if (theta < -1.01 * s0 / lam) theta = -1.01 * s0 / lam;
            if (theta < -1.01 * s1 / mu) theta = -1.01 * s1 / mu;
            theta = 1.0 / theta;
            lam += theta * s0;
            mu += theta * s1;
            lam = fmax(lam, 0.0);
            if ((rc = eval(lam))) return rc;
            const double y2 = fmax(0.0, lam - cc);
            err = fmax(fabs(-b - y2 + mu + h[0]), fabs(mu * lam - epsi));
        }
        epsi *= 0.1;
    }
    if (newton_steps) *newton_steps = steps;
    return SGLD_OK;
}

}  // namespace

extern "C" int sgld_mma_update(sgld_ctx *ctx, int m, int n, const double *xval, const double *xmin,
                               const double *xmax, const double *xold1, const double *xold2, const double *df0dx,
                               const double *fval, const double *dfdx, double *xnew, double *xold1_out,
                               double *xold2_out) {
    if (!ctx) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    if (m != 1) return tfail(ctx, SGLD_ERR_ARG, "sgld_mma_update supports one constraint (m = 1)");
    if (n < 1 || !xval || !xmin || !xmax || !xold1 || !df0dx || !fval || !dfdx || !xnew)
        return tfail(ctx, SGLD_ERR_ARG, "null argument or n < 1");
    (void)xold2;
    Ctx &c = ctx->c;
    const int nb = mma_blocks(n);
    double *d = nullptr;
    const size_t words = 6 * (size_t)n + 2 * (size_t)nb + 2;
    TCK(cudaMalloc((void **)&d, words * sizeof(double)));
    double *dx = d, *dmin = d + n, *dmax = d + 2 * (size_t)n, *ddf0 = d + 3 * (size_t)n, *ddg = d + 4 * (size_t)n,
           *dout = d + 5 * (size_t)n, *p1 = d + 6 * (size_t)n, *p2 = p1 + nb, *sums = p2 + nb;
    const size_t bytes = sizeof(double) * (size_t)n;
    int rc = SGLD_OK;
    cudaError_t e = cudaSuccess;
    for (auto pr : {std::make_pair(dx, xval), std::make_pair(dmin, xmin), std::make_pair(dmax, xmax),
                    std::make_pair(ddf0, df0dx), std::make_pair(ddg, dfdx)})
        if (e == cudaSuccess) e = cudaMemcpyAsync(pr.first, pr.second, bytes, cudaMemcpyHostToDevice, c.stream);
    if (e != cudaSuccess) {
        cudaFree(d);
        return tfail(ctx, SGLD_ERR_CUDA, std::string("sgld_mma_update upload: ") + cudaGetErrorString(e));
    }
    rc = mma_solve_device(ctx, n, dx, dmin, dmax, ddf0, ddg, fval[0], dout, p1, p2, sums, nullptr);
    if (rc == SGLD_OK) {
        e = cudaMemcpyAsync(xnew, dout, bytes, cudaMemcpyDeviceToHost, c.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
        if (e != cudaSuccess) rc = tfail(ctx, SGLD_ERR_CUDA, std::string("sgld_mma_update: ") + cudaGetErrorString(e));
    }
    cudaFree(d);
    if (rc) return rc;
    // MMAseq::Update: xo2 <- xo1 (the incoming xold1), xo1 <- xval
    if (xold1_out) memcpy(xold1_out, xval, bytes);
    if (xold2_out) memcpy(xold2_out, xold1, bytes);
    return SGLD_OK;
}

namespace {

// TopOpti_PDEFiltering_matrixFree.m:1-36 on full-grid element fields xe -> ye
// (device): element -> node (x/8 to each corner), Jacobi-preconditioned PCG on
// K_pde from 0 (Solving_PreconditionedConjugateGradientSolver.m), node ->
// element (mean of the 8 corners).  Scratch: its own node vectors, so the
// elasticity solve's vectors (U, F) survive.
int pde_filter_dev(sgld_ctx *ctx, double rhat, const double *xe, double *ye, double tol, int maxit, int *iterations) {
    Ctx &c = ctx->c;
    const Level &l0 = c.lv[0];
    const int64_t nn = l0.nnode;
    if (!c.t_pde) TCK(cudaMalloc((void **)&c.t_pde, 7 * sizeof(double) * (size_t)nn));
    double *b = c.t_pde, *x = b + nn, *r = x + nn, *z = r + nn, *p = z + nn, *q = p + nn, *dinv = q + nn;
    double K[64];
    pde_element_matrix(rhat, K);
    if (!c.t_kp) TCK(cudaMalloc((void **)&c.t_kp, sizeof(double) * 64));
    upload_kpde(K, c.t_kp, c.stream);
    launch_pde_e2n(l0, xe, b, c.stream);
    launch_pde_diag(l0, c.t_kp, dinv, c.stream);
    const int nbv = reduce_blocks(nn);
    launch_pcg_scalar(5, c.d_scal, c.d_iflag, c.d_part, 1, tol, maxit, c.stream);
    launch_dot(b, b, nn, c.d_part, nbv, c.stream);
    launch_pcg_scalar(0, c.d_scal, c.d_iflag, c.d_part, nbv, tol, maxit, c.stream);
    TCK(cudaMemsetAsync(x, 0, sizeof(double) * nn, c.stream));
    TCK(cudaMemcpyAsync(r, b, sizeof(double) * nn, cudaMemcpyDeviceToDevice, c.stream));
    launch_pde_jacobi(r, dinv, nn, z, c.d_part, nbv, c.stream);
    launch_pcg_scalar(1, c.d_scal, c.d_iflag, c.d_part, nbv, tol, maxit, c.stream);
    TCK(cudaMemcpyAsync(p, z, sizeof(double) * nn, cudaMemcpyDeviceToDevice, c.stream));
    int h_flag[4] = {0, 0, 0, 0};
    for (int k = 1; k <= maxit; ++k) {
        const int nb = launch_pde_kbyu(l0, c.t_kp, p, q, c.d_part, c.stream);
        launch_pcg_scalar(2, c.d_scal, c.d_iflag, c.d_part, nb, tol, maxit, c.stream);
        launch_pcg_update(x, r, p, q, nn, c.d_scal, c.d_iflag, c.d_part, nbv, c.stream);
        launch_pcg_scalar(3, c.d_scal, c.d_iflag, c.d_part, nbv, tol, maxit, c.stream);
        TCK(cudaMemcpyAsync(h_flag, c.d_iflag, sizeof(int) * 4, cudaMemcpyDeviceToHost, c.stream));
        TCK(cudaStreamSynchronize(c.stream));
        if (h_flag[2]) break;
        launch_pde_jacobi(r, dinv, nn, z, c.d_part, nbv, c.stream);
        launch_pcg_scalar(4, c.d_scal, c.d_iflag, c.d_part, nbv, tol, maxit, c.stream);
        launch_pcg_pupdate(p, z, nn, c.d_scal, c.d_iflag, c.stream);
    }
    launch_pde_n2e(l0, x, ye, c.stream);
    TCK(cudaGetLastError());
    if (iterations) *iterations = h_flag[0];
    return SGLD_OK;
}

}  // namespace

extern "C" int sgld_pde_filter(sgld_ctx *ctx, double rhat, const double *x, double *y, double tol, int maxit,
                               int *iterations) {
    if (!ctx || !x || !y) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    Ctx &c = ctx->c;
    if (!(rhat > 0.0) || maxit < 1 || !(tol >= 0.0)) return tfail(ctx, SGLD_ERR_ARG, "rhat > 0, maxit >= 1, tol >= 0");
    int rc = ensure_topo(ctx);
    if (rc) return rc;
    const Level &l0 = c.lv[0];
    const int64_t ne = (int64_t)c.h_elemap.size();
    TCK(cudaMemcpyAsync(c.d_tmp, x, sizeof(double) * ne, cudaMemcpyHostToDevice, c.stream));
    TCK(cudaMemsetAsync(c.t_tmp, 0, sizeof(double) * l0.nel, c.stream));
    launch_scatter_elems(c.d_elemap, ne, c.d_tmp, c.t_tmp, c.stream);
    if ((rc = pde_filter_dev(ctx, rhat, c.t_tmp, c.t_q, tol, maxit, iterations))) return rc;
    launch_gather_elems(c.d_elemap, ne, c.t_q, c.d_tmp, c.stream);
    TCK(cudaGetLastError());
    TCK(cudaMemcpyAsync(y, c.d_tmp, sizeof(double) * ne, cudaMemcpyDeviceToHost, c.stream));
    TCK(cudaStreamSynchronize(c.stream));
    return SGLD_OK;
}

extern "C" int sgld_set_passive(sgld_ctx *ctx, int64_t n, const int64_t *elements) {
    if (!ctx || n < 0 || (n > 0 && !elements)) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    Ctx &c = ctx->c;
    const int64_t ne = (int64_t)c.h_elemap.size();
    std::vector<int64_t> full((size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        if (elements[i] < 0 || elements[i] >= ne) return tfail(ctx, SGLD_ERR_ARG, "passive element index out of range");
        full[i] = c.h_elemap[elements[i]];
    }
    std::sort(full.begin(), full.end());
    full.erase(std::unique(full.begin(), full.end()), full.end());
    int64_t *d_full = nullptr;
    if (!full.empty()) {
        TCK(cudaMalloc((void **)&d_full, sizeof(int64_t) * full.size()));
        TCK(cudaMemcpyAsync(d_full, full.data(), sizeof(int64_t) * full.size(), cudaMemcpyHostToDevice, c.stream));
    }
    launch_mark_passive(c.lv[0], d_full, (int64_t)full.size(), reduce_blocks(c.lv[0].nel), c.stream);
    const cudaError_t e = cudaStreamSynchronize(c.stream);
    if (d_full) cudaFree(d_full);
    TCK(e);
    c.h_passive = std::move(full);
    return SGLD_OK;
}

extern "C" int sgld_topopt(sgld_ctx *ctx, const sgld_topopt_opts *opts, const double *F, const double *x0,
                           double *xphys, sgld_topopt_iter *hist, int *n_iter) {
    if (!ctx || !opts || !F) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    Ctx &c = ctx->c;
    if (!c.have_fixed) return tfail(ctx, SGLD_ERR_STATE, "fixed DOFs not set (sgld_set_fixed_dofs)");
    sgld_topopt_opts o = *opts;
    if (o.move == 0) o.move = 0.1;
    if (o.min_change == 0) o.min_change = 1e-4;
    if (o.max_sharpness == 0) o.max_sharpness = 0.05;
    if (o.penalty == 0) o.penalty = 3.0;
    if (o.E0 == 0) o.E0 = 1.0;
    if (o.Emin == 0) o.Emin = 1e-6;
    if (o.n_loop < 1 || !(o.volfrac > 0.0 && o.volfrac <= 1.0))
        return tfail(ctx, SGLD_ERR_ARG, "n_loop >= 1 and volfrac in (0, 1] required");
    int rc = ensure_topo(ctx);
    if (rc) return rc;
    int r = 0;
    if ((rc = setup_filter(ctx, o.rmin, &r))) return rc;
    const Level &l0 = c.lv[0];
    const int64_t ne = (int64_t)c.h_elemap.size(), nn = (int64_t)c.h_nodemap.size();
    const size_t nv = 3 * (size_t)l0.nnode;
    const int nb = reduce_blocks(l0.nel);
    const double nact = (double)ne;
    cudaStream_t s = c.stream;
    // loads: F -> d_b, U = 0 (TopOpti_CallTopOpti.m:15), x = x0 or volfrac
    TCK(cudaMemsetAsync(c.d_b, 0, sizeof(double) * nv, s));
    TCK(cudaMemsetAsync(c.d_x, 0, sizeof(double) * nv, s));
    TCK(cudaMemcpyAsync(c.d_tmp, F, sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, s));
    launch_scatter_nodes(c.d_nodemap, nn, c.d_tmp, c.d_b, s);
    if (x0) {
        TCK(cudaMemsetAsync(c.t_x, 0, sizeof(double) * l0.nel, s));
        TCK(cudaMemcpyAsync(c.d_tmp, x0, sizeof(double) * ne, cudaMemcpyHostToDevice, s));
        launch_scatter_elems(c.d_elemap, ne, c.d_tmp, c.t_x, s);
    } else {
        launch_fill_active(l0, c.t_x, o.volfrac, nb, s);
    }
    if (o.xphys0) {   // resume: the checkpoint's filtered design
        TCK(cudaMemsetAsync(c.t_xp, 0, sizeof(double) * l0.nel, s));
        TCK(cudaMemcpyAsync(c.d_tmp, o.xphys0, sizeof(double) * ne, cudaMemcpyHostToDevice, s));
        launch_scatter_elems(c.d_elemap, ne, c.d_tmp, c.t_xp, s);
    } else {
        TCK(cudaMemcpyAsync(c.t_xp, c.t_x, sizeof(double) * l0.nel, cudaMemcpyDeviceToDevice, s));
    }
    if (o.U0) {       // resume: the checkpoint's displacement as the first warm start
        TCK(cudaMemcpyAsync(c.d_tmp, o.U0, sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, s));
        launch_scatter_nodes(c.d_nodemap, nn, c.d_tmp, c.d_x, s);
    }
    launch_topo_modulus(l0, c.t_xp, o.penalty, o.E0, o.Emin, c.E, c.d_part, c.d_part2, nb, s);
    launch_finalize_sum(c.d_part, nb, c.t_st + T_VOL, s);
    launch_finalize_sum(c.d_part2, nb, c.t_st + T_SHARP, s);
    c.have_E = true;
    TCK(cudaGetLastError());
    cudaEvent_t ev[5];
    for (auto &e : ev) TCK(cudaEventCreate(&e));
    // MMA: design variables = active elements that are not passive
    int64_t nvar = 0;
    int64_t *d_var = nullptr;
    double *mma_buf = nullptr, *mma_xv = nullptr, *mma_xmin = nullptr, *mma_xmax = nullptr, *mma_df0 = nullptr,
           *mma_dg = nullptr, *mma_xo = nullptr, *mma_p1 = nullptr, *mma_p2 = nullptr, *mma_sums = nullptr;
    struct Free {
        void *a, *b;
        ~Free() {
            if (a) cudaFree(a);
            if (b) cudaFree(b);
        }
    } mma_free{nullptr, nullptr};
    if (o.optimizer == SGLD_OPT_MMA) {
        std::vector<int64_t> var;
        var.reserve(c.h_elemap.size());
        for (int64_t e : c.h_elemap)
            if (!std::binary_search(c.h_passive.begin(), c.h_passive.end(), e)) var.push_back(e);
        nvar = (int64_t)var.size();
        if (nvar == 0) return tfail(ctx, SGLD_ERR_ARG, "MMA: no design variables (every element passive)");
        const int nbm = mma_blocks(nvar);
        TCK(cudaMalloc((void **)&d_var, sizeof(int64_t) * nvar));
        mma_free.a = d_var;
        TCK(cudaMemcpyAsync(d_var, var.data(), sizeof(int64_t) * nvar, cudaMemcpyHostToDevice, s));
        TCK(cudaMalloc((void **)&mma_buf, sizeof(double) * (6 * (size_t)nvar + 2 * (size_t)nbm + 2)));
        mma_free.b = mma_buf;
        mma_xv = mma_buf;
        mma_xmin = mma_xv + nvar;
        mma_xmax = mma_xmin + nvar;
        mma_df0 = mma_xmax + nvar;
        mma_dg = mma_df0 + nvar;
        mma_xo = mma_dg + nvar;
        mma_p1 = mma_xo + nvar;
        mma_p2 = mma_p1 + nbm;
        mma_sums = mma_p2 + nbm;
    } else if (o.optimizer != SGLD_OPT_OC) {
        return tfail(ctx, SGLD_ERR_ARG, "optimizer must be SGLD_OPT_OC or SGLD_OPT_MMA");
    }
    if (o.learned < 0 || o.learned > 2) return tfail(ctx, SGLD_ERR_ARG, "learned must be 0, 1 or 2");
    if (o.learned) {   // a fresh network per loop
        learned_free(c.lws);
        c.lws = nullptr;
        if ((rc = learned_setup(ctx, &c.lws, o.net_level, o.learned == 1))) return rc;
    }
    const int net_steps = o.net_train_steps > 0 ? o.net_train_steps : 4;
    const float net_lr = o.net_lr > 0.f ? o.net_lr : 1e-3f;
    cudaEvent_t evn[4];
    for (auto &e : evn) TCK(cudaEventCreate(&e));
    sgld_solve_opts so = o.solve;
    so.use_x0 = 1;
    so.history = nullptr;
    double change = 1.0, sharp = 1.0;
    const int loop0 = o.loop0 > 0 ? o.loop0 : 0;
    int loop = loop0;
    while (loop < o.n_loop && change > o.min_change && sharp > o.max_sharpness) {   // :47
        ++loop;
        NvtxRange iter_range("SIMP iteration");
        double vol = 0.0;
        TCK(cudaMemcpyAsync(&vol, c.t_st + T_VOL, sizeof(double), cudaMemcpyDeviceToHost, s));
        launch_oc_scalar(0, c.t_st, c.t_st + T_VOL, 1, nact, o.volfrac, s);        // g (:83), bisection bounds
        TCK(cudaEventRecord(ev[0], s));
        if ((rc = sgld_assemble(ctx))) return rc;                                  // :54
        int net_used = 0, net_acc = 0;
        double net_ratio = 0.0, net_ext = 0.0, net_loss = 0.0;
        TCK(cudaEventRecord(evn[0], s));
        if (o.learned &&
            (rc = learned_before_solve(ctx, c.lws, o.learned, o.E0, &net_used, &net_acc, &net_ratio, &net_ext)))
            return rc;
        TCK(cudaEventRecord(evn[1], s));
        TCK(cudaEventRecord(ev[1], s));
        sgld_solve_info si;
        if ((rc = solve_on_device(ctx, &so, &si))) return rc;                      // :57
        TCK(cudaEventRecord(ev[2], s));
        if (o.learned && (rc = learned_after_solve(ctx, c.lws, o.learned, net_steps, net_lr, &net_loss))) return rc;
        TCK(cudaEventRecord(evn[2], s));
        int nbc = 0;
        launch_unit_compliance(l0, c.d_x, c.E, c.t_ce, c.d_part, &nbc, s);        // :59, :63
        launch_finalize_sum(c.d_part, nbc, c.t_st + T_C, s);
        launch_topo_sens(l0, c.t_xp, c.t_ce, c.t_hs, o.penalty, o.E0, o.Emin, c.t_dcs, c.t_dvs, nb, s);   // :66
        TCK(cudaEventRecord(ev[3], s));
        launch_density_filter(l0, c.t_dcs, r, c.t_fw, c.t_dc, s);                          // :76
        launch_density_filter(l0, c.t_dvs, r, c.t_fw, c.t_dv, s);                          // :77
        cudaEvent_t evf;
        TCK(cudaEventCreate(&evf));
        TCK(cudaEventRecord(evf, s));
        if (o.optimizer == SGLD_OPT_MMA) {
            // TopOpti_GlobalVolumeConstraint.m:139-156: one MMA update of the
            // design variables under fval = sum(xPhys)/(n V) - 1 <= 0
            const int nbm = launch_mma_gather(d_var, nvar, c.t_x, c.t_dc, c.t_dv, o.move, 1.0 / (nact * o.volfrac),
                                              mma_xv, mma_xmin, mma_xmax, mma_df0, mma_dg, s);
            const double fval = vol / (nact * o.volfrac) - 1.0;
            if ((rc = mma_solve_device(ctx, nvar, mma_xv, mma_xmin, mma_xmax, mma_df0, mma_dg, fval, mma_xo,
                                       mma_p1, mma_p2, mma_sums, nullptr)))
                return rc;
            if (!c.h_passive.empty()) launch_set_passive_x(l0, c.t_x, nb, s);
            launch_mma_scatter(d_var, nvar, mma_xo, mma_xv, c.t_x, c.d_part, nbm, s);
            launch_max_partials(c.d_part, nbm, c.t_st + T_CHANGE, s);
        } else {
            launch_topo_q(l0, c.t_x, c.t_dc, c.t_dv, c.t_q, nb, s);
            double done = 0.0;
            for (int round = 0; round < 8 && done == 0.0; ++round) {               // :85-90
                for (int k = 0; k < 32; ++k) {
                    launch_oc_step(l0, c.t_x, c.t_q, c.t_dv, o.move, c.t_st, c.d_part, nb, s);
                    launch_oc_scalar(1, c.t_st, c.d_part, nb, nact, o.volfrac, s);
                }
                TCK(cudaMemcpyAsync(&done, c.t_st + OC_DONE, sizeof(double), cudaMemcpyDeviceToHost, s));
                TCK(cudaStreamSynchronize(s));
            }
            launch_oc_apply(l0, c.t_x, c.t_q, o.move, c.t_st, c.d_part, nb, s);   // :91-92
            launch_max_partials(c.d_part, nb, c.t_st + T_CHANGE, s);
        }
        cudaEvent_t evo;
        TCK(cudaEventCreate(&evo));
        TCK(cudaEventRecord(evo, s));
        launch_density_filter(l0, c.t_x, r, c.t_fw, c.t_tmp, s);                           // :99
        launch_div(l0, c.t_tmp, c.t_hs, c.t_xp, nb, s);
        TCK(cudaEventRecord(ev[4], s));
        launch_topo_modulus(l0, c.t_xp, o.penalty, o.E0, o.Emin, c.E, c.d_part, c.d_part2, nb, s);   // :52, :102
        launch_finalize_sum(c.d_part, nb, c.t_st + T_VOL, s);
        launch_finalize_sum(c.d_part2, nb, c.t_st + T_SHARP, s);
        TCK(cudaGetLastError());
        double st[16];
        TCK(cudaMemcpyAsync(st, c.t_st, sizeof st, cudaMemcpyDeviceToHost, s));
        TCK(cudaStreamSynchronize(s));
        change = st[T_CHANGE];
        sharp = st[T_SHARP] / nact;
        if (hist) {
            sgld_topopt_iter &h = hist[loop - 1 - loop0];
            h.loop = loop;
            h.cg_iterations = si.iterations;
            h.compliance = st[T_C];
            h.volume = vol / nact;
            h.sharpness = sharp;
            h.change = change;
            h.constraint = st[OC_G];
            h.t_assemble = elapsed(ev[0], ev[1]) * 1e-3;
            h.t_solve = elapsed(ev[1], ev[2]) * 1e-3;
            h.t_opt = (elapsed(ev[2], ev[3]) + elapsed(evf, evo)) * 1e-3;
            h.t_filter = (elapsed(ev[3], evf) + elapsed(evo, ev[4])) * 1e-3;
            h.inner_iterations = si.inner_iterations;
            h.net_used = net_used;
            h.net_accepted = net_acc;
            h.net_r0_ratio = net_ratio;
            h.ext_r0_ratio = net_ext;
            h.net_loss = net_loss;
            h.t_net = (elapsed(evn[0], evn[1]) + elapsed(ev[2], evn[2])) * 1e-3;
        }
        cudaEventDestroy(evf);
        cudaEventDestroy(evo);
    }
    for (auto &e : ev) cudaEventDestroy(e);
    for (auto &e : evn) cudaEventDestroy(e);
    if (n_iter) *n_iter = loop - loop0;
    if (o.x_out) {
        launch_gather_elems(c.d_elemap, ne, c.t_x, c.d_tmp, s);
        TCK(cudaMemcpyAsync(o.x_out, c.d_tmp, sizeof(double) * ne, cudaMemcpyDeviceToHost, s));
        TCK(cudaStreamSynchronize(s));
    }
    if (xphys) {
        launch_gather_elems(c.d_elemap, ne, c.t_xp, c.d_tmp, s);
        TCK(cudaMemcpyAsync(xphys, c.d_tmp, sizeof(double) * ne, cudaMemcpyDeviceToHost, s));
        TCK(cudaStreamSynchronize(s));
    }
    c.assembled = false;   // E now holds the final design's moduli
    return SGLD_OK;
}

// The projected loops: TopOpti_LocalVolumeConstraint.m:33-269 (porous infill)
// and TopOpti_GlobalVolumeConstraint.m:50-228 with MMA.  Every field operation
// runs on the device; the host runs the MMA dual iteration and the
// continuation schedule.  Buffers (full element grid): t_x design x, t_tmp
// xTilde, t_xp xPhys, t_hs filter weight sums, t_ce unit compliance, t_dvs
// dx = H'(xTilde), t_dcs / t_dc sensitivity before / after the density
// filter, t_q the PDE-filtered field, t_dv the constraint gradient.
extern "C" int sgld_topopt_projected(sgld_ctx *ctx, const sgld_topopt_projected_opts *opts, const double *F,
                                     double *xphys, sgld_topopt_iter *hist, int *n_iter) {
    if (!ctx || !opts || !F) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    Ctx &c = ctx->c;
    if (!c.have_fixed) return tfail(ctx, SGLD_ERR_STATE, "fixed DOFs not set (sgld_set_fixed_dofs)");
    sgld_topopt_projected_opts o = *opts;
    const bool local = o.constraint == SGLD_CONS_LOCAL;
    if (!local && o.constraint != SGLD_CONS_VOLUME)
        return tfail(ctx, SGLD_ERR_ARG, "constraint must be SGLD_CONS_LOCAL or SGLD_CONS_VOLUME");
    if (!local && !(o.volfrac > 0.0 && o.volfrac <= 1.0)) return tfail(ctx, SGLD_ERR_ARG, "volfrac in (0, 1]");
    if (o.rhat == 0) o.rhat = 8.0;
    if (o.alpha == 0) o.alpha = 0.5;
    if (o.pnorm == 0) o.pnorm = 16.0;
    if (o.move == 0) o.move = 0.1;
    if (o.min_change == 0) o.min_change = 1e-4;
    if (o.max_sharpness == 0) o.max_sharpness = 0.05;
    if (o.simp_penalty == 0) o.simp_penalty = 3.0;
    if (o.penalty == 0) o.penalty = 3.0;
    if (o.beta == 0) o.beta = 1.0;
    if (o.eta == 0) o.eta = 0.5;
    if (o.beta_max == 0) o.beta_max = 128.0;
    if (o.beta_interval == 0) o.beta_interval = 40;
    if (o.E0 == 0) o.E0 = 1.0;
    if (o.Emin == 0) o.Emin = 1e-6;
    if (o.n_loop < 1 || !(o.alpha > 0.0 && o.alpha <= 1.0) || !(o.pnorm >= 1.0) || !(o.rhat > 0.0))
        return tfail(ctx, SGLD_ERR_ARG, "n_loop >= 1, alpha in (0, 1], pnorm >= 1, rhat > 0 required");
    int rc = ensure_topo(ctx);
    if (rc) return rc;
    int r = 0;
    if ((rc = setup_filter(ctx, o.rmin, &r))) return rc;
    const Level &l0 = c.lv[0];
    const int64_t ne = (int64_t)c.h_elemap.size(), nn = (int64_t)c.h_nodemap.size();
    const size_t nv = 3 * (size_t)l0.nnode;
    const int nb = reduce_blocks(l0.nel);
    const double N = (double)ne;
    cudaStream_t s = c.stream;
    const double pde_tol = o.solve.tol > 0 ? o.solve.tol : 1e-6;
    const int pde_maxit = o.solve.maxit > 0 ? o.solve.maxit : 500;
    // design variables: the active elements that are not passive (:63)
    std::vector<int64_t> var;
    var.reserve(c.h_elemap.size());
    for (int64_t e : c.h_elemap)
        if (!std::binary_search(c.h_passive.begin(), c.h_passive.end(), e)) var.push_back(e);
    const int64_t nvar = (int64_t)var.size();
    if (nvar == 0) return tfail(ctx, SGLD_ERR_ARG, "no design variables (every element passive)");
    const int nbm = mma_blocks(nvar);
    int64_t *d_var = nullptr;
    double *mma_buf = nullptr;
    struct Free {
        void *a = nullptr, *b = nullptr;
        ~Free() {
            if (a) cudaFree(a);
            if (b) cudaFree(b);
        }
    } fr;
    TCK(cudaMalloc((void **)&d_var, sizeof(int64_t) * nvar));
    fr.a = d_var;
    TCK(cudaMemcpyAsync(d_var, var.data(), sizeof(int64_t) * nvar, cudaMemcpyHostToDevice, s));
    TCK(cudaMalloc((void **)&mma_buf, sizeof(double) * (6 * (size_t)nvar + 2 * (size_t)nbm + 2)));
    fr.b = mma_buf;
    double *xv = mma_buf, *xmin = xv + nvar, *xmax = xmin + nvar, *df0 = xmax + nvar, *dg = df0 + nvar,
           *xo = dg + nvar, *p1 = xo + nvar, *p2 = p1 + nbm, *sums = p2 + nbm;
    // loads, U = 0
    TCK(cudaMemsetAsync(c.d_b, 0, sizeof(double) * nv, s));
    TCK(cudaMemsetAsync(c.d_x, 0, sizeof(double) * nv, s));
    TCK(cudaMemcpyAsync(c.d_tmp, F, sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, s));
    launch_scatter_nodes(c.d_nodemap, nn, c.d_tmp, c.d_b, s);
    // x = alpha or volfrac (passive 1), xTilde = x, xPhys = H(xTilde)  (TopOpti_CallTopOpti.m:34-45)
    launch_fill_active(l0, c.t_x, local ? o.alpha : o.volfrac, nb, s);
    if (!c.h_passive.empty()) launch_set_passive_x(l0, c.t_x, nb, s);
    TCK(cudaMemcpyAsync(c.t_tmp, c.t_x, sizeof(double) * l0.nel, cudaMemcpyDeviceToDevice, s));
    double beta = o.beta, penalty = o.penalty;
    launch_heaviside(l0, c.t_tmp, beta, o.eta, c.t_xp, nullptr, nb, s);
    sgld_solve_opts so = o.solve;
    so.use_x0 = 1;
    so.history = nullptr;
    // :79-86 compliance of the fully solid domain
    launch_fill_active(l0, c.E, o.E0, nb, s);
    c.have_E = true;
    if ((rc = sgld_assemble(ctx))) return rc;
    sgld_solve_info si;
    if ((rc = solve_on_device(ctx, &so, &si))) return rc;
    int nbc = 0;
    launch_unit_compliance(l0, c.d_x, c.E, c.t_ce, c.d_part, &nbc, s);
    launch_finalize_sum(c.d_part, nbc, c.t_st + T_C, s);
    double c_solid = 0.0;
    TCK(cudaMemcpyAsync(&c_solid, c.t_st + T_C, sizeof(double), cudaMemcpyDeviceToHost, s));
    TCK(cudaStreamSynchronize(s));
    if (!(c_solid > 0.0)) return tfail(ctx, SGLD_ERR_NUMERIC, "compliance of the solid domain is not positive");
    // E = SIMP(xPhys) for the first iteration, with vol / sharpness sums
    launch_topo_modulus(l0, c.t_xp, o.simp_penalty, o.E0, o.Emin, c.E, c.d_part, c.d_part2, nb, s);
    launch_finalize_sum(c.d_part, nb, c.t_st + T_VOL, s);
    launch_finalize_sum(c.d_part2, nb, c.t_st + T_SHARP, s);
    cudaEvent_t ev[5];
    for (auto &e : ev) TCK(cudaEventCreate(&e));
    double change = 1.0, sharp = 1.0;
    int loop = 0, loopbeta = 0;
    while (loop < o.n_loop && change > o.min_change && sharp > o.max_sharpness) {   // :116
        ++loopbeta;
        ++loop;
        NvtxRange iter_range("projected SIMP iteration");
        double vol = 0.0;
        TCK(cudaMemcpyAsync(&vol, c.t_st + T_VOL, sizeof(double), cudaMemcpyDeviceToHost, s));
        TCK(cudaEventRecord(ev[0], s));
        if ((rc = sgld_assemble(ctx))) return rc;                                   // :123
        TCK(cudaEventRecord(ev[1], s));
        if ((rc = solve_on_device(ctx, &so, &si))) return rc;                       // :126
        TCK(cudaEventRecord(ev[2], s));
        launch_unit_compliance(l0, c.d_x, c.E, c.t_ce, c.d_part, &nbc, s);         // :128
        launch_finalize_sum(c.d_part, nbc, c.t_st + T_C, s);                        // :133-134
        // sensitivity of the normalised compliance through the projection (:136, :151-153)
        launch_heaviside(l0, c.t_tmp, beta, o.eta, nullptr, c.t_dvs, nb, s);
        launch_local_sens(l0, c.t_xp, c.t_ce, c.t_dvs, c.t_hs, penalty, o.E0, o.Emin, 1.0 / c_solid, c.t_dcs, nb, s);
        launch_density_filter(l0, c.t_dcs, r, c.t_fw, c.t_dc, s);
        TCK(cudaEventRecord(ev[3], s));
        double fval = 0.0, dg_scale = 1.0;
        if (local) {
            // local volume: x_hat = PDE(xPhys), its p-norm and gradient (Local...m:142-146, :162-169)
            int its_pde = 0;
            if ((rc = pde_filter_dev(ctx, o.rhat, c.t_xp, c.t_q, pde_tol, pde_maxit, &its_pde))) return rc;
            launch_pnorm(l0, c.t_q, o.pnorm, o.alpha, c.d_part, c.t_st + 12, N, c.t_dv, nb, s);
            if ((rc = pde_filter_dev(ctx, o.rhat, c.t_dv, c.t_q, pde_tol, pde_maxit, &its_pde))) return rc;
            launch_mul_div(l0, c.t_q, c.t_dvs, c.t_hs, c.t_dcs, nb, s);
            launch_density_filter(l0, c.t_dcs, r, c.t_fw, c.t_dv, s);
            double S = 0.0;
            TCK(cudaMemcpyAsync(&S, c.t_st + 12, sizeof(double), cudaMemcpyDeviceToHost, s));
            TCK(cudaStreamSynchronize(s));
            fval = pow(S / N, 1.0 / o.pnorm) - 1.0;                                 // Local...m:179
        } else {
            // volume: dv = filter(dx ./ Hs), dfdx = dv / (N V), fval = sum(xPhys) / (N V) - 1
            // (Global...m:119, :128-129, :139-141)
            launch_mul_div(l0, c.t_dvs, nullptr, c.t_hs, c.t_dcs, nb, s);
            launch_density_filter(l0, c.t_dcs, r, c.t_fw, c.t_dv, s);
            dg_scale = 1.0 / (N * o.volfrac);
            fval = vol / (N * o.volfrac) - 1.0;
        }
        // MMA (Local...m:180-192, Global...m:136-150)
        launch_mma_gather(d_var, nvar, c.t_x, c.t_dc, c.t_dv, o.move, dg_scale, xv, xmin, xmax, df0, dg, s);
        if ((rc = mma_solve_device(ctx, nvar, xv, xmin, xmax, df0, dg, fval, xo, p1, p2, sums, nullptr))) return rc;
        if (!c.h_passive.empty()) launch_set_passive_x(l0, c.t_x, nb, s);
        launch_mma_scatter(d_var, nvar, xo, xv, c.t_x, c.d_part, nbm, s);
        launch_max_partials(c.d_part, nbm, c.t_st + T_CHANGE, s);
        // xTilde = filter(x) / Hs, xPhys = H(xTilde), passive 1 (:197-204)
        launch_density_filter(l0, c.t_x, r, c.t_fw, c.t_q, s);
        launch_mul_div(l0, c.t_q, nullptr, c.t_hs, c.t_tmp, nb, s);
        launch_heaviside(l0, c.t_tmp, beta, o.eta, c.t_xp, nullptr, nb, s);
        TCK(cudaEventRecord(ev[4], s));
        launch_topo_modulus(l0, c.t_xp, o.simp_penalty, o.E0, o.Emin, c.E, c.d_part, c.d_part2, nb, s);   // :121, :205
        launch_finalize_sum(c.d_part, nb, c.t_st + T_VOL, s);
        launch_finalize_sum(c.d_part2, nb, c.t_st + T_SHARP, s);
        TCK(cudaGetLastError());
        double st[16];
        TCK(cudaMemcpyAsync(st, c.t_st, sizeof st, cudaMemcpyDeviceToHost, s));
        TCK(cudaStreamSynchronize(s));
        change = st[T_CHANGE];
        sharp = st[T_SHARP] / N;
        if (hist) {
            sgld_topopt_iter &h = hist[loop - 1];
            memset(&h, 0, sizeof h);
            h.loop = loop;
            h.cg_iterations = si.iterations;
            h.inner_iterations = si.inner_iterations;
            h.compliance = st[T_C];
            h.volume = vol / N;
            h.sharpness = sharp;
            h.change = change;
            h.constraint = fval;
            h.t_assemble = elapsed(ev[0], ev[1]) * 1e-3;
            h.t_solve = elapsed(ev[1], ev[2]) * 1e-3;
            h.t_opt = elapsed(ev[2], ev[3]) * 1e-3;
            h.t_filter = elapsed(ev[3], ev[4]) * 1e-3;
        }
        if (beta < o.beta_max && (loopbeta >= o.beta_interval || (!local && change <= 1e-3))) {   // Local :246, Global :212
            beta *= 2.0;
            loopbeta = 0;
            change = sharp = 1.0;
        }
        if (o.penalty_interval > 0 && loop % o.penalty_interval == 0)               // :256-261
            penalty = std::min(penalty + o.penalty_increment, 3.0);
    }
    for (auto &e : ev) cudaEventDestroy(e);
    if (n_iter) *n_iter = loop;
    if (xphys) {
        launch_gather_elems(c.d_elemap, ne, c.t_xp, c.d_tmp, s);
        TCK(cudaMemcpyAsync(xphys, c.d_tmp, sizeof(double) * ne, cudaMemcpyDeviceToHost, s));
        TCK(cudaStreamSynchronize(s));
    }
    c.assembled = false;
    return SGLD_OK;
}

extern "C" int sgld_topopt_displacement(sgld_ctx *ctx, double *U) {
    if (!ctx || !U) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    Ctx &c = ctx->c;
    const int64_t nn = (int64_t)c.h_nodemap.size();
    launch_gather_nodes(c.d_nodemap, nn, c.d_x, c.d_tmp, c.stream);
    TCK(cudaMemcpyAsync(U, c.d_tmp, sizeof(double) * 3 * nn, cudaMemcpyDeviceToHost, c.stream));
    TCK(cudaStreamSynchronize(c.stream));
    return SGLD_OK;
}
