// The learned warm start of the SIMP loop (sgld_topopt with learned = 1).  No
// counterpart in the reference: TopOpti_GlobalVolumeConstraint.m:57 calls
// Solving_CG_GMGS, which always starts from the previous displacement U_
// (Solving_CG_GMGS.m:7).  Here that start may be improved by a U-Net
// (sgld_net.cuh) trained online on the loop's own solves:
//
//   before solve k:  r0 = F - K U_{k-1}   (finest level, double-float K*u)
//                    features on level l: restricted r0, the injected last
//                    change U_{k-1} - U_{k-2}, a log-modulus field, the
//                    active-node mask (each vector scaled to unit RMS)
//                    v = P (net(features))  prolongated to the finest level,
//                    fixed DOFs zeroed
//                    alpha = v'r0 / v'Kv   (minimises the energy error of
//                    U_{k-1} + alpha v over alpha)
//                    start from U_{k-1} + alpha v iff it lowers the residual
//                    in the preconditioner's norm, r'Mr with M the FP64
//                    V-cycle (an SPD approximation of K^-1, so r'Mr tracks
//                    the energy norm of the error; the plain 2-norm of r is
//                    dominated by the high-frequency residual that any
//                    interpolated coarse correction leaves and would reject
//                    a guess that removes most of the error)
//   after solve k:   target = injected (U_k - U_{k-1}) at unit RMS; the
//                    sample (features, target) joins a ring of the last 4;
//                    a few Adam steps, most recent sample first.
//
// The solve itself is unchanged and runs to the same tolerance, so the
// converged displacement is the plain method's; the network can only change
// the iteration count.
#include <math.h>

#include <string>

#include "../../include/sgld_gpu.h"
#include "sgld_net.cuh"

namespace sgld {

constexpr int LW_RING = 4;

struct LearnedWS {
    Net net;
    bool net_ok = false, ready = false, have_prev = false;
    int level = 0, S = 1;                 // network level (0-based) and its cumulative span
    int cn[3] = {0, 0, 0}, fn[3] = {0, 0, 0}, fe3[3] = {0, 0, 0};   // coarse nodes, fine nodes, fine elements
    int64_t Vc = 0;
    double *d_uprev = nullptr, *d_prev = nullptr;   // finest level: U_{k-1}, U_{k-1} - U_{k-2}
    double *d_kd = nullptr, *d_r1 = nullptr;        // finest level: K d_prev, a trial residual
    double *d_dc = nullptr, *d_ec = nullptr;        // network level: injected vectors
    float *d_fe = nullptr;
    bf16 *x_cur = nullptr;                         // features of the pending solve
    bf16 *xs[LW_RING] = {};
    float *ts[LW_RING] = {}, *ms[LW_RING] = {};
    int nsamp = 0, head = 0;
    double *d_sc = nullptr;                        // device scalars read back by the host
    std::vector<void *> allocs;
};

namespace {

int lfail(sgld_ctx *ctx, int code, const std::string &m) {
    ctx->c.err = m;
    return code;
}

#define LCK(x)                                                                                  \
    do {                                                                                        \
        cudaError_t e_ = (x);                                                                   \
        if (e_ != cudaSuccess) return lfail(ctx, SGLD_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
cudaError_t lalloc(LearnedWS &w, T **p, int64_t n) {
    const cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (size_t)(n > 0 ? n : 1));
    if (e == cudaSuccess) w.allocs.push_back(*p);
    return e;
}

// sum a*b over n entries into d_sc[slot] (device), via the solver's partial-sum buffer
void dot_to(Ctx &c, const double *a, const double *b, int64_t n, double *out, cudaStream_t s) {
    const int nb = reduce_blocks(n);
    launch_dot(a, b, n, c.d_part, nb, s);
    launch_finalize_sum(c.d_part, nb, out, s);
}

}  // namespace

void learned_free(LearnedWS *w) {
    if (!w) return;
    if (w->net_ok) net_free(w->net);
    for (void *p : w->allocs) cudaFree(p);
    delete w;
}

// (Re)creates the warm-start state for the context's hierarchy; net_level is
// the MATLAB level index (0 = 3).
int learned_setup(sgld_ctx *ctx, LearnedWS **pw, int net_level, bool need_net) {
    Ctx &c = ctx->c;
    int lvl = (net_level > 0 ? net_level : 3) - 1;
    if (lvl > c.L - 1) lvl = c.L - 1;
    if (lvl < 0) lvl = 0;
    if (*pw && (*pw)->level == lvl && (*pw)->net_ok == need_net) return SGLD_OK;
    learned_free(*pw);
    *pw = nullptr;
    LearnedWS *w = new LearnedWS();
    w->level = lvl;
    w->S = 1;
    for (int i = 1; i <= lvl; ++i) w->S *= c.lv[i].span;
    const Level &l0 = c.lv[0], &ll = c.lv[lvl];
    w->cn[0] = ll.ny + 1;
    w->cn[1] = ll.nx + 1;
    w->cn[2] = ll.nz + 1;
    w->fn[0] = l0.ny + 1;
    w->fn[1] = l0.nx + 1;
    w->fn[2] = l0.nz + 1;
    w->fe3[0] = l0.ny;
    w->fe3[1] = l0.nx;
    w->fe3[2] = l0.nz;
    w->Vc = (int64_t)w->cn[0] * w->cn[1] * w->cn[2];
    const int64_t nv = 3 * l0.nnode;
    cudaError_t e = cudaSuccess;
#define LA(p, n) \
    if (e == cudaSuccess) e = lalloc(*w, p, n)
    LA(&w->d_uprev, nv);
    LA(&w->d_prev, nv);
    LA(&w->d_kd, nv);
    LA(&w->d_r1, nv);
    LA(&w->d_dc, 3 * w->Vc);
    LA(&w->d_ec, 3 * w->Vc);
    LA(&w->d_fe, w->Vc);
    LA(&w->x_cur, 8 * w->Vc);
    for (int i = 0; i < LW_RING; ++i) {
        LA(&w->xs[i], 8 * w->Vc);
        LA(&w->ts[i], 3 * w->Vc);
        LA(&w->ms[i], w->Vc);
    }
    LA(&w->d_sc, 8);
#undef LA
    if (e != cudaSuccess) {
        learned_free(w);
        return lfail(ctx, SGLD_ERR_NOMEM, std::string("learned warm start: ") + cudaGetErrorString(e));
    }
    if (!need_net) {
        *pw = w;
        return SGLD_OK;
    }
    std::string err;
    const int rc = net_init(w->net, w->cn[0], w->cn[1], w->cn[2], 8, 3, 4, nullptr, 0x5eedull, c.stream, err);
    if (rc) {
        learned_free(w);
        return lfail(ctx, rc, err);
    }
    w->net_ok = true;
    *pw = w;
    return SGLD_OK;
}

namespace {

// r'Mr (M = FP64 V-cycle) into d_sc[slot]
int mnorm_to(sgld_ctx *ctx, const double *r, double *out) {
    Ctx &c = ctx->c;
    int nb = 0;
    const int rc = vcycle_f64(ctx, r, c.d_z, c.d_part2, &nb);
    if (rc) return rc;
    launch_finalize_sum(c.d_part2, nb, out, c.stream);
    return SGLD_OK;
}

}  // namespace

// Before the solve: U_{k-1} is in c.d_x, F in c.d_b, the stencil assembled.
// mode 1: subspace {d, v} (previous change and the network's correction);
// mode 2: {d} only (the method without the network).  Fills the diagnostics;
// may replace c.d_x by the better start.
int learned_before_solve(sgld_ctx *ctx, LearnedWS *w, int mode, double E0, int *used, int *accepted,
                         double *ratio, double *ext_ratio) {
    NvtxRange range("learned start");
    Ctx &c = ctx->c;
    cudaStream_t s = c.stream;
    const Level &l0 = c.lv[0], &ll = c.lv[w->level];
    const int64_t nv = 3 * l0.nnode;
    *used = *accepted = 0;
    *ratio = *ext_ratio = 0.0;
    LCK(cudaMemcpyAsync(w->d_uprev, c.d_x, sizeof(double) * nv, cudaMemcpyDeviceToDevice, s));
    if (!w->have_prev) return SGLD_OK;
    // r0 = F - K U_{k-1} (fixed DOFs zero)
    launch_kbyu_df(l0, c.E, c.d_x, c.d_q, nullptr, nullptr, s);
    launch_residual(c.d_r, c.d_b, c.d_q, nv, s);
    launch_mask_fixed(l0, c.d_r, s);
    const bool with_net = mode == 1;
    if (with_net) {   // features on the network's level
        const double *rc = c.d_r;
        for (int i = 1; i <= w->level; ++i) {
            launch_restrict<double>(c.lv[i - 1], c.lv[i], rc, c.lv[i].r, s);
            rc = c.lv[i].r;
        }
        net_inject(w->d_prev, w->fn, w->S, w->cn, w->d_dc, s);
        net_logE(c.E, w->fe3, w->S, w->cn, E0, w->d_fe, s);
        dot_to(c, rc, rc, 3 * w->Vc, w->d_sc + 0, s);
        dot_to(c, w->d_dc, w->d_dc, 3 * w->Vc, w->d_sc + 1, s);
        double h[2];
        LCK(cudaMemcpyAsync(h, w->d_sc, sizeof h, cudaMemcpyDeviceToHost, s));
        LCK(cudaStreamSynchronize(s));
        const double nvc = 3.0 * (double)w->Vc;
        const double sr = h[0] > 0 ? 1.0 / sqrt(h[0] / nvc) : 0.0, sd = h[1] > 0 ? 1.0 / sqrt(h[1] / nvc) : 0.0;
        net_pack(rc, w->d_dc, w->d_fe, ll.nflag, w->Vc, sr, sd, w->x_cur, s);
    }
    const bool net_in = with_net && w->ready;
    if (net_in) {   // v = P net(features) in c.d_p, fixed DOFs zero; K v in c.d_q
        w->net.X.a = w->x_cur;
        net_forward(w->net);
        double *vl = (w->level == 0) ? c.d_p : c.lv[w->level].x;
        net_unpack(w->net.Y, ll.nflag, w->Vc, vl, s);
        LCK(cudaMemsetAsync(c.d_tmp, 0, sizeof(double) * nv, s));
        for (int i = w->level - 1; i >= 0; --i) {
            double *out = (i == 0) ? c.d_p : c.lv[i].x;
            launch_prolong_smooth<double>(c.lv[i], c.lv[i + 1], c.lv[i + 1].x, c.d_tmp, c.lv[i].idiag, 0.0, out,
                                          false, nullptr, nullptr, s);
        }
        launch_mask_fixed(l0, c.d_p, s);
        launch_kbyu_df(l0, c.E, c.d_p, c.d_q, nullptr, nullptr, s);
        *used = 1;
    }
    // Galerkin system of the subspace: H [a b]' = g, H = [d'Kd d'Kv; v'Kd v'Kv], g = [d'r0 v'r0]
    launch_kbyu_df(l0, c.E, w->d_prev, w->d_kd, nullptr, nullptr, s);
    dot_to(c, w->d_prev, c.d_r, nv, w->d_sc + 2, s);
    dot_to(c, w->d_prev, w->d_kd, nv, w->d_sc + 3, s);
    if (net_in) {
        dot_to(c, c.d_p, c.d_r, nv, w->d_sc + 4, s);
        dot_to(c, c.d_p, w->d_kd, nv, w->d_sc + 5, s);
        dot_to(c, c.d_p, c.d_q, nv, w->d_sc + 6, s);
    }
    double q[5] = {0, 0, 0, 0, 0};
    LCK(cudaMemcpyAsync(q, w->d_sc + 2, (net_in ? 5 : 2) * sizeof(double), cudaMemcpyDeviceToHost, s));
    LCK(cudaStreamSynchronize(s));
    if (net_in && net_take_error(w->net)) {
        w->ready = false;
        return lfail(ctx, SGLD_ERR_CUDA, "a tensor-core convolution's MMA wait gave up in the network's forward pass");
    }
    const double g1 = q[0], h11 = q[1], g2 = q[2], h12 = q[3], h22 = q[4];
    if (!(h11 > 0.0) || !isfinite(g1) || !isfinite(h11)) return SGLD_OK;
    // r'Mr of r0, of the extrapolation alone, and of the subspace step
    int rc;
    if ((rc = mnorm_to(ctx, c.d_r, w->d_sc + 0))) return rc;
    const double ae = g1 / h11;
    LCK(cudaMemcpyAsync(w->d_r1, c.d_r, sizeof(double) * nv, cudaMemcpyDeviceToDevice, s));
    net_axpby(w->d_r1, w->d_kd, -ae, 1.0, nv, s);
    if ((rc = mnorm_to(ctx, w->d_r1, w->d_sc + 1))) return rc;
    double a = ae, b = 0.0;
    const double det = h11 * h22 - h12 * h12;
    const bool two = net_in && h22 > 0.0 && isfinite(g2) && isfinite(h22) && det > 1e-12 * h11 * h22;
    if (two) {
        a = (h22 * g1 - h12 * g2) / det;
        b = (h11 * g2 - h12 * g1) / det;
        LCK(cudaMemcpyAsync(w->d_r1, c.d_r, sizeof(double) * nv, cudaMemcpyDeviceToDevice, s));
        net_axpby(w->d_r1, w->d_kd, -a, 1.0, nv, s);
        net_axpby(w->d_r1, c.d_q, -b, 1.0, nv, s);
        if ((rc = mnorm_to(ctx, w->d_r1, w->d_sc + 7))) return rc;
    }
    double m[8];
    LCK(cudaMemcpyAsync(m, w->d_sc, sizeof m, cudaMemcpyDeviceToHost, s));
    LCK(cudaStreamSynchronize(s));
    if (!(m[0] > 0.0)) return SGLD_OK;
    *ext_ratio = sqrt(fmax(m[1], 0.0) / m[0]);
    *ratio = two ? sqrt(fmax(m[7], 0.0) / m[0]) : *ext_ratio;
    if (!(*ratio < 1.0)) return SGLD_OK;
    net_axpby(c.d_x, w->d_prev, a, 1.0, nv, s);
    if (two) net_axpby(c.d_x, c.d_p, b, 1.0, nv, s);
    *accepted = 1;
    return SGLD_OK;
}

// After the solve: U_k in c.d_x.  Stores the change, trains on the sample.
int learned_after_solve(sgld_ctx *ctx, LearnedWS *w, int mode, int steps, float lr, double *loss) {
    Ctx &c = ctx->c;
    cudaStream_t s = c.stream;
    const Level &l0 = c.lv[0], &ll = c.lv[w->level];
    const int64_t nv = 3 * l0.nnode;
    *loss = 0.0;
    NvtxRange range("learned training");
    const bool had_features = w->have_prev;
    // d_prev = U_k - U_{k-1}
    LCK(cudaMemcpyAsync(w->d_prev, c.d_x, sizeof(double) * nv, cudaMemcpyDeviceToDevice, s));
    net_axpby(w->d_prev, w->d_uprev, -1.0, 1.0, nv, s);
    w->have_prev = true;
    if (!had_features || mode != 1) return SGLD_OK;   // no features for this solve
    net_inject(w->d_prev, w->fn, w->S, w->cn, w->d_ec, s);
    dot_to(c, w->d_ec, w->d_ec, 3 * w->Vc, w->d_sc + 6, s);
    double e2 = 0.0;
    LCK(cudaMemcpyAsync(&e2, w->d_sc + 6, sizeof(double), cudaMemcpyDeviceToHost, s));
    LCK(cudaStreamSynchronize(s));
    if (!(e2 > 0.0)) return SGLD_OK;
    const double se = 1.0 / sqrt(e2 / (3.0 * (double)w->Vc));
    const int slot = w->head;
    LCK(cudaMemcpyAsync(w->xs[slot], w->x_cur, sizeof(bf16) * 8 * w->Vc, cudaMemcpyDeviceToDevice, s));
    net_target(w->d_ec, ll.nflag, w->Vc, se, w->ts[slot], w->ms[slot], s);
    w->head = (w->head + 1) % LW_RING;
    if (w->nsamp < LW_RING) ++w->nsamp;
    for (int k = 0; k < steps; ++k) {
        const int i = (slot - (k % w->nsamp) + LW_RING) % LW_RING;
        w->net.X.a = w->xs[i];
        net_forward(w->net);
        net_loss(w->net, w->ts[i], w->ms[i]);
        net_backward(w->net);
        net_adam_step(w->net, lr);
    }
    w->ready = true;
    LCK(cudaGetLastError());
    LCK(cudaMemcpyAsync(loss, w->net.d_loss, sizeof(double), cudaMemcpyDeviceToHost, s));
    LCK(cudaStreamSynchronize(s));
    if (net_take_error(w->net)) {
        w->ready = false;
        return lfail(ctx, SGLD_ERR_CUDA, "a tensor-core convolution's MMA wait gave up while training the network");
    }
    return SGLD_OK;
}

}  // namespace sgld
