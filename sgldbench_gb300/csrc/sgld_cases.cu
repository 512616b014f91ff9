// Learned start for a sequence of load cases on one model (sgld_cases_*).  No
// counterpart in the reference: its solves start from the previous
// displacement U_ (src/Solving_CG_GMGS.m:7), which is zero for a new load
// case, and its multi-load exploration solves every case from scratch
// (GUIs/Mtd_StructuralRobustnessExploration.m:119).
//
// The object learns from the solves it is given for training:
//   * a basis W of the training solutions, K-orthonormal (W_i' K W_j = d_ij,
//     classical Gram-Schmidt applied twice, K by the double-float K*u), stored
//     in FP64 in the compact DOF order;
//   * a U-Net (sgld_net.cuh) on a coarse multigrid level, trained on the
//     training solves' own pairs: features of the residual that the basis
//     start leaves, r0 = F - K x_b, with the basis start x_b, the log-modulus
//     and the active-node mask -> the correction U - x_b the solve then found.
// For a new load F the start is
//   x_b = sum_i (W_i' F) W_i       the energy-optimal start in span(W), and
//   x   = x_b + beta P net(.)      beta = v'r0 / v'Kv for v = P net(.),
// kept only if it lowers r'Mr (M = the FP32 V-cycle, an SPD approximation of
// K^-1, so r'Mr tracks the energy norm of the error; the start's residual and
// the correction's energy come from the FP32 K*u, since they only choose
// between two starts).  The solve then runs to
// its tolerance on the true residual as any other, so the start changes the
// iteration count and never the converged answer.
#include <math.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/sgld_gpu.h"
#include "sgld_net.cuh"

namespace sgld {
int basis_max();
int basis_partials(int64_t nd);
void launch_basis_dots(const double *W, int k, int64_t nd, const double *v, const int64_t *map, double *part,
                       double scale, double *out, cudaStream_t s);
void launch_basis_combine(const double *W, int k, int64_t nd, const double *coef, double alpha, double beta,
                          double *x, const int64_t *map, cudaStream_t s);
void launch_basis_store(const double *w, const int64_t *map, int64_t nd, double scale, double *Wk, cudaStream_t s);
}  // namespace sgld

using namespace sgld;

struct sgld_cases {
    sgld_ctx *ctx = nullptr;
    int kmax = 0, k = 0;
    int64_t nd = 0;                       // compact DOFs
    double *W = nullptr;                  // [kmax][nd] K-orthonormal basis, compact order
    double *d_coef = nullptr;             // [2 * CB_MAXK] projection coefficients
    double *d_bpart = nullptr;            // basis dot partials
    double *d_xb = nullptr, *d_r0 = nullptr, *d_w = nullptr, *d_kw = nullptr;   // full-grid FP64
    double *d_sc = nullptr;               // [16] device scalars read back
    // network
    Net net;
    bool net_ok = false, ready = false;
    int level = 0, S = 1, cn[3] = {0, 0, 0}, fn[3] = {0, 0, 0}, fe3[3] = {0, 0, 0};
    int64_t Vc = 0;
    double *d_dc = nullptr, *d_ec = nullptr;
    float *d_fe = nullptr;
    bf16 *x_cur = nullptr;
    bool have_features = false;
    std::vector<bf16 *> xs;
    std::vector<float *> ts, ms;
    int nsamp = 0, head = 0;
    int train_steps = 8;
    float lr = 1e-3f;
    std::vector<void *> allocs;
};

namespace {

int cfail(sgld_ctx *ctx, int code, const std::string &m) {
    ctx->c.err = m;
    return code;
}

#define CCK(x)                                                                                           \
    do {                                                                                                 \
        cudaError_t e_ = (x);                                                                            \
        if (e_ != cudaSuccess) return cfail(ctx, SGLD_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
cudaError_t calloc_dev(sgld_cases *cs, T **p, int64_t n) {
    const cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (size_t)(n > 0 ? n : 1));
    if (e == cudaSuccess) cs->allocs.push_back(*p);
    return e;
}

void free_cases(sgld_cases *cs) {
    if (!cs) return;
    if (cs->net_ok) net_free(cs->net);
    for (void *p : cs->allocs) cudaFree(p);
    delete cs;
}

void dot_into(Ctx &c, const double *a, const double *b, int64_t n, double *out, cudaStream_t s) {
    const int nb = reduce_blocks(n);
    launch_dot(a, b, n, c.d_part, nb, s);
    launch_finalize_sum(c.d_part, nb, out, s);
}

// r'Mr (M = FP64 V-cycle) into *out (device)
int mnorm_into(sgld_ctx *ctx, const double *r, double *out) {
    Ctx &c = ctx->c;
    int nb = 0;
    const int rc = vcycle_f64(ctx, r, c.d_z, c.d_part2, &nb);
    if (rc) return rc;
    launch_finalize_sum(c.d_part2, nb, out, c.stream);
    return SGLD_OK;
}

// The choice between two starts only compares r'Mr values, so it runs on the FP32
// operators (the solve itself forms its true residual with the double-float K*u):
// r'Mr with the FP32 V-cycle, r narrowed to FP32, into *out (device)
int mnorm32_into(sgld_ctx *ctx, const double *r, double *out) {
    Ctx &c = ctx->c;
    launch_narrow(r, c.d_r32, 3 * c.lv[0].nnode, c.stream);
    int nb = 0;
    const int rc = vcycle_f32(ctx, c.d_r32, c.d_z32, c.d_part2, &nb);
    if (rc) return rc;
    launch_finalize_sum(c.d_part2, nb, out, c.stream);
    return SGLD_OK;
}

// y = K x with the FP32 operator (x narrowed, the product widened); 0 or a CUDA error
int kbyu32_into(Ctx &c, const double *x, double *y, cudaStream_t s) {
    const Level &l0 = c.lv[0];
    const int64_t nv = 3 * l0.nnode;
    launch_narrow(x, c.d_r32, nv, s);
    if (int e = launch_kbyu_f32(l0, c.d_E32, c.d_r32, c.d_t32, nullptr, nullptr, s)) return e;
    launch_widen(c.d_t32, y, nv, s);
    return 0;
}

// the network's level: the finest one with at most 110K nodes (MATLAB level
// index net_level when given)
int pick_level(const Ctx &c, int net_level) {
    if (net_level > 0) return std::min(std::max(net_level - 1, 0), c.L - 1);
    for (int l = 0; l < c.L; ++l)
        if (c.lv[l].nnode <= 110000) return l;
    return c.L - 1;
}

// x_b = sum_i (W_i' b) W_i into c.d_x (zero when the basis is empty)
void basis_start(sgld_cases *cs, cudaStream_t s) {
    Ctx &c = cs->ctx->c;
    const int64_t nv = 3 * c.lv[0].nnode;
    cudaMemsetAsync(c.d_x, 0, sizeof(double) * nv, s);
    if (cs->k == 0) return;
    launch_basis_dots(cs->W, cs->k, cs->nd, c.d_b, c.d_nodemap, cs->d_bpart, 1.0, cs->d_coef, s);
    launch_basis_combine(cs->W, cs->k, cs->nd, cs->d_coef, 1.0, 0.0, c.d_x, c.d_nodemap, s);
}

// Adds the solution in c.d_x to the basis (classical Gram-Schmidt, twice, in
// the K inner product).  A solution already in the span (relative K-norm of
// the remainder below 1e-6) is not added.
int basis_add(sgld_cases *cs) {
    sgld_ctx *ctx = cs->ctx;
    Ctx &c = ctx->c;
    cudaStream_t s = c.stream;
    const Level &l0 = c.lv[0];
    const int64_t nv = 3 * l0.nnode;
    if (cs->k >= cs->kmax) return SGLD_OK;
    CCK(cudaMemcpyAsync(cs->d_w, c.d_x, sizeof(double) * nv, cudaMemcpyDeviceToDevice, s));
    launch_kbyu_df(l0, c.E, cs->d_w, cs->d_kw, nullptr, nullptr, s);
    dot_into(c, cs->d_w, cs->d_kw, nv, cs->d_sc + 8, s);   // |U|_K^2
    for (int pass = 0; pass < 2 && cs->k > 0; ++pass) {
        if (pass) launch_kbyu_df(l0, c.E, cs->d_w, cs->d_kw, nullptr, nullptr, s);
        launch_basis_dots(cs->W, cs->k, cs->nd, cs->d_kw, c.d_nodemap, cs->d_bpart, 1.0, cs->d_coef, s);
        launch_basis_combine(cs->W, cs->k, cs->nd, cs->d_coef, -1.0, 1.0, cs->d_w, c.d_nodemap, s);
    }
    launch_kbyu_df(l0, c.E, cs->d_w, cs->d_kw, nullptr, nullptr, s);
    dot_into(c, cs->d_w, cs->d_kw, nv, cs->d_sc + 9, s);   // |w|_K^2
    double h[2];
    CCK(cudaMemcpyAsync(h, cs->d_sc + 8, sizeof h, cudaMemcpyDeviceToHost, s));
    CCK(cudaStreamSynchronize(s));
    if (!(h[0] > 0.0) || !(h[1] > 1e-12 * h[0]) || !isfinite(h[1])) return SGLD_OK;
    launch_basis_store(cs->d_w, c.d_nodemap, cs->nd, 1.0 / sqrt(h[1]), cs->W + (int64_t)cs->k * cs->nd, s);
    ++cs->k;
    CCK(cudaGetLastError());
    return SGLD_OK;
}

// Features of the pending solve (restricted r0, injected x_b, log-modulus,
// mask) into cs->x_cur.  r0 must be in cs->d_r0 and x_b in cs->d_xb.
int make_features(sgld_cases *cs) {
    sgld_ctx *ctx = cs->ctx;
    Ctx &c = ctx->c;
    cudaStream_t s = c.stream;
    const Level &ll = c.lv[cs->level];
    const double *rc = cs->d_r0;
    for (int i = 1; i <= cs->level; ++i) {
        launch_restrict<double>(c.lv[i - 1], c.lv[i], rc, c.lv[i].r, s);
        rc = c.lv[i].r;
    }
    net_inject(cs->d_xb, cs->fn, cs->S, cs->cn, cs->d_dc, s);
    net_logE(c.E, cs->fe3, cs->S, cs->cn, 1.0, cs->d_fe, s);
    dot_into(c, rc, rc, 3 * cs->Vc, cs->d_sc + 10, s);
    dot_into(c, cs->d_dc, cs->d_dc, 3 * cs->Vc, cs->d_sc + 11, s);
    double h[2];
    CCK(cudaMemcpyAsync(h, cs->d_sc + 10, sizeof h, cudaMemcpyDeviceToHost, s));
    CCK(cudaStreamSynchronize(s));
    const double nvc = 3.0 * (double)cs->Vc;
    const double sr = h[0] > 0 ? 1.0 / sqrt(h[0] / nvc) : 0.0, sd = h[1] > 0 ? 1.0 / sqrt(h[1] / nvc) : 0.0;
    net_pack(rc, cs->d_dc, cs->d_fe, ll.nflag, cs->Vc, sr, sd, cs->x_cur, s);
    cs->have_features = true;
    return SGLD_OK;
}

// x += beta v, v = P net(features), if that lowers r'Mr.  r0 in cs->d_r0.
int net_correction(sgld_cases *cs, sgld_cases_stats *st) {
    sgld_ctx *ctx = cs->ctx;
    Ctx &c = ctx->c;
    cudaStream_t s = c.stream;
    const Level &l0 = c.lv[0], &ll = c.lv[cs->level];
    const int64_t nv = 3 * l0.nnode;
    cs->net.X.a = cs->x_cur;
    net_forward(cs->net);
    double *vl = (cs->level == 0) ? c.d_p : c.lv[cs->level].x;
    net_unpack(cs->net.Y, ll.nflag, cs->Vc, vl, s);
    CCK(cudaMemsetAsync(c.d_tmp, 0, sizeof(double) * nv, s));
    for (int i = cs->level - 1; i >= 0; --i) {
        double *out = (i == 0) ? c.d_p : c.lv[i].x;
        launch_prolong_smooth<double>(c.lv[i], c.lv[i + 1], c.lv[i + 1].x, c.d_tmp, c.lv[i].idiag, 0.0, out, false,
                                      nullptr, nullptr, s);
    }
    launch_mask_fixed(l0, c.d_p, s);
    if (kbyu32_into(c, c.d_p, c.d_q, s)) return cfail(ctx, SGLD_ERR_CUDA, "FP32 K*u of the network's correction");
    dot_into(c, c.d_p, cs->d_r0, nv, cs->d_sc + 0, s);
    dot_into(c, c.d_p, c.d_q, nv, cs->d_sc + 1, s);
    double h[2];
    CCK(cudaMemcpyAsync(h, cs->d_sc, sizeof h, cudaMemcpyDeviceToHost, s));
    CCK(cudaStreamSynchronize(s));
    if (net_take_error(cs->net)) {
        cs->ready = false;
        return cfail(ctx, SGLD_ERR_CUDA, "a tensor-core convolution's MMA wait gave up in the network's forward pass");
    }
    if (!(h[1] > 0.0) || !isfinite(h[0]) || !isfinite(h[1])) return SGLD_OK;
    const double beta = h[0] / h[1];
    int rc;
    if ((rc = mnorm32_into(ctx, cs->d_r0, cs->d_sc + 2))) return rc;
    CCK(cudaMemcpyAsync(cs->d_w, cs->d_r0, sizeof(double) * nv, cudaMemcpyDeviceToDevice, s));
    net_axpby(cs->d_w, c.d_q, -beta, 1.0, nv, s);
    if ((rc = mnorm32_into(ctx, cs->d_w, cs->d_sc + 3))) return rc;
    double m[2];
    CCK(cudaMemcpyAsync(m, cs->d_sc + 2, sizeof m, cudaMemcpyDeviceToHost, s));
    CCK(cudaStreamSynchronize(s));
    st->net_used = 1;
    if (!(m[0] > 0.0) || !(m[1] < m[0])) return SGLD_OK;
    net_axpby(c.d_x, c.d_p, beta, 1.0, nv, s);
    st->net_accepted = 1;
    st->net_ratio = sqrt(fmax(m[1], 0.0) / m[0]);
    return SGLD_OK;
}

// one (features, correction U - x_b) sample and `steps` Adam steps
int net_train(sgld_cases *cs, int steps, float lr, sgld_cases_stats *st) {
    sgld_ctx *ctx = cs->ctx;
    Ctx &c = ctx->c;
    cudaStream_t s = c.stream;
    const Level &ll = c.lv[cs->level];
    const int64_t nv = 3 * c.lv[0].nnode;
    // correction U - x_b (c.d_x holds U)
    CCK(cudaMemcpyAsync(cs->d_w, c.d_x, sizeof(double) * nv, cudaMemcpyDeviceToDevice, s));
    net_axpby(cs->d_w, cs->d_xb, -1.0, 1.0, nv, s);
    net_inject(cs->d_w, cs->fn, cs->S, cs->cn, cs->d_ec, s);
    dot_into(c, cs->d_ec, cs->d_ec, 3 * cs->Vc, cs->d_sc + 12, s);
    double e2 = 0.0;
    CCK(cudaMemcpyAsync(&e2, cs->d_sc + 12, sizeof(double), cudaMemcpyDeviceToHost, s));
    CCK(cudaStreamSynchronize(s));
    if (!(e2 > 0.0) || !isfinite(e2)) return SGLD_OK;
    const double se = 1.0 / sqrt(e2 / (3.0 * (double)cs->Vc));
    const int slot = cs->head, ring = (int)cs->xs.size();
    CCK(cudaMemcpyAsync(cs->xs[slot], cs->x_cur, sizeof(bf16) * 8 * cs->Vc, cudaMemcpyDeviceToDevice, s));
    net_target(cs->d_ec, ll.nflag, cs->Vc, se, cs->ts[slot], cs->ms[slot], s);
    cs->head = (cs->head + 1) % ring;
    if (cs->nsamp < ring) ++cs->nsamp;
    // the new sample's loss before training (the network as it stood for this case)
    cs->net.X.a = cs->xs[slot];
    net_forward(cs->net);
    net_loss(cs->net, cs->ts[slot], cs->ms[slot]);
    CCK(cudaMemcpyAsync(&st->net_loss_before, cs->net.d_loss, sizeof(double), cudaMemcpyDeviceToHost, s));
    // most recent sample first, then back through the ring
    for (int k = 0; k < steps; ++k) {
        const int i = (slot - (k % cs->nsamp) + ring) % ring;
        cs->net.X.a = cs->xs[i];
        net_forward(cs->net);
        net_loss(cs->net, cs->ts[i], cs->ms[i]);
        net_backward(cs->net);
        net_adam_step(cs->net, lr);
    }
    cs->ready = true;
    // and after
    cs->net.X.a = cs->xs[slot];
    net_forward(cs->net);
    net_loss(cs->net, cs->ts[slot], cs->ms[slot]);
    CCK(cudaGetLastError());
    CCK(cudaMemcpyAsync(&st->net_loss, cs->net.d_loss, sizeof(double), cudaMemcpyDeviceToHost, s));
    CCK(cudaStreamSynchronize(s));
    if (net_take_error(cs->net)) {
        cs->ready = false;
        return cfail(ctx, SGLD_ERR_CUDA, "a tensor-core convolution's MMA wait gave up while training the network");
    }
    return SGLD_OK;
}

float elapsed_s(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms * 1e-3f;
}

// the whole call on the context's full-grid vectors: F in c.d_b, U to c.d_x
int cases_run(sgld_cases *cs, const sgld_solve_opts *o, int mode, int train, sgld_solve_info *info,
              sgld_cases_stats *st) {
    sgld_ctx *ctx = cs->ctx;
    Ctx &c = ctx->c;
    cudaStream_t s = c.stream;
    const Level &l0 = c.lv[0];
    const int64_t nv = 3 * l0.nnode;
    cudaEvent_t ev[4];
    for (auto &e : ev) CCK(cudaEventCreate(&e));
    struct Guard {
        cudaEvent_t *e;
        ~Guard() {
            for (int i = 0; i < 4; ++i) cudaEventDestroy(e[i]);
        }
    } guard{ev};
    st->basis = cs->k;
    CCK(cudaEventRecord(ev[0], s));
    // the start
    if (mode >= 1) basis_start(cs, s);
    else CCK(cudaMemsetAsync(c.d_x, 0, sizeof(double) * nv, s));
    const bool want_net = mode == 2 && cs->net_ok;
    if (want_net || st->diagnostics) {
        // r0 = F - K x_b for the network's features and the choice of start (FP32 K*u)
        CCK(cudaMemcpyAsync(cs->d_xb, c.d_x, sizeof(double) * nv, cudaMemcpyDeviceToDevice, s));
        if (kbyu32_into(c, c.d_x, c.d_q, s)) return cfail(ctx, SGLD_ERR_CUDA, "FP32 K*u of the basis start");
        launch_residual(cs->d_r0, c.d_b, c.d_q, nv, s);
        launch_mask_fixed(l0, cs->d_r0, s);
    }
    int rc;
    cs->have_features = false;
    if (want_net) {
        if ((rc = make_features(cs))) return rc;
        if (cs->ready && (rc = net_correction(cs, st))) return rc;
    }
    if (st->diagnostics) {   // sqrt(r'Mr) of the basis start and of the chosen start, relative to x = 0
        if ((rc = mnorm_into(ctx, c.d_b, cs->d_sc + 4))) return rc;
        if ((rc = mnorm_into(ctx, cs->d_r0, cs->d_sc + 5))) return rc;
        double m[2];
        CCK(cudaMemcpyAsync(m, cs->d_sc + 4, sizeof m, cudaMemcpyDeviceToHost, s));
        CCK(cudaStreamSynchronize(s));
        st->basis_ratio = m[0] > 0.0 ? sqrt(fmax(m[1], 0.0) / m[0]) : 0.0;
        st->start_ratio = st->net_accepted ? st->basis_ratio * st->net_ratio : st->basis_ratio;
    }
    CCK(cudaEventRecord(ev[1], s));
    // the solve, from the start unless it is zero
    sgld_solve_opts o2 = *o;
    o2.use_x0 = (mode >= 1 && cs->k > 0) || st->net_accepted;
    if ((rc = solve_on_device(ctx, &o2, info))) return rc;
    CCK(cudaEventRecord(ev[2], s));
    if (train) {
        if (want_net && cs->have_features && (rc = net_train(cs, cs->train_steps, cs->lr, st)))
            return rc;
        if ((rc = basis_add(cs))) return rc;
    }
    CCK(cudaEventRecord(ev[3], s));
    CCK(cudaEventSynchronize(ev[3]));
    st->t_start = elapsed_s(ev[0], ev[1]);
    st->t_solve = elapsed_s(ev[1], ev[2]);
    st->t_train = elapsed_s(ev[2], ev[3]);
    return SGLD_OK;
}

}  // namespace

extern "C" {

int sgld_cases_create(sgld_ctx *ctx, int max_basis, int net_level, int train_steps, sgld_cases **out) {
    if (!ctx || !out) return SGLD_ERR_ARG;
    *out = nullptr;
    if (int rc = bind_ctx(ctx)) return rc;
    Ctx &c = ctx->c;
    if (max_basis < 0 || max_basis > basis_max())
        return cfail(ctx, SGLD_ERR_ARG, "max_basis must be in [0, " + std::to_string(basis_max()) + "]");
    if (train_steps < 0) return cfail(ctx, SGLD_ERR_ARG, "train_steps must be >= 0");
    sgld_cases *cs = new sgld_cases();
    cs->ctx = ctx;
    cs->kmax = max_basis;
    cs->nd = 3 * (int64_t)c.h_nodemap.size();
    cs->train_steps = train_steps;
    const int64_t nv = 3 * c.lv[0].nnode;
    cudaError_t e = cudaSuccess;
#define CA(p, n) \
    if (e == cudaSuccess) e = calloc_dev(cs, p, n)
    CA(&cs->W, (int64_t)max_basis * cs->nd);
    CA(&cs->d_coef, 2 * basis_max());
    CA(&cs->d_bpart, (int64_t)basis_max() * basis_partials(cs->nd));
    CA(&cs->d_xb, nv);
    CA(&cs->d_r0, nv);
    CA(&cs->d_w, nv);
    CA(&cs->d_kw, nv);
    CA(&cs->d_sc, 16);
    if (net_level >= 0) {
        cs->level = pick_level(c, net_level);
        cs->S = 1;
        for (int i = 1; i <= cs->level; ++i) cs->S *= c.lv[i].span;
        const Level &l0 = c.lv[0], &ll = c.lv[cs->level];
        cs->cn[0] = ll.ny + 1;
        cs->cn[1] = ll.nx + 1;
        cs->cn[2] = ll.nz + 1;
        cs->fn[0] = l0.ny + 1;
        cs->fn[1] = l0.nx + 1;
        cs->fn[2] = l0.nz + 1;
        cs->fe3[0] = l0.ny;
        cs->fe3[1] = l0.nx;
        cs->fe3[2] = l0.nz;
        cs->Vc = (int64_t)cs->cn[0] * cs->cn[1] * cs->cn[2];
        CA(&cs->d_dc, 3 * cs->Vc);
        CA(&cs->d_ec, 3 * cs->Vc);
        CA(&cs->d_fe, cs->Vc);
        CA(&cs->x_cur, 8 * cs->Vc);
        const int ring = std::max(max_basis, 1);
        cs->xs.assign(ring, nullptr);
        cs->ts.assign(ring, nullptr);
        cs->ms.assign(ring, nullptr);
        for (int i = 0; i < ring; ++i) {
            CA(&cs->xs[i], 8 * cs->Vc);
            CA(&cs->ts[i], 3 * cs->Vc);
            CA(&cs->ms[i], cs->Vc);
        }
    }
#undef CA
    if (e != cudaSuccess) {
        free_cases(cs);
        return cfail(ctx, SGLD_ERR_NOMEM, std::string("load-case start: ") + cudaGetErrorString(e));
    }
    if (net_level >= 0) {
        std::string err;
        const int rc = net_init(cs->net, cs->cn[0], cs->cn[1], cs->cn[2], 8, 3, 4, nullptr, 0xca5e5ull, c.stream, err);
        if (rc) {
            free_cases(cs);
            return cfail(ctx, rc, err);
        }
        cs->net_ok = true;
    }
    *out = cs;
    return SGLD_OK;
}

void sgld_cases_destroy(sgld_cases *cs) {
    if (!cs) return;
    if (cs->ctx) bind_ctx(cs->ctx);
    free_cases(cs);
}

int sgld_cases_basis_size(const sgld_cases *cs) { return cs ? cs->k : -1; }

static int cases_check(sgld_cases *cs, const void *F, const void *U, const sgld_solve_opts *o, int mode,
                       sgld_cases_stats *st) {
    if (!cs || !cs->ctx) return SGLD_ERR_ARG;
    sgld_ctx *ctx = cs->ctx;
    if (int rc = bind_ctx(ctx)) return rc;
    Ctx &c = ctx->c;
    if (!F || !U || !o || !st) return cfail(ctx, SGLD_ERR_ARG, "null argument");
    if (mode < 0 || mode > 2) return cfail(ctx, SGLD_ERR_ARG, "mode must be 0, 1 or 2");
    if (!c.assembled) return cfail(ctx, SGLD_ERR_STATE, "stencil not assembled (sgld_assemble)");
    const int diag = st->diagnostics;
    memset(st, 0, sizeof *st);
    st->diagnostics = diag;
    return SGLD_OK;
}

int sgld_cases_solve(sgld_cases *cs, const double *F, double *U, const sgld_solve_opts *o, int mode, int train,
                     sgld_solve_info *info, sgld_cases_stats *st) {
    int rc = cases_check(cs, F, U, o, mode, st);
    if (rc) return rc;
    sgld_ctx *ctx = cs->ctx;
    Ctx &c = ctx->c;
    const int64_t n = (int64_t)c.h_nodemap.size();
    sgld_solve_info local;
    if (!info) info = &local;
    CCK(cudaMemsetAsync(c.d_b, 0, sizeof(double) * 3 * c.lv[0].nnode, c.stream));
    CCK(cudaMemcpyAsync(c.d_tmp, F, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c.stream));
    launch_scatter_nodes(c.d_nodemap, n, c.d_tmp, c.d_b, c.stream);
    if ((rc = cases_run(cs, o, mode, train, info, st))) return rc;
    launch_gather_nodes(c.d_nodemap, n, c.d_x, c.d_tmp, c.stream);
    CCK(cudaMemcpyAsync(U, c.d_tmp, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c.stream));
    CCK(cudaStreamSynchronize(c.stream));
    return SGLD_OK;
}

int sgld_cases_solve_device(sgld_cases *cs, const double *d_F, double *d_U, const sgld_solve_opts *o, int mode,
                            int train, sgld_solve_info *info, sgld_cases_stats *st) {
    int rc = cases_check(cs, d_F, d_U, o, mode, st);
    if (rc) return rc;
    sgld_ctx *ctx = cs->ctx;
    Ctx &c = ctx->c;
    const int64_t n = (int64_t)c.h_nodemap.size();
    sgld_solve_info local;
    if (!info) info = &local;
    CCK(cudaMemsetAsync(c.d_b, 0, sizeof(double) * 3 * c.lv[0].nnode, c.stream));
    launch_scatter_nodes(c.d_nodemap, n, d_F, c.d_b, c.stream);
    if ((rc = cases_run(cs, o, mode, train, info, st))) return rc;
    launch_gather_nodes(c.d_nodemap, n, c.d_x, d_U, c.stream);
    CCK(cudaStreamSynchronize(c.stream));
    return SGLD_OK;
}

}  // extern "C"
