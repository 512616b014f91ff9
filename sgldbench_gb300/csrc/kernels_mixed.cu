// Kernels of the mixed-precision solve (SGLD_PREC_MIXED).
//
// The outer loop is the reference's PCG in FP64 made flexible (Polak-Ribiere
// beta = -lambda z_new'q / z'r), so that the preconditioner may change from
// one application to the next.  The preconditioner is a fixed number of FP32
// CG iterations on K e = r, each preconditioned by the reference's additive
// V-cycle in FP32.  The inner loop runs entirely on the device (scalars in
// device memory) and is captured once into a CUDA graph.
#include "sgld_internal.cuh"

namespace sgld {

constexpr int MB = 256;

__device__ __forceinline__ double mblock_reduce(double v) {
    __shared__ double red[MB / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < MB / 32; ++i) s += red[i];
    return s;
}

// four independent accumulators per thread, so that four loads are in flight
// (a K*u launch on a large grid leaves tens of thousands of partials)
__device__ double msum_partials(const double *__restrict__ part, int nb) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int i = threadIdx.x;
    for (; i + 3 * MB < nb; i += 4 * MB) {
        s0 += part[i];
        s1 += part[i + MB];
        s2 += part[i + 2 * MB];
        s3 += part[i + 3 * MB];
    }
    for (; i < nb; i += MB) s0 += part[i];
    return mblock_reduce((s0 + s1) + (s2 + s3));
}

// inner scalars (FP64 storage): rho = z.s of the last iteration, alpha, beta,
// r0 = s.s at entry, the iteration count of this inner solve, the current
// iteration cap, whether the last inner solve stopped at that cap short of
// its tolerance, and (slot 8) the total over the outer solve (reset by the
// host at the start of each solve)
enum { IS_RHO = 0, IS_ALPHA = 1, IS_BETA = 2, IS_R0 = 3, IS_IT = 4, IS_KCAP = 5, IS_CAPHIT = 6, IS_TOT = 8 };

// op 0 (entry of an inner solve): r0 = sum, rho = 0, it = 0, and the cap:
// kbase at the first inner solve of an outer solve, doubled (up to klimit)
// after an inner solve that hit its cap without reaching its tolerance;
// op 1: alpha = rho / sum;  op 2: beta = sum / rho (0 on the first iteration,
// rho = 0), rho = sum
__global__ void k_icg_scalar(int op, double *__restrict__ sc, const double *__restrict__ part, int nb, int kbase,
                             int klimit) {
    const double s = msum_partials(part, nb);
    if (threadIdx.x != 0) return;
    if (op == 0) {
        if (sc[IS_TOT] == 0.0) {
            sc[IS_KCAP] = (double)kbase;
        } else if (sc[IS_CAPHIT] != 0.0) {
            sc[IS_KCAP] = fmin(2.0 * sc[IS_KCAP], (double)klimit);
        }
        sc[IS_CAPHIT] = 0.0;
        sc[IS_R0] = s;
        sc[IS_RHO] = 0.0;
        sc[IS_IT] = 0.0;
        sc[IS_ALPHA] = 0.0;   // the first d update adds alpha * d = 0 to e
    } else if (op == 1) {
        sc[IS_ALPHA] = (s != 0.0) ? sc[IS_RHO] / s : 0.0;
    } else {
        sc[IS_BETA] = (sc[IS_RHO] != 0.0) ? s / sc[IS_RHO] : 0.0;
        sc[IS_RHO] = s;
    }
}

// end of an inner iteration: count it and keep iterating while it < kmax and
// ||s|| > eta ||s_0||, eta = max(eta_min, tol / (2 relres)) with the outer
// solve's tolerance and current relative residual (outer[15], outer[3]): the
// inner solve of the last outer step only goes as far as the outer tolerance
// needs.  eta_min <= 0: exactly kmax iterations.  Sets the condition of the
// graph's while node.
__global__ void k_icg_cond(cudaGraphConditionalHandle h, double *__restrict__ sc, const double *__restrict__ part,
                           int nb, int kmax, double eta_min, const double *__restrict__ outer,
                           double *__restrict__ total) {
    const double ss = msum_partials(part, nb);
    if (threadIdx.x != 0) return;
    const double it = sc[IS_IT] + 1.0;
    sc[IS_IT] = it;
    *total += 1.0;
    const double cap = eta_min > 0.0 ? sc[IS_KCAP] : (double)kmax;
    bool more = it < cap;
    if (eta_min > 0.0) {
        const double relres = outer[3], tol = outer[15];
        const double eta = (relres > 0.0) ? fmax(eta_min, 0.5 * tol / relres) : eta_min;
        const bool above = ss > eta * eta * sc[IS_R0];
        if (!more && above) sc[IS_CAPHIT] = 1.0;
        more = more && above;
    }
    cudaGraphSetConditional(h, more ? 1u : 0u);
}

// sets a conditional handle: a handle's default value is applied when the
// top-level graph is launched, not when a conditional body containing its
// node runs again, so a loop nested in another loop's body is re-armed with
// this kernel before each entry
__global__ void k_set_cond(cudaGraphConditionalHandle h, unsigned v) {
    if (threadIdx.x == 0) cudaGraphSetConditional(h, v);
}

void launch_set_cond(cudaGraphConditionalHandle h, unsigned v, cudaStream_t s) {
    ++g_launches;
    k_set_cond<<<1, 32, 0, s>>>(h, v);
}

// after the outer residual test: keep the outer while loop going and apply
// the preconditioner (the if node) unless the solve stopped (iflag[2])
__global__ void k_outer_cond(cudaGraphConditionalHandle hw, cudaGraphConditionalHandle hi,
                             const int *__restrict__ iflag) {
    if (threadIdx.x != 0) return;
    const unsigned go = iflag[2] ? 0u : 1u;
    cudaGraphSetConditional(hw, go);
    cudaGraphSetConditional(hi, go);
}

void launch_outer_cond(cudaGraphConditionalHandle hw, cudaGraphConditionalHandle hi, const int *iflag,
                       cudaStream_t s) {
    ++g_launches;
    k_outer_cond<<<1, 32, 0, s>>>(hw, hi, iflag);
}

// the same decision written to *flag for a host-driven loop (profiling: the
// kernels of a conditional graph body do not appear in a profiler's launch list)
__global__ void k_icg_cond_flag(int *flag, double *__restrict__ sc, const double *__restrict__ part, int nb,
                                int kmax, double eta_min, const double *__restrict__ outer,
                                double *__restrict__ total) {
    const double ss = msum_partials(part, nb);
    if (threadIdx.x != 0) return;
    const double it = sc[IS_IT] + 1.0;
    sc[IS_IT] = it;
    *total += 1.0;
    const double cap = eta_min > 0.0 ? sc[IS_KCAP] : (double)kmax;
    bool more = it < cap;
    if (eta_min > 0.0) {
        const double relres = outer[3], tol = outer[15];
        const double eta = (relres > 0.0) ? fmax(eta_min, 0.5 * tol / relres) : eta_min;
        const bool above = ss > eta * eta * sc[IS_R0];
        if (!more && above) sc[IS_CAPHIT] = 1.0;
        more = more && above;
    }
    *flag = more ? 1 : 0;
}

void launch_icg_cond_flag(int *flag, double *sc, const double *part, int nb, int kmax, double eta_min,
                          const double *outer, double *total, cudaStream_t s) {
    ++g_launches;
    k_icg_cond_flag<<<1, MB, 0, s>>>(flag, sc, part, nb, kmax, eta_min, outer, total);
}

void launch_icg_cond(cudaGraphConditionalHandle h, double *sc, const double *part, int nb, int kmax,
                     double eta_min, const double *outer, double *total, cudaStream_t s) {
    ++g_launches;
    k_icg_cond<<<1, MB, 0, s>>>(h, sc, part, nb, kmax, eta_min, outer, total);
}

// s = r, e = 0, d = 0 and partial sums of s.s (entry of an inner solve)
__global__ void k_icg_init(const float *__restrict__ r, float *__restrict__ s, float *__restrict__ e,
                           float *__restrict__ d, int64_t n, double *__restrict__ part) {
    float acc = 0.f;
    for (int64_t i = blockIdx.x * (int64_t)MB + threadIdx.x; i < n; i += (int64_t)gridDim.x * MB) {
        const float v = r[i];
        s[i] = v;
        e[i] = 0.f;
        d[i] = 0.f;
        acc = fmaf(v, v, acc);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double wred[MB / 32];
    if ((threadIdx.x & 31) == 0) wred[threadIdx.x >> 5] = (double)acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < MB / 32; ++i) t += wred[i];
        part[blockIdx.x] = t;
    }
}

int launch_icg_init(const float *r, float *s, float *e, float *d, int64_t n, double *part, cudaStream_t st) {
    ++g_launches;
    const int nb = reduce_blocks(n);
    k_icg_init<<<nb, MB, 0, st>>>(r, s, e, d, n, part);
    return nb;
}

void launch_icg_scalar(int op, double *sc, const double *part, int nb, cudaStream_t s, int kbase, int klimit) {
    ++g_launches;
    k_icg_scalar<<<1, MB, 0, s>>>(op, sc, part, nb, kbase, klimit);
}

// The FP32 vectors are separate allocations (256-byte aligned), so the
// streaming kernels below move them as float4 and finish the n % 4 tail
// element-wise.
__device__ __forceinline__ float4 fma4(float a, float4 x, float4 y) {
    return make_float4(fmaf(a, x.x, y.x), fmaf(a, x.y, y.y), fmaf(a, x.z, y.z), fmaf(a, x.w, y.w));
}

// s -= alpha t; partial sums of s.s (new s) when part != null.  The matching
// e += alpha d is deferred to the next d update (k_icg_dupdate), or, after the
// last iteration, to k_widen_dots: d is read there anyway, which saves one
// pass over e and d per iteration.
__global__ void k_icg_update(float *__restrict__ e, float *__restrict__ s, const float *__restrict__ d,
                             const float *__restrict__ t, int64_t n, const double *__restrict__ sc,
                             double *__restrict__ part) {
    (void)e;
    (void)d;
    const float a = (float)sc[IS_ALPHA];
    const int64_t n4 = n >> 2, stride = (int64_t)gridDim.x * MB;
    float4 *s4 = reinterpret_cast<float4 *>(s);
    const float4 *t4 = reinterpret_cast<const float4 *>(t);
    float acc = 0.f;
    for (int64_t i = blockIdx.x * (int64_t)MB + threadIdx.x; i < n4; i += stride) {
        const float4 v = fma4(-a, t4[i], s4[i]);
        s4[i] = v;
        acc = fmaf(v.x, v.x, fmaf(v.y, v.y, fmaf(v.z, v.z, fmaf(v.w, v.w, acc))));
    }
    const int64_t i = 4 * n4 + blockIdx.x * (int64_t)MB + threadIdx.x;
    if (i < n) {
        const float v = fmaf(-a, t[i], s[i]);
        s[i] = v;
        acc = fmaf(v, v, acc);
    }
    if (part) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        __shared__ double wred[MB / 32];
        if ((threadIdx.x & 31) == 0) wred[threadIdx.x >> 5] = (double)acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double tt = 0.0;
            for (int k = 0; k < MB / 32; ++k) tt += wred[k];
            part[blockIdx.x] = tt;
        }
    }
}

int launch_icg_update(float *e, float *s, const float *d, const float *t, int64_t n, const double *sc,
                      double *part, cudaStream_t st) {
    ++g_launches;
    const int nb = reduce_blocks(n);
    k_icg_update<<<nb, MB, 0, st>>>(e, s, d, t, n, sc, part);
    return nb;
}

// e += alpha d (the previous iteration's step, alpha still in place); then
// d = w + beta d
__global__ void k_icg_dupdate(float *__restrict__ e, float *__restrict__ d, const float *__restrict__ w, int64_t n,
                              const double *__restrict__ sc) {
    const float a = (float)sc[IS_ALPHA], b = (float)sc[IS_BETA];
    const int64_t n4 = n >> 2, stride = (int64_t)gridDim.x * MB;
    float4 *e4 = reinterpret_cast<float4 *>(e), *d4 = reinterpret_cast<float4 *>(d);
    const float4 *w4 = reinterpret_cast<const float4 *>(w);
    for (int64_t i = blockIdx.x * (int64_t)MB + threadIdx.x; i < n4; i += stride) {
        const float4 dv = d4[i];
        e4[i] = fma4(a, dv, e4[i]);
        d4[i] = fma4(b, dv, w4[i]);
    }
    const int64_t i = 4 * n4 + blockIdx.x * (int64_t)MB + threadIdx.x;
    if (i < n) {
        const float dv = d[i];
        e[i] = fmaf(a, dv, e[i]);
        d[i] = fmaf(b, dv, w[i]);
    }
}

void launch_icg_dupdate(float *e, float *d, const float *w, int64_t n, const double *sc, cudaStream_t st) {
    ++g_launches;
    k_icg_dupdate<<<reduce_blocks(n), MB, 0, st>>>(e, d, w, n, sc);
}

// ---- the same two updates over the active runs only -------------------------
// On a grid with inactive regions the inner CG's vectors are exactly zero at
// inactive nodes: the inner solve's entry kernel writes every node, K*u and
// the V-cycle leave zeros there, and these updates keep zeros zero.  So the
// updates may visit only the active nodes' words.
// The active y-runs (merged where they touch or lie a few nodes apart) are
// cut into chunks of at most 2048 floats, each cut on a 16-byte boundary
// (runs[i] = first DOF | floats << 40).  A warp takes a chunk: the words up to
// the first 16-byte boundary one by one, then float4 groups, then the last
// words.  Sums visit the chunks in a fixed order.
constexpr int RUN_SHIFT = 40;
constexpr int64_t RUN_MASK = (int64_t(1) << RUN_SHIFT) - 1;

// the chunk's words [b, b + len): head words before a 16-byte boundary, the
// float4 groups of the body, tail words; f(i) for single words, f4(i4) for a
// float4 group at float index 4 * i4
template <typename F1, typename F4>
__device__ __forceinline__ void run_chunk(int64_t b, int len, int lane, F1 f1, F4 f4) {
    const int head = min((int)((4 - (b & 3)) & 3), len);
    if (lane < head) f1(b + lane);
    const int64_t a4 = (b + head) >> 2;
    const int n4 = (len - head) >> 2;
    // unrolled so that several groups' loads are in flight at once
#pragma unroll 4
    for (int k = lane; k < n4; k += 32) f4(a4 + k);
    const int rest = len - head - 4 * n4;
    if (lane < rest) f1(b + head + 4 * (int64_t)n4 + lane);
}

__global__ void __launch_bounds__(MB) k_icg_update_runs(float *__restrict__ s, const float *__restrict__ t,
                                                        const int64_t *__restrict__ runs, int64_t nruns,
                                                        const double *__restrict__ sc, double *__restrict__ part) {
    const float a = (float)sc[IS_ALPHA];
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (int64_t)blockIdx.x * (MB / 32) + (threadIdx.x >> 5), nw = (int64_t)gridDim.x * (MB / 32);
    float4 *s4 = reinterpret_cast<float4 *>(s);
    const float4 *t4 = reinterpret_cast<const float4 *>(t);
    float acc = 0.f;
    for (int64_t r = w0; r < nruns; r += nw) {
        const int64_t rv = runs[r];
        run_chunk(
            rv & RUN_MASK, (int)(rv >> RUN_SHIFT), lane,
            [&](int64_t i) {
                const float v = fmaf(-a, t[i], s[i]);
                s[i] = v;
                acc = fmaf(v, v, acc);
            },
            [&](int64_t i4) {
                const float4 v = fma4(-a, t4[i4], s4[i4]);
                s4[i4] = v;
                acc = fmaf(v.x, v.x, fmaf(v.y, v.y, fmaf(v.z, v.z, fmaf(v.w, v.w, acc))));
            });
    }
    if (part) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        __shared__ double wred[MB / 32];
        if (lane == 0) wred[threadIdx.x >> 5] = (double)acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double tt = 0.0;
            for (int k = 0; k < MB / 32; ++k) tt += wred[k];
            part[blockIdx.x] = tt;
        }
    }
}

__global__ void __launch_bounds__(MB) k_icg_dupdate_runs(float *__restrict__ e, float *__restrict__ d,
                                                         const float *__restrict__ w,
                                                         const int64_t *__restrict__ runs, int64_t nruns,
                                                         const double *__restrict__ sc) {
    const float a = (float)sc[IS_ALPHA], bt = (float)sc[IS_BETA];
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (int64_t)blockIdx.x * (MB / 32) + (threadIdx.x >> 5), nw = (int64_t)gridDim.x * (MB / 32);
    float4 *e4 = reinterpret_cast<float4 *>(e), *d4 = reinterpret_cast<float4 *>(d);
    const float4 *w4 = reinterpret_cast<const float4 *>(w);
    for (int64_t r = w0; r < nruns; r += nw) {
        const int64_t rv = runs[r];
        run_chunk(
            rv & RUN_MASK, (int)(rv >> RUN_SHIFT), lane,
            [&](int64_t i) {
                const float dv = d[i];
                e[i] = fmaf(a, dv, e[i]);
                d[i] = fmaf(bt, dv, w[i]);
            },
            [&](int64_t i4) {
                const float4 dv = d4[i4];
                e4[i4] = fma4(a, dv, e4[i4]);
                d4[i4] = fma4(bt, dv, w4[i4]);
            });
    }
}

static int run_blocks(int64_t nruns) {
    const int64_t b = (nruns + MB / 32 - 1) / (MB / 32);
    return (int)(b < 1216 ? (b > 0 ? b : 1) : 1216);   // 152 SMs x 8 CTAs
}

int launch_icg_update_runs(float *s, const float *t, const int64_t *runs, int64_t nruns, const double *sc,
                           double *part, cudaStream_t st) {
    ++g_launches;
    const int nb = run_blocks(nruns);
    k_icg_update_runs<<<nb, MB, 0, st>>>(s, t, runs, nruns, sc, part);
    return nb;
}

void launch_icg_dupdate_runs(float *e, float *d, const float *w, const int64_t *runs, int64_t nruns,
                             const double *sc, cudaStream_t st) {
    ++g_launches;
    k_icg_dupdate_runs<<<run_blocks(nruns), MB, 0, st>>>(e, d, w, runs, nruns, sc);
}

// z64 = e32 + alpha d32 (the last iteration's deferred step; masked at fixed
// DOFs by construction), partials of z.r and z.q
__global__ void k_widen_dots(const float *__restrict__ e, const float *__restrict__ d,
                             const double *__restrict__ sc, double *__restrict__ z, const double *__restrict__ r,
                             const double *__restrict__ q, int64_t n, double *__restrict__ p1,
                             double *__restrict__ p2) {
    const float al = (float)sc[IS_ALPHA];
    double a = 0.0, b = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)MB + threadIdx.x; i < n; i += (int64_t)gridDim.x * MB) {
        const double zi = (double)fmaf(al, d[i], e[i]);
        z[i] = zi;
        a += zi * r[i];
        b += zi * q[i];
    }
    a = mblock_reduce(a);
    b = mblock_reduce(b);
    if (threadIdx.x == 0) {
        p1[blockIdx.x] = a;
        p2[blockIdx.x] = b;
    }
}

void launch_widen_dots(const float *e, const float *d, const double *sc, double *z, const double *r,
                       const double *q, int64_t n, double *p1, double *p2, int nb, cudaStream_t st) {
    ++g_launches;
    k_widen_dots<<<nb, MB, 0, st>>>(e, d, sc, z, r, q, n, p1, p2);
}

// outer flexible-PCG scalars after the preconditioner: beta = -lambda zq / x1, x1 = zr
// (slots as in kernels_vec.cu: S_X1 = 1, S_LAM = 2, S_BETA = 4)
__global__ void k_flex_beta(double *__restrict__ scal, const int *__restrict__ iflag, const double *__restrict__ p1,
                            const double *__restrict__ p2, int nb, int first) {
    const double zr = msum_partials(p1, nb);
    const double zq = msum_partials(p2, nb);
    if (threadIdx.x != 0) return;
    if (first) {
        scal[1] = zr;
        return;
    }
    if (iflag[2]) return;
    scal[4] = -scal[2] * zq / scal[1];
    scal[1] = zr;
}

void launch_flex_beta(double *scal, const int *iflag, const double *p1, const double *p2, int nb, int first,
                      cudaStream_t st) {
    ++g_launches;
    k_flex_beta<<<1, MB, 0, st>>>(scal, iflag, p1, p2, nb, first);
}

// r32 = (float) r64
__global__ void k_narrow(const double *__restrict__ a, float *__restrict__ b, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)MB + threadIdx.x; i < n; i += (int64_t)gridDim.x * MB) b[i] = (float)a[i];
}

void launch_narrow(const double *a, float *b, int64_t n, cudaStream_t st) {
    ++g_launches;
    k_narrow<<<reduce_blocks(n), MB, 0, st>>>(a, b, n);
}

// r64 = (double) r32
__global__ void k_widen(const float *__restrict__ a, double *__restrict__ b, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)MB + threadIdx.x; i < n; i += (int64_t)gridDim.x * MB) b[i] = (double)a[i];
}

void launch_widen(const float *a, double *b, int64_t n, cudaStream_t st) {
    ++g_launches;
    k_widen<<<reduce_blocks(n), MB, 0, st>>>(a, b, n);
}

}  // namespace sgld
