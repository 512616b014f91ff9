// SIMP topology-optimisation kernels around the solve
// (reference: src/TopOpti_GlobalVolumeConstraint_Tmp.m:26-120 with the cone
// density filter of src/MEXfuncs/TopOpti_SetupDensityFilter_mex.cpp:23-50 and
// TopOpti_PerformDensityFiltering_mex.cpp:75-102).
//
// Element fields live on the finest level's full element grid (inactive = 0).
// The filter weights max(0, rmin - |d|) depend only on the offset d, so they
// are formed once on the host with the reference's expression and kept in a
// small device buffer of the context; the kernel sums over the box in the
// reference's loop order (z outer, x, y inner).
#include <math.h>

#include <algorithm>

#include "sgld_internal.cuh"

namespace sgld {

constexpr int FW_MAX = 7;   // box side up to 7 (rmin <= 4)

// The weights go to the context's own device buffer d_w (FW_MAX^3 doubles), not
// to constant memory shared by the device, so that contexts filtering with
// different radii do not overwrite each other's.
void upload_filter_weights(double rmin, int *radius, double *d_w, cudaStream_t s) {
    const int r = (int)ceil(rmin) - 1;
    const int side = 2 * r + 1;
    double w[FW_MAX * FW_MAX * FW_MAX];
    for (int dz = -r; dz <= r; ++dz)
        for (int dx = -r; dx <= r; ++dx)
            for (int dy = -r; dy <= r; ++dy) {
                const double d = rmin - sqrt((double)(dx * dx + dy * dy + dz * dz));
                w[(dz + r) * side * side + (dx + r) * side + (dy + r)] = d > 0.0 ? d : 0.0;
            }
    cudaMemcpyAsync(d_w, w, sizeof(double) * side * side * side, cudaMemcpyHostToDevice, s);
    *radius = r;
}

// y_e = sum_{e2 in box, active} w(e - e2) x_e2   (x == nullptr: the weight sums Hs)
__global__ void k_density_filter(const double *__restrict__ x, const uint8_t *__restrict__ eact, int ny, int nx,
                                 int nz, int r, const double *__restrict__ fw, double *__restrict__ y) {
    const int pl = blockIdx.x * blockDim.x + threadIdx.x;
    if (pl >= ny * nx) return;
    const int jj = pl % ny, ii = pl / ny, kk = blockIdx.y;
    const int64_t e = (int64_t)pl + (int64_t)ny * nx * kk;
    if (!eact[e]) {
        y[e] = 0.0;
        return;
    }
    const int side = 2 * r + 1;
    double acc = 0.0;
    for (int k2 = max(kk - r, 0); k2 <= min(kk + r, nz - 1); ++k2)
        for (int i2 = max(ii - r, 0); i2 <= min(ii + r, nx - 1); ++i2)
            for (int j2 = max(jj - r, 0); j2 <= min(jj + r, ny - 1); ++j2) {
                const int64_t e2 = (int64_t)j2 + (int64_t)ny * (i2 + (int64_t)nx * k2);
                if (!eact[e2]) continue;
                const double w = fw[(k2 - kk + r) * side * side + (i2 - ii + r) * side + (j2 - jj + r)];
                acc += x ? w * x[e2] : w;
            }
    y[e] = acc;
}

void launch_density_filter(const Level &l0, const double *x, int r, const double *fw, double *y, cudaStream_t s) {
    const dim3 g((unsigned)((l0.ny * l0.nx + 255) / 256), (unsigned)l0.nz);
    ++g_launches;
    k_density_filter<<<g, 256, 0, s>>>(x, l0.eact, l0.ny, l0.nx, l0.nz, r, fw, y);
}

constexpr int TB = 256;

__device__ __forceinline__ double tblock_sum(double v) {
    __shared__ double red[TB / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < TB / 32; ++i) s += red[i];
    return s;
}

__device__ __forceinline__ double tblock_max(double v) {
    __shared__ double red[TB / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < TB / 32; ++i) s = fmax(s, red[i]);
    return s;
}

// E = Emin + xPhys^p (E0 - Emin) on active elements (TopOpti_MaterialInterpolationSIMP.m:5);
// partial sums of xPhys (volume) and of 4 xPhys (1 - xPhys) (sharpness, :102)
__global__ void k_topo_modulus(const double *__restrict__ xp, const uint8_t *__restrict__ eact, int64_t n, double p,
                               double E0, double Emin, double *__restrict__ E, double *__restrict__ part_v,
                               double *__restrict__ part_s) {
    double sv = 0.0, ss = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)TB + threadIdx.x; e < n; e += (int64_t)gridDim.x * TB) {
        if (!eact[e]) {
            E[e] = 0.0;
            continue;
        }
        const double v = xp[e];
        E[e] = Emin + pow(v, p) * (E0 - Emin);
        sv += v;
        ss += 4.0 * v * (1.0 - v);
    }
    sv = tblock_sum(sv);
    ss = tblock_sum(ss);
    if (threadIdx.x == 0) {
        part_v[blockIdx.x] = sv;
        part_s[blockIdx.x] = ss;
    }
}

// dc/Hs and dv/Hs (TopOpti_GlobalVolumeConstraint_Tmp.m:66-77, ft = 2):
// dc = -p (E0 - Emin) xPhys^(p-1) ce (TopOpti_DeMaterialInterpolation.m:5)
__global__ void k_topo_sens(const double *__restrict__ xp, const double *__restrict__ ce,
                            const double *__restrict__ Hs, const uint8_t *__restrict__ eact, int64_t n, double p,
                            double E0, double Emin, double *__restrict__ dcs, double *__restrict__ dvs) {
    for (int64_t e = blockIdx.x * (int64_t)TB + threadIdx.x; e < n; e += (int64_t)gridDim.x * TB) {
        if (!eact[e]) {
            dcs[e] = 0.0;
            dvs[e] = 0.0;
            continue;
        }
        const double dc = -(p * (E0 - Emin) * pow(xp[e], p - 1.0)) * ce[e];
        dcs[e] = dc / Hs[e];
        dvs[e] = 1.0 / Hs[e];
    }
}

// q = x sqrt(-dc/dv) once per update, so that a bisection step needs one
// multiply per element: x sqrt(-dc/dv/lmid) = q / sqrt(lmid)
__global__ void k_topo_q(const double *__restrict__ x, const double *__restrict__ dc, const double *__restrict__ dv,
                         const uint8_t *__restrict__ eact, int64_t n, double *__restrict__ q) {
    for (int64_t e = blockIdx.x * (int64_t)TB + threadIdx.x; e < n; e += (int64_t)gridDim.x * TB)
        q[e] = eact[e] ? x[e] * sqrt(-dc[e] / dv[e]) : 0.0;
}

// bisection state (device): [0] lo [1] hi [2] lmid [3] g [4] done [5] steps
enum { OC_LO = 0, OC_HI = 1, OC_MID = 2, OC_G = 3, OC_DONE = 4, OC_STEPS = 5 };

__device__ __forceinline__ double oc_new(double xe, double qe, double rs, double move) {
    // max(0, max(x - move, min(1, min(x + move, x sqrt(-dc/dv/lmid)))))   (:87)
    return fmax(0.0, fmax(xe - move, fmin(1.0, fmin(xe + move, qe * rs))));
}

// element flags of level 1: bit 0 active, bit 1 passive (kept solid by the
// SIMP loop; TopOpti_GlobalVolumeConstraint.m:162,179)
constexpr uint8_t EF_PASSIVE = 2;

__global__ void k_oc_step(const double *__restrict__ x, const double *__restrict__ q, const double *__restrict__ dv,
                          const uint8_t *__restrict__ eact, int64_t n, double move, const double *__restrict__ st,
                          double *__restrict__ part) {
    if (st[OC_DONE] != 0.0) return;
    const double lmid = 0.5 * (st[OC_HI] + st[OC_LO]);
    const double rs = 1.0 / sqrt(lmid);
    double s = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)TB + threadIdx.x; e < n; e += (int64_t)gridDim.x * TB) {
        if (!eact[e]) continue;
        const double xn = (eact[e] & EF_PASSIVE) ? 1.0 : oc_new(x[e], q[e], rs, move);
        s += dv[e] * (xn - x[e]);
    }
    s = tblock_sum(s);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__device__ double tsum_partials(const double *__restrict__ part, int nb) {
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += TB) s += part[i];
    return tblock_sum(s);
}

// op 0: init (g = sum_v / n - V, lo = 0, hi = 1e9); op 1: bisection update (:88-89)
__global__ void k_oc_scalar(int op, double *__restrict__ st, const double *__restrict__ part, int nb, double nact,
                            double volfrac) {
    const double s = tsum_partials(part, nb);
    if (threadIdx.x != 0) return;
    if (op == 0) {
        st[OC_G] = s / nact - volfrac;
        st[OC_LO] = 0.0;
        st[OC_HI] = 1e9;
        st[OC_DONE] = 0.0;
        st[OC_STEPS] = 0.0;
        st[OC_MID] = 0.5e9;
        return;
    }
    if (st[OC_DONE] != 0.0) return;
    const double lmid = 0.5 * (st[OC_HI] + st[OC_LO]);
    st[OC_MID] = lmid;
    const double gt = st[OC_G] + s;
    if (gt > 0.0)
        st[OC_LO] = lmid;
    else
        st[OC_HI] = lmid;
    st[OC_STEPS] += 1.0;
    if (!((st[OC_HI] - st[OC_LO]) / (st[OC_LO] + st[OC_HI]) > 1e-6)) st[OC_DONE] = 1.0;
}

// x <- xnew(lmid of the last bisection step); partial max |xnew - x| (:91-92)
__global__ void k_oc_apply(double *__restrict__ x, const double *__restrict__ q, const uint8_t *__restrict__ eact,
                           int64_t n, double move, const double *__restrict__ st, double *__restrict__ part) {
    const double rs = 1.0 / sqrt(st[OC_MID]);
    double m = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)TB + threadIdx.x; e < n; e += (int64_t)gridDim.x * TB) {
        if (!eact[e]) continue;
        const double xn = (eact[e] & EF_PASSIVE) ? 1.0 : oc_new(x[e], q[e], rs, move);
        m = fmax(m, fabs(xn - x[e]));
        x[e] = xn;
    }
    m = tblock_max(m);
    if (threadIdx.x == 0) part[blockIdx.x] = m;
}

__global__ void k_max_partials(const double *__restrict__ part, int nb, double *__restrict__ out) {
    double m = 0.0;
    for (int i = threadIdx.x; i < nb; i += TB) m = fmax(m, part[i]);
    m = tblock_max(m);
    if (threadIdx.x == 0) out[0] = m;
}

// y = a / b on active elements (passive ones: 1), 0 elsewhere
__global__ void k_div(const double *__restrict__ a, const double *__restrict__ b, const uint8_t *__restrict__ eact,
                      int64_t n, double *__restrict__ y) {
    for (int64_t e = blockIdx.x * (int64_t)TB + threadIdx.x; e < n; e += (int64_t)gridDim.x * TB)
        y[e] = eact[e] ? ((eact[e] & EF_PASSIVE) ? 1.0 : a[e] / b[e]) : 0.0;
}

// MMA inputs of the design variables (active, not passive elements; full-grid
// indices var[i]): xval, xmin = max(0, x - move), xmax = min(1, x + move),
// df0dx = dc, dfdx = dv * scale (TopOpti_GlobalVolumeConstraint.m:142-151)
__global__ void k_mma_gather(const int64_t *__restrict__ var, int64_t nvar, const double *__restrict__ x,
                             const double *__restrict__ dc, const double *__restrict__ dv, double move, double scale,
                             double *__restrict__ xv, double *__restrict__ xmin, double *__restrict__ xmax,
                             double *__restrict__ df0, double *__restrict__ dg) {
    for (int64_t i = blockIdx.x * (int64_t)TB + threadIdx.x; i < nvar; i += (int64_t)gridDim.x * TB) {
        const int64_t e = var[i];
        const double xe = x[e];
        xv[i] = xe;
        xmin[i] = fmax(0.0, xe - move);
        xmax[i] = fmin(1.0, xe + move);
        df0[i] = dc[e];
        dg[i] = dv[e] * scale;
    }
}

// x(var) = MMA result; passive elements to 1 (x = onesArrSingle before the
// variables are written, :154-155); partial max |xnew - xval| (:153)
__global__ void k_mma_scatter(const int64_t *__restrict__ var, int64_t nvar, const double *__restrict__ xn,
                              const double *__restrict__ xv, double *__restrict__ x, double *__restrict__ part) {
    double m = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)TB + threadIdx.x; i < nvar; i += (int64_t)gridDim.x * TB) {
        x[var[i]] = xn[i];
        m = fmax(m, fabs(xn[i] - xv[i]));
    }
    m = tblock_max(m);
    if (threadIdx.x == 0) part[blockIdx.x] = m;
}

__global__ void k_set_passive_x(double *__restrict__ x, const uint8_t *__restrict__ eact, int64_t n) {
    for (int64_t e = blockIdx.x * (int64_t)TB + threadIdx.x; e < n; e += (int64_t)gridDim.x * TB)
        if (eact[e] & EF_PASSIVE) x[e] = 1.0;
}

// eact bit 1: cleared everywhere, then set for the listed full-grid elements
__global__ void k_clear_passive(uint8_t *__restrict__ eact, int64_t n) {
    for (int64_t e = blockIdx.x * (int64_t)TB + threadIdx.x; e < n; e += (int64_t)gridDim.x * TB)
        eact[e] = (uint8_t)(eact[e] & ~EF_PASSIVE);
}
__global__ void k_mark_passive(uint8_t *__restrict__ eact, const int64_t *__restrict__ full, int64_t np) {
    for (int64_t i = blockIdx.x * (int64_t)TB + threadIdx.x; i < np; i += (int64_t)gridDim.x * TB)
        eact[full[i]] = (uint8_t)(eact[full[i]] | EF_PASSIVE);
}

__global__ void k_fill_active(double *__restrict__ y, const uint8_t *__restrict__ eact, int64_t n, double v) {
    for (int64_t e = blockIdx.x * (int64_t)TB + threadIdx.x; e < n; e += (int64_t)gridDim.x * TB)
        y[e] = eact[e] ? v : 0.0;
}

// ---- launchers ----------------------------------------------------------------
void launch_topo_modulus(const Level &l0, const double *xp, double p, double E0, double Emin, double *E,
                         double *pv, double *ps, int nb, cudaStream_t s) {
    ++g_launches;
    k_topo_modulus<<<nb, TB, 0, s>>>(xp, l0.eact, l0.nel, p, E0, Emin, E, pv, ps);
}
void launch_topo_sens(const Level &l0, const double *xp, const double *ce, const double *Hs, double p, double E0,
                      double Emin, double *dcs, double *dvs, int nb, cudaStream_t s) {
    ++g_launches;
    k_topo_sens<<<nb, TB, 0, s>>>(xp, ce, Hs, l0.eact, l0.nel, p, E0, Emin, dcs, dvs);
}
void launch_topo_q(const Level &l0, const double *x, const double *dc, const double *dv, double *q, int nb,
                   cudaStream_t s) {
    ++g_launches;
    k_topo_q<<<nb, TB, 0, s>>>(x, dc, dv, l0.eact, l0.nel, q);
}
void launch_oc_step(const Level &l0, const double *x, const double *q, const double *dv, double move,
                    const double *st, double *part, int nb, cudaStream_t s) {
    ++g_launches;
    k_oc_step<<<nb, TB, 0, s>>>(x, q, dv, l0.eact, l0.nel, move, st, part);
}
void launch_oc_scalar(int op, double *st, const double *part, int nb, double nact, double volfrac, cudaStream_t s) {
    ++g_launches;
    k_oc_scalar<<<1, TB, 0, s>>>(op, st, part, nb, nact, volfrac);
}
void launch_oc_apply(const Level &l0, double *x, const double *q, double move, const double *st, double *part,
                     int nb, cudaStream_t s) {
    ++g_launches;
    k_oc_apply<<<nb, TB, 0, s>>>(x, q, l0.eact, l0.nel, move, st, part);
}
void launch_max_partials(const double *part, int nb, double *out, cudaStream_t s) {
    ++g_launches;
    k_max_partials<<<1, TB, 0, s>>>(part, nb, out);
}
void launch_div(const Level &l0, const double *a, const double *b, double *y, int nb, cudaStream_t s) {
    ++g_launches;
    k_div<<<nb, TB, 0, s>>>(a, b, l0.eact, l0.nel, y);
}
int launch_mma_gather(const int64_t *var, int64_t nvar, const double *x, const double *dc, const double *dv,
                      double move, double scale, double *xv, double *xmin, double *xmax, double *df0, double *dg,
                      cudaStream_t s) {
    ++g_launches;
    const int nb = (int)std::min<int64_t>((nvar + TB - 1) / TB, 152 * 8);
    k_mma_gather<<<std::max(nb, 1), TB, 0, s>>>(var, nvar, x, dc, dv, move, scale, xv, xmin, xmax, df0, dg);
    return std::max(nb, 1);
}
void launch_mma_scatter(const int64_t *var, int64_t nvar, const double *xn, const double *xv, double *x,
                        double *part, int nb, cudaStream_t s) {
    ++g_launches;
    k_mma_scatter<<<nb, TB, 0, s>>>(var, nvar, xn, xv, x, part);
}
void launch_set_passive_x(const Level &l0, double *x, int nb, cudaStream_t s) {
    ++g_launches;
    k_set_passive_x<<<nb, TB, 0, s>>>(x, l0.eact, l0.nel);
}
void launch_mark_passive(const Level &l0, const int64_t *full, int64_t np, int nb, cudaStream_t s) {
    ++g_launches;
    k_clear_passive<<<nb, TB, 0, s>>>(l0.eact, l0.nel);
    if (np > 0) {
        ++g_launches;
        const int nb2 = (int)std::max<int64_t>(1, std::min<int64_t>((np + TB - 1) / TB, 152 * 8));
        k_mark_passive<<<nb2, TB, 0, s>>>(l0.eact, full, np);
    }
}
void launch_fill_active(const Level &l0, double *y, double v, int nb, cudaStream_t s) {
    ++g_launches;
    k_fill_active<<<nb, TB, 0, s>>>(y, l0.eact, l0.nel, v);
}

// ---- local-volume loop (TopOpti_LocalVolumeConstraint.m) ------------------------
// Heaviside projection xp = H(xt) (TopOpti_DualizeDesignVariable.m:4) and, if
// dx != null, its derivative (TopOpti_DeDualizeDesignVariable.m:4); passive
// elements are set to 1 (TopOpti_LocalVolumeConstraint.m:204), void to 0
__global__ void k_heaviside(const double *__restrict__ xt, const uint8_t *__restrict__ eact, int64_t n,
                            double beta, double eta, double *__restrict__ xp, double *__restrict__ dx) {
    const double den = tanh(beta * eta) + tanh(beta * (1.0 - eta));
    for (int64_t e = blockIdx.x * (int64_t)TB + threadIdx.x; e < n; e += (int64_t)gridDim.x * TB) {
        if (!eact[e]) {
            if (xp) xp[e] = 0.0;
            if (dx) dx[e] = 0.0;
            continue;
        }
        const double t = tanh(beta * (xt[e] - eta));
        if (xp) xp[e] = (eact[e] & EF_PASSIVE) ? 1.0 : (tanh(beta * eta) + t) / den;
        if (dx) dx[e] = beta * (1.0 - t * t) / den;
    }
}

// dcs = dc .* dx ./ Hs with dc = -p (E0 - Emin) xp^(p-1) ce / c_solid
// (TopOpti_LocalVolumeConstraint.m:132-136, :153)
__global__ void k_local_sens(const double *__restrict__ xp, const double *__restrict__ ce,
                             const double *__restrict__ dx, const double *__restrict__ Hs,
                             const uint8_t *__restrict__ eact, int64_t n, double p, double E0, double Emin,
                             double inv_csolid, double *__restrict__ dcs) {
    for (int64_t e = blockIdx.x * (int64_t)TB + threadIdx.x; e < n; e += (int64_t)gridDim.x * TB) {
        if (!eact[e]) {
            dcs[e] = 0.0;
            continue;
        }
        const double dc = -(p * (E0 - Emin) * pow(xp[e], p - 1.0)) * ce[e] * inv_csolid;
        dcs[e] = dc * dx[e] / Hs[e];
    }
}

// partial sums of (xh / vmax)^p, vmax = alpha (1 on passive elements)
__global__ void k_pnorm_sum(const double *__restrict__ xh, const uint8_t *__restrict__ eact, int64_t n, double p,
                            double alpha, double *__restrict__ part) {
    double s = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)TB + threadIdx.x; e < n; e += (int64_t)gridDim.x * TB) {
        if (!eact[e]) continue;
        const double vm = (eact[e] & EF_PASSIVE) ? 1.0 : alpha;
        s += pow(xh[e], p) / pow(vm, p);
    }
    s = tblock_sum(s);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// dfdx_pde = (S/N)^(1/p-1) xh^(p-1) / vmax^p / N  (TopOpti_LocalVolumeConstraint.m:146); S on the device
__global__ void k_pnorm_grad(const double *__restrict__ xh, const uint8_t *__restrict__ eact, int64_t n, double p,
                             double alpha, const double *__restrict__ S, double N, double *__restrict__ g) {
    const double f = pow(*S / N, 1.0 / p - 1.0) / N;
    for (int64_t e = blockIdx.x * (int64_t)TB + threadIdx.x; e < n; e += (int64_t)gridDim.x * TB) {
        if (!eact[e]) {
            g[e] = 0.0;
            continue;
        }
        const double vm = (eact[e] & EF_PASSIVE) ? 1.0 : alpha;
        g[e] = f * pow(xh[e], p - 1.0) / pow(vm, p);
    }
}

// y = a .* b ./ c on active elements (b = null: y = a ./ c)
__global__ void k_mul_div(const double *__restrict__ a, const double *__restrict__ b, const double *__restrict__ c,
                          const uint8_t *__restrict__ eact, int64_t n, double *__restrict__ y) {
    for (int64_t e = blockIdx.x * (int64_t)TB + threadIdx.x; e < n; e += (int64_t)gridDim.x * TB)
        y[e] = eact[e] ? a[e] * (b ? b[e] : 1.0) / c[e] : 0.0;
}

void launch_heaviside(const Level &l0, const double *xt, double beta, double eta, double *xp, double *dx, int nb,
                      cudaStream_t s) {
    ++g_launches;
    k_heaviside<<<nb, TB, 0, s>>>(xt, l0.eact, l0.nel, beta, eta, xp, dx);
}

void launch_local_sens(const Level &l0, const double *xp, const double *ce, const double *dx, const double *Hs,
                       double p, double E0, double Emin, double inv_csolid, double *dcs, int nb, cudaStream_t s) {
    ++g_launches;
    k_local_sens<<<nb, TB, 0, s>>>(xp, ce, dx, Hs, l0.eact, l0.nel, p, E0, Emin, inv_csolid, dcs);
}

void launch_pnorm(const Level &l0, const double *xh, double p, double alpha, double *part, double *S, double N,
                  double *g, int nb, cudaStream_t s) {
    g_launches += 2;   // the finalize launch counts itself
    k_pnorm_sum<<<nb, TB, 0, s>>>(xh, l0.eact, l0.nel, p, alpha, part);
    launch_finalize_sum(part, nb, S, s);
    k_pnorm_grad<<<nb, TB, 0, s>>>(xh, l0.eact, l0.nel, p, alpha, S, N, g);
}

void launch_mul_div(const Level &l0, const double *a, const double *b, const double *c, double *y, int nb,
                    cudaStream_t s) {
    ++g_launches;
    k_mul_div<<<nb, TB, 0, s>>>(a, b, c, l0.eact, l0.nel, y);
}

}  // namespace sgld
