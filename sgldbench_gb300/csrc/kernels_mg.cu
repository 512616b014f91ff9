// Multigrid transfer, smoothing and bookkeeping kernels on the full grid.
//
// Restriction / prolongation (reference: src/Solving_RestrictResidual.m,
// src/Solving_InterpolationDeviation.m and their MEX kernels).  The
// reference builds a per-coarse-element table of the (s+1)^3 fine nodes,
// scatters RI' r / multiplicity into the coarse nodes and averages RI x over
// the elements sharing a fine node.  Because trilinear interpolation from a
// continuous coarse field gives the same value from every element that
// contains a fine node, that operator is exactly P = trilinear interpolation
// restricted to active fine nodes and R = P'.  On the structured grid this is
// a separable tent stencil of half-width s: w(d) = (s - |d|) / s per axis.
// Inactive nodes carry zeros on every level, so no tables are needed.
//
// The additive V-cycle of the reference (src/Solving_Vcycle.m:12-50) is
//   r_l = R r_{l-1};  x_L = A_L^-1 r_L;
//   x_{l} = t_l + P x_{l+1} + t_l  with t_l = (omega r_l) ./ D_l,
// summed in that order.  1 ./ D_l is formed once per assembly (the division
// is the most expensive FP64 operation of the cycle), so t_l may differ from
// the reference's (omega r_l) ./ D_l in the last bit.
#include "sgld_internal.cuh"

namespace sgld {

template <typename T>
__global__ void k_restrict(const T *__restrict__ rf, T *__restrict__ rc, int nyc, int nxc, int nzc, int s) {
    const int NYc = nyc + 1, NXc = nxc + 1, NZc = nzc + 1;
    const int NYf = s * nyc + 1, NXf = s * nxc + 1, NZf = s * nzc + 1;
    // grid: x over the (y, x) plane of coarse nodes, y over z (32-bit index math)
    const int pl = blockIdx.x * blockDim.x + threadIdx.x;
    if (pl >= NYc * NXc) return;
    const int I = pl % NYc, J = pl / NYc, Kz = blockIdx.y;
    const int64_t n = (int64_t)pl + (int64_t)NYc * NXc * Kz;
    (void)NZc;
    const T inv = T(1) / T(s);
    T a0 = T(0), a1 = T(0), a2 = T(0);
    for (int dz = -s + 1; dz < s; ++dz) {
        const int fz = s * Kz + dz;
        if (fz < 0 || fz >= NZf) continue;
        const T wz = T(s - abs(dz)) * inv;
        for (int dx = -s + 1; dx < s; ++dx) {
            const int fx = s * J + dx;
            if (fx < 0 || fx >= NXf) continue;
            const T wxz = T(s - abs(dx)) * inv * wz;
            for (int dy = -s + 1; dy < s; ++dy) {
                const int fy = s * I + dy;
                if (fy < 0 || fy >= NYf) continue;
                const T w = T(s - abs(dy)) * inv * wxz;
                const int64_t f = (int64_t)fy + (int64_t)NYf * (fx + (int64_t)NXf * fz);
                a0 += w * rf[3 * f];
                a1 += w * rf[3 * f + 1];
                a2 += w * rf[3 * f + 2];
            }
        }
    }
    rc[3 * n] = a0;
    rc[3 * n + 1] = a1;
    rc[3 * n + 2] = a2;
}

// The same restriction with the span S a compile-time constant: the
// (2S-1)^3 taps unroll, the weights are constants and the indices stay 32-bit
// (grids below 2^31 / 3 nodes).  Lanes hold consecutive coarse y, so for one
// (dx, dz) a warp's taps cover a contiguous run of fine nodes.
// A coarse node outside the active domain (cflag) gets 0 without reading the
// fine grid: all 8 coarse elements around it are empty, so every fine node
// strictly inside their union -- the tent's support -- is inactive and holds 0.
// With keep_zeros (the FP32 V-cycle, whose coarse vectors are zeroed when
// allocated) an inactive coarse node is not written at all: it holds 0 already.
template <typename T, int S>
__global__ void __launch_bounds__(128) k_restrict_s(const T *__restrict__ rf, T *__restrict__ rc,
                                                    const uint8_t *__restrict__ cflag, int nyc, int nxc, int nzc,
                                                    int keep_zeros) {
    const int NYc = nyc + 1, NXc = nxc + 1;
    const int NYf = S * nyc + 1, NXf = S * nxc + 1, NZf = S * nzc + 1;
    const int pl = blockIdx.x * blockDim.x + threadIdx.x;
    if (pl >= NYc * NXc) return;
    const int I = pl % NYc, J = pl / NYc, Kz = blockIdx.y;
    if (!(cflag[pl + NYc * NXc * Kz] & NF_ACTIVE)) {
        if (keep_zeros) return;
        const int n = 3 * (pl + NYc * NXc * Kz);
        rc[n] = rc[n + 1] = rc[n + 2] = T(0);
        return;
    }
    const T inv = T(1) / T(S);
    T a0 = T(0), a1 = T(0), a2 = T(0);
#pragma unroll
    for (int dz = -S + 1; dz < S; ++dz) {
        const int fz = S * Kz + dz;
        if (fz < 0 || fz >= NZf) continue;
        const T wz = T(S - (dz < 0 ? -dz : dz)) * inv;
#pragma unroll
        for (int dx = -S + 1; dx < S; ++dx) {
            const int fx = S * J + dx;
            if (fx < 0 || fx >= NXf) continue;
            const T wxz = T(S - (dx < 0 ? -dx : dx)) * inv * wz;
            const int base = NYf * (fx + NXf * fz);
#pragma unroll
            for (int dy = -S + 1; dy < S; ++dy) {
                const int fy = S * I + dy;
                if (fy < 0 || fy >= NYf) continue;
                const T w = T(S - (dy < 0 ? -dy : dy)) * inv * wxz;
                const int f = 3 * (fy + base);
                a0 += w * rf[f];
                a1 += w * rf[f + 1];
                a2 += w * rf[f + 2];
            }
        }
    }
    const int n = 3 * (pl + NYc * NXc * Kz);
    rc[n] = a0;
    rc[n + 1] = a1;
    rc[n + 2] = a2;
}

template <typename T>
void launch_restrict(const Level &fine, const Level &coarse, const T *rf, T *rc, cudaStream_t st) {
    ++g_launches;
    const dim3 g((unsigned)(((coarse.ny + 1) * (coarse.nx + 1) + 127) / 128), (unsigned)(coarse.nz + 1));
    const bool small = 3 * (int64_t)fine.nnode < (int64_t)INT32_MAX;
    // FP32: the coarse vectors (the levels' r32) are zeroed at allocation and keep zeros at
    // inactive nodes
    const int keep = sizeof(T) == sizeof(float) && static_cast<const void *>(rc) == coarse.r32;
    if (small && coarse.span == 2)
        k_restrict_s<T, 2><<<g, 128, 0, st>>>(rf, rc, coarse.nflag, coarse.ny, coarse.nx, coarse.nz, keep);
    else if (small && coarse.span == 4)
        k_restrict_s<T, 4><<<g, 128, 0, st>>>(rf, rc, coarse.nflag, coarse.ny, coarse.nx, coarse.nz, keep);
    else
        k_restrict<T><<<g, 128, 0, st>>>(rf, rc, coarse.ny, coarse.nx, coarse.nz, coarse.span);
}
template void launch_restrict<double>(const Level &, const Level &, const double *, double *, cudaStream_t);
template void launch_restrict<float>(const Level &, const Level &, const float *, float *, cudaStream_t);

// warp stage in the kernel's precision T, the warp sums added in FP64
template <typename T>
__device__ __forceinline__ double warp_block_sum(T v, double *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = (double)v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
    return s;
}

// x_f = t + P x_c + t, t = (omega r_f) .* D on active fine nodes, 0 elsewhere,
// where D holds the reciprocal Jacobi diagonal.
// FINAL (finest level): fixed DOFs set to 0 and partial sums of x_f . r_f.
template <typename T, bool FINAL>
__global__ void k_prolong_smooth(const T *__restrict__ xc, const T *__restrict__ rf, const T *__restrict__ D,
                                 const uint8_t *__restrict__ nflag, T omega, T *__restrict__ xf, int nyc, int nxc,
                                 int nzc, int s, double *__restrict__ partial) {
    const int NYc = nyc + 1, NXc = nxc + 1;
    const int NYf = s * nyc + 1, NXf = s * nxc + 1, NZf = s * nzc + 1;
    // grid: x over the (y, x) plane of fine nodes, y over z (32-bit index math)
    const int pl = blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)pl + (int64_t)NYf * NXf * blockIdx.y;
    T dot = T(0);
    (void)NZf;
    if (pl < NYf * NXf) {
        const uint8_t f = nflag[n];
        T o0 = T(0), o1 = T(0), o2 = T(0);
        if (f & NF_ACTIVE) {
            const int iy = pl % NYf, ix = pl / NYf, iz = blockIdx.y;
            const int I = iy / s, J = ix / s, Kz = iz / s;
            const int ry = iy - s * I, rx = ix - s * J, rz = iz - s * Kz;
            const T inv = T(1) / T(s);
            const T wy[2] = {T(s - ry) * inv, T(ry) * inv};
            const T wx[2] = {T(s - rx) * inv, T(rx) * inv};
            const T wz[2] = {T(s - rz) * inv, T(rz) * inv};
            T p0 = T(0), p1 = T(0), p2 = T(0);
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                if (c && rz == 0) continue;
#pragma unroll
                for (int b = 0; b < 2; ++b) {
                    if (b && rx == 0) continue;
#pragma unroll
                    for (int a = 0; a < 2; ++a) {
                        if (a && ry == 0) continue;
                        const T w = wy[a] * wx[b] * wz[c];
                        const int64_t m = (int64_t)(I + a) + (int64_t)NYc * ((J + b) + (int64_t)NXc * (Kz + c));
                        p0 += w * xc[3 * m];
                        p1 += w * xc[3 * m + 1];
                        p2 += w * xc[3 * m + 2];
                    }
                }
            }
            const T r0 = rf[3 * n], r1 = rf[3 * n + 1], r2 = rf[3 * n + 2];
            const T t0 = (omega * r0) * D[3 * n], t1 = (omega * r1) * D[3 * n + 1], t2 = (omega * r2) * D[3 * n + 2];
            o0 = (t0 + p0) + t0;
            o1 = (t1 + p1) + t1;
            o2 = (t2 + p2) + t2;
            if (FINAL) {
                if (f & NF_FIXX) o0 = T(0);
                if (f & NF_FIXY) o1 = T(0);
                if (f & NF_FIXZ) o2 = T(0);
                dot = o0 * r0 + o1 * r1 + o2 * r2;
            }
        }
        xf[3 * n] = o0;
        xf[3 * n + 1] = o1;
        xf[3 * n + 2] = o2;
    }
    if (FINAL && partial) {
        __shared__ double red[8];
        const double sum = warp_block_sum<T>(dot, red);
        if (threadIdx.x == 0) partial[blockIdx.x + gridDim.x * blockIdx.y] = sum;
    }
}

// The same operator with a thread per coarse node (I, J, K) writing the
// fine nodes (S I + ry, S J + rx, S K + rz), 0 <= ry, rx, rz < S (only 0
// past the last coarse cell of an axis): the 8 coarse corners are loaded once
// per S^3 fine nodes instead of once per fine node, and the interpolation is
// done axis by axis (z, then x, then y).  Span S is a compile-time constant,
// indices are 32-bit.  Same result as k_prolong_smooth up to the order of the
// interpolation sums.
// With cflag (the coarse node flags; passed for the FP32 V-cycle, whose output
// vectors are zeroed when allocated), a thread whose 8 coarse corners are all
// inactive writes nothing: every fine element touching one of its fine nodes
// lies in a coarse element sharing a corner with the cell, and an active
// coarse element makes all 8 of its corners active, so those fine nodes are
// inactive and already hold 0.
template <typename T, int S, bool FINAL>
__global__ void __launch_bounds__(128) k_prolong_cells(const T *__restrict__ xc, const T *__restrict__ rf,
                                                       const T *__restrict__ D, const uint8_t *__restrict__ nflag,
                                                       const uint8_t *__restrict__ cflag, T omega,
                                                       T *__restrict__ xf, int nyc, int nxc, int nzc, int zp,
                                                       double *__restrict__ partial) {
    const int NYc = nyc + 1, NXc = nxc + 1;
    const int NYf = S * nyc + 1, NXf = S * nxc + 1;
    const int pl = blockIdx.x * blockDim.x + threadIdx.x;
    T dot = T(0);
    // coarse planes K = blockIdx.y * zp .. + zp - 1 (fewer CTAs, so fewer partial sums)
    for (int K = blockIdx.y * zp; K < min(nzc + 1, (int)(blockIdx.y + 1) * zp); ++K) {
    bool live = pl < NYc * NXc;
    if (live && cflag) {
        const int I = pl % NYc, J = pl / NYc;
        bool any = false;
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int a = 0; a < 2; ++a)
                    if (!((a && I == nyc) || (b && J == nxc) || (c && K == nzc)))
                        any |= (cflag[(I + a) + NYc * ((J + b) + NXc * (K + c))] & NF_ACTIVE) != 0;
        live = any;
    }
    if (live) {
        const int I = pl % NYc, J = pl / NYc;
        const int ly = I < nyc ? S : 1, lx = J < nxc ? S : 1, lz = K < nzc ? S : 1;
        T cv[2][2][2][3];   // [c (z)][b (x)][a (y)][component]
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    const bool in = !((a && I == nyc) || (b && J == nxc) || (c && K == nzc));
                    const int m = 3 * ((I + a) + NYc * ((J + b) + NXc * (K + c)));
#pragma unroll
                    for (int q = 0; q < 3; ++q) cv[c][b][a][q] = in ? xc[m + q] : T(0);
                }
        const T inv = T(1) / T(S);
#pragma unroll
        for (int rz = 0; rz < S; ++rz) {
            if (rz >= lz) break;
            const T wz1 = T(rz) * inv, wz0 = T(S - rz) * inv;
            T qz[2][2][3];
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int q = 0; q < 3; ++q) qz[b][a][q] = wz0 * cv[0][b][a][q] + wz1 * cv[1][b][a][q];
#pragma unroll
            for (int rx = 0; rx < S; ++rx) {
                if (rx >= lx) break;
                const T wx1 = T(rx) * inv, wx0 = T(S - rx) * inv;
                T qx[2][3];
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int q = 0; q < 3; ++q) qx[a][q] = wx0 * qz[0][a][q] + wx1 * qz[1][a][q];
                const int rowbase = NYf * ((S * J + rx) + NXf * (S * K + rz)) + S * I;
#pragma unroll
                for (int ry = 0; ry < S; ++ry) {
                    if (ry >= ly) break;
                    const T wy1 = T(ry) * inv, wy0 = T(S - ry) * inv;
                    const int f = rowbase + ry;
                    const uint8_t fl = nflag[f];
                    const bool act = (fl & NF_ACTIVE) != 0;
                    // r and D are loaded whatever the flag says, so that these loads do not
                    // wait for the flag load (one round trip per fine node, not two); what
                    // an inactive node holds is discarded by the selects below
                    T r[3], dg[3], o[3];
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        r[q] = rf[3 * f + q];
                        dg[q] = D[3 * f + q];
                    }
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        const T t = (omega * r[q]) * dg[q];
                        o[q] = act ? (t + (wy0 * qx[0][q] + wy1 * qx[1][q])) + t : T(0);
                    }
                    if (FINAL) {
#pragma unroll
                        for (int q = 0; q < 3; ++q)
                            if (fl & (NF_FIXX << q)) o[q] = T(0);
                        if (act) dot += o[0] * r[0] + o[1] * r[1] + o[2] * r[2];
                    }
                    // inactive nodes of an output that keeps zeros there (cflag set) are not rewritten
                    if (act || !cflag) {
#pragma unroll
                        for (int q = 0; q < 3; ++q) xf[3 * f + q] = o[q];
                    }
                }
            }
        }
    }
    }
    if (FINAL && partial) {
        __shared__ double red[4];
        const double sum = warp_block_sum<T>(dot, red);
        if (threadIdx.x == 0) partial[blockIdx.x + gridDim.x * blockIdx.y] = sum;
    }
}

template <typename T>
void launch_prolong_smooth(const Level &fine, const Level &coarse, const T *xc, const T *rf, const T *diag, T omega,
                           T *xf, bool final_level, double *partial_dot, int *nblocks_out, cudaStream_t st) {
    const bool small = 3 * (int64_t)fine.nnode < (int64_t)INT32_MAX;
    // empty cells are skipped in FP32 only: the FP32 V-cycle's outputs (d_z32 and the
    // levels' x32) are zeroed at allocation, so their inactive nodes hold 0 throughout
    const bool skip_inactive = sizeof(T) == sizeof(float);
    if (small && (coarse.span == 2 || coarse.span == 4)) {
        // 8 (else 4) coarse planes per CTA while that keeps at least 8 CTAs per SM
        const int64_t plane_ctas = ((coarse.ny + 1) * (int64_t)(coarse.nx + 1) + 127) / 128;
        int zp = 8;
        while (zp > 1 && plane_ctas * ((coarse.nz + zp) / zp) < 152 * 8) zp >>= 1;
        const dim3 g((unsigned)plane_ctas, (unsigned)((coarse.nz + zp) / zp));
        if (nblocks_out) *nblocks_out = (int)(g.x * g.y);
        ++g_launches;
#define PCELLS(S, F)                                                                                              \
    k_prolong_cells<T, S, F><<<g, 128, 0, st>>>(xc, rf, diag, fine.nflag, skip_inactive ? coarse.nflag : nullptr, \
                                                omega, xf, coarse.ny, coarse.nx, coarse.nz, zp,                  \
                                                F ? partial_dot : nullptr)
        if (coarse.span == 2) {
            if (final_level)
                PCELLS(2, true);
            else
                PCELLS(2, false);
        } else {
            if (final_level)
                PCELLS(4, true);
            else
                PCELLS(4, false);
        }
#undef PCELLS
        return;
    }
    const dim3 nb((unsigned)(((fine.ny + 1) * (fine.nx + 1) + 255) / 256), (unsigned)(fine.nz + 1));
    if (nblocks_out) *nblocks_out = (int)(nb.x * nb.y);
    ++g_launches;
    if (final_level)
        k_prolong_smooth<T, true><<<nb, 256, 0, st>>>(xc, rf, diag, fine.nflag, omega, xf, coarse.ny, coarse.nx,
                                                      coarse.nz, coarse.span, partial_dot);
    else
        k_prolong_smooth<T, false><<<nb, 256, 0, st>>>(xc, rf, diag, fine.nflag, omega, xf, coarse.ny, coarse.nx,
                                                       coarse.nz, coarse.span, nullptr);
}
template void launch_prolong_smooth<double>(const Level &, const Level &, const double *, const double *,
                                            const double *, double, double *, bool, double *, int *, cudaStream_t);
template void launch_prolong_smooth<float>(const Level &, const Level &, const float *, const float *, const float *,
                                           float, float *, bool, double *, int *, cudaStream_t);

// ---- Jacobi diagonals (src/Solving_AssembleFEAstencil.m:82-121) -------------
// reference corner order j = 1..8 as offsets (dy, dx, dz)
__constant__ int c_cdy[8] = {1, 1, 0, 0, 1, 1, 0, 0};
__constant__ int c_cdx[8] = {0, 1, 1, 0, 0, 1, 1, 0};
__constant__ int c_cdz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
__constant__ double c_dKe[24];

__global__ void k_diag_finest(const double *__restrict__ E, const uint8_t *__restrict__ nflag, int ny, int nx, int nz,
                              double *__restrict__ D) {
    const int NY = ny + 1, NX = nx + 1, NZ = nz + 1;
    const int64_t nn = (int64_t)NY * NX * NZ;
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= nn) return;
    double d0 = 0.0, d1 = 0.0, d2 = 0.0;
    if (nflag[n] & NF_ACTIVE) {
        const int iy = (int)(n % NY), ix = (int)((n / NY) % NX), iz = (int)(n / ((int64_t)NY * NX));
        for (int j = 0; j < 8; ++j) {
            const int ey = iy - c_cdy[j], ex = ix - c_cdx[j], ez = iz - c_cdz[j];
            if (ey < 0 || ex < 0 || ez < 0 || ey >= ny || ex >= nx || ez >= nz) continue;
            const double ev = E[(int64_t)ey + (int64_t)ny * (ex + (int64_t)nx * ez)];
            d0 += c_dKe[3 * j] * ev;
            d1 += c_dKe[3 * j + 1] * ev;
            d2 += c_dKe[3 * j + 2] * ev;
        }
    }
    D[3 * n] = d0;
    D[3 * n + 1] = d1;
    D[3 * n + 2] = d2;
}

void launch_diag_finest(const Level &l0, const double *E, const double *Ke, double *diag, cudaStream_t s) {
    double dk[24];
    for (int i = 0; i < 24; ++i) dk[i] = Ke[i + 24 * i];
    cudaMemcpyToSymbolAsync(c_dKe, dk, sizeof dk, 0, cudaMemcpyHostToDevice, s);
    ++g_launches;
    k_diag_finest<<<(unsigned)((l0.nnode + 255) / 256), 256, 0, s>>>(E, l0.nflag, l0.ny, l0.nx, l0.nz, diag);
}

__global__ void k_diag_from_Ks(const double *__restrict__ Ks, const uint8_t *__restrict__ eact,
                               const uint8_t *__restrict__ nflag, int ny, int nx, int nz, double *__restrict__ D) {
    const int NY = ny + 1, NX = nx + 1, NZ = nz + 1;
    const int64_t nn = (int64_t)NY * NX * NZ;
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= nn) return;
    double d0 = 0.0, d1 = 0.0, d2 = 0.0;
    if (nflag[n] & NF_ACTIVE) {
        const int iy = (int)(n % NY), ix = (int)((n / NY) % NX), iz = (int)(n / ((int64_t)NY * NX));
        for (int j = 0; j < 8; ++j) {
            const int ey = iy - c_cdy[j], ex = ix - c_cdx[j], ez = iz - c_cdz[j];
            if (ey < 0 || ex < 0 || ez < 0 || ey >= ny || ex >= nx || ez >= nz) continue;
            const int64_t e = (int64_t)ey + (int64_t)ny * (ex + (int64_t)nx * ez);
            if (!eact[e]) continue;
            const double *k = Ks + 576 * e;
            d0 += k[(3 * j) * 25];
            d1 += k[(3 * j + 1) * 25];
            d2 += k[(3 * j + 2) * 25];
        }
    }
    D[3 * n] = d0;
    D[3 * n + 1] = d1;
    D[3 * n + 2] = d2;
}

void launch_diag_from_Ks(const Level &l, double *diag, cudaStream_t s) {
    ++g_launches;
    k_diag_from_Ks<<<(unsigned)((l.nnode + 255) / 256), 256, 0, s>>>(l.Ks, l.eact, l.nflag, l.ny, l.nx, l.nz, diag);
}

__global__ void k_inverse_diag(const double *__restrict__ D, const uint8_t *__restrict__ nflag, int64_t nn,
                               double *__restrict__ iD, float *__restrict__ iD32) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= 3 * nn) return;
    const double v = (nflag[i / 3] & NF_ACTIVE) ? 1.0 / D[i] : 0.0;
    iD[i] = v;
    iD32[i] = (float)v;
}

void launch_inverse_diag(const Level &l, cudaStream_t s) {
    ++g_launches;
    k_inverse_diag<<<(unsigned)((3 * l.nnode + 255) / 256), 256, 0, s>>>(l.diag, l.nflag, l.nnode, l.idiag, l.idiag32);
}

// ---- compact <-> full conversions -------------------------------------------
__global__ void k_scatter_nodes(const int64_t *__restrict__ map, int64_t n, const double *__restrict__ src,
                                double *__restrict__ dst) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= 3 * n) return;
    const int64_t node = i / 3;
    const int c = (int)(i - 3 * node);
    dst[3 * map[node] + c] = src[i];
}
__global__ void k_gather_nodes(const int64_t *__restrict__ map, int64_t n, const double *__restrict__ src,
                               double *__restrict__ dst) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= 3 * n) return;
    const int64_t node = i / 3;
    const int c = (int)(i - 3 * node);
    dst[i] = src[3 * map[node] + c];
}
__global__ void k_scatter_elems(const int64_t *__restrict__ map, int64_t n, const double *__restrict__ src,
                                double *__restrict__ dst) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) dst[map[i]] = src[i];
}
__global__ void k_gather_elems(const int64_t *__restrict__ map, int64_t n, const double *__restrict__ src,
                               double *__restrict__ dst) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[map[i]];
}

void launch_scatter_nodes(const int64_t *map, int64_t n, const double *compact, double *full, cudaStream_t s) {
    if (n > 0) {
        ++g_launches;
        k_scatter_nodes<<<(unsigned)((3 * n + 255) / 256), 256, 0, s>>>(map, n, compact, full);
    }
}
void launch_gather_nodes(const int64_t *map, int64_t n, const double *full, double *compact, cudaStream_t s) {
    if (n > 0) {
        ++g_launches;
        k_gather_nodes<<<(unsigned)((3 * n + 255) / 256), 256, 0, s>>>(map, n, full, compact);
    }
}
void launch_scatter_elems(const int64_t *map, int64_t n, const double *compact, double *full, cudaStream_t s) {
    if (n > 0) {
        ++g_launches;
        k_scatter_elems<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(map, n, compact, full);
    }
}
void launch_gather_elems(const int64_t *map, int64_t n, const double *full, double *compact, cudaStream_t s) {
    if (n > 0) {
        ++g_launches;
        k_gather_elems<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(map, n, full, compact);
    }
}

// ---- fixed-DOF bookkeeping (src/FEA_SetupVoxelBased.m:13-26) ----------------
__global__ void k_fixed_indicator(const uint8_t *__restrict__ nflag, int64_t nn, double *__restrict__ v) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const uint8_t f = nflag[n];
    v[3 * n] = (f & NF_FIXX) ? 1.0 : 0.0;
    v[3 * n + 1] = (f & NF_FIXY) ? 1.0 : 0.0;
    v[3 * n + 2] = (f & NF_FIXZ) ? 1.0 : 0.0;
}
void launch_fixed_indicator(const Level &l, double *v, cudaStream_t s) {
    ++g_launches;
    k_fixed_indicator<<<(unsigned)((l.nnode + 255) / 256), 256, 0, s>>>(l.nflag, l.nnode, v);
}
// a coarse DOF is fixed iff the restricted fixed indicator is nonzero
__global__ void k_mark_fixed(uint8_t *__restrict__ nflag, int64_t nn, const double *__restrict__ v) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= nn) return;
    uint8_t f = nflag[n] & NF_ACTIVE;
    if (v[3 * n] != 0.0) f |= NF_FIXX;
    if (v[3 * n + 1] != 0.0) f |= NF_FIXY;
    if (v[3 * n + 2] != 0.0) f |= NF_FIXZ;
    nflag[n] = f;
}
void launch_mark_fixed(Level &l, const double *restricted, cudaStream_t s) {
    ++g_launches;
    k_mark_fixed<<<(unsigned)((l.nnode + 255) / 256), 256, 0, s>>>(l.nflag, l.nnode, restricted);
}

__global__ void k_mask_fixed(const uint8_t *__restrict__ nflag, int64_t nn, double *__restrict__ v) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const uint8_t f = nflag[n];
    if (f & NF_FIXX) v[3 * n] = 0.0;
    if (f & NF_FIXY) v[3 * n + 1] = 0.0;
    if (f & NF_FIXZ) v[3 * n + 2] = 0.0;
}
void launch_mask_fixed(const Level &l0, double *v, cudaStream_t s) {
    ++g_launches;
    k_mask_fixed<<<(unsigned)((l0.nnode + 255) / 256), 256, 0, s>>>(l0.nflag, l0.nnode, v);
}

}  // namespace sgld
