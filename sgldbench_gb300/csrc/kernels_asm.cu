// Galerkin coarse-level assembly and the coarsest-level direct solve
// (reference: src/Solving_AssembleFEAstencil.m:7-135 with
// src/MEXfuncs/Solving_AssembleCmptStencilFromFinestLevel.cpp and
// src/MEXfuncs/Solving_AssembleCmptStencilFromNonFinestLevel.cpp).
//
//  * level 2:  Ks_E = sum_q E_q H_q, H_q = P_q' Ke P_q (templates built on the
//    host, q = child position, s^3 of them);
//  * level l>2: Ks_E = sum_q P_q' Ks_q P_q with P_q = W_q (x) I3, W_q the 8x8
//    trilinear weights of the parent's corners at child q's corners;
//  * coarsest: dense K on the free DOFs (in a bandwidth-reducing order),
//    blocked band Cholesky K = L L' and the explicit triangular inverse
//    M = L^-1, captured once into a CUDA graph; each V-cycle applies
//    K^-1 r = M' (M r) as two dense triangular mat-vecs.  The reference
//    applies its sparse Cholesky factor with two triangular solves
//    (src/Solving_Vcycle.m:116-118); M' M gives the same numbers to rounding
//    and turns two sequential solves into parallel mat-vecs.
#include <math.h>

#include <atomic>
#include <vector>

#include "sgld_internal.cuh"
#include "df_arith.cuh"

namespace sgld {

// Element matrices are symmetric: the kernels form the 300 entries of the
// upper triangle (row <= col) and mirror them.
__constant__ unsigned char c_pr[300], c_pc[300];

// The tables below are the same for every context; each device gets them once.
static std::atomic<bool> g_pairs_done[kMaxDevices], g_weights_done[kMaxDevices];

static int current_device() {
    int dev = 0;
    cudaGetDevice(&dev);
    return dev;
}

void forget_asm_tables(int dev) {
    g_pairs_done[dev] = false;
    g_weights_done[dev] = false;
}

static void upload_pairs(cudaStream_t s) {
    std::atomic<bool> &done = g_pairs_done[current_device()];
    if (done) return;
    unsigned char pr[300], pc[300];
    int k = 0;
    for (int col = 0; col < 24; ++col)
        for (int row = 0; row <= col; ++row) {
            pr[k] = (unsigned char)row;
            pc[k] = (unsigned char)col;
            ++k;
        }
    cudaMemcpyToSymbolAsync(c_pr, pr, sizeof pr, 0, cudaMemcpyHostToDevice, s);
    cudaMemcpyToSymbolAsync(c_pc, pc, sizeof pc, 0, cudaMemcpyHostToDevice, s);
    done = true;
}

// ---- coarse element matrices straight from the finest level ------------------
// Ks_E = sum_q E_q H_q over the S^3 finest elements q inside coarse element E,
// with templates H_q = P_q' Ke P_q (P_q: trilinear interpolation from E's
// corners to q's corners; span S = 2 or 4).  Composed trilinear
// interpolation is trilinear, so S = 4 gives the same matrices as two
// Galerkin steps of span 2.  A CTA handles EB consecutive coarse elements;
// thread t owns one upper-triangle entry and keeps EB accumulators.
constexpr int EB = 16;

// The sums run in compensated double-float arithmetic (Dot2 accumulators, at
// the FP32 issue rate): in FP64 the kernel was bound by GB300's FP64 pipe
// (ncu: 99 % busy).  H2 holds the templates as (hi, lo) float pairs; E is
// split on load.
template <int NQ>
__global__ void __launch_bounds__(320) k_asm_templates_df(const double *__restrict__ E,
                                                          const uint8_t *__restrict__ eact_c,
                                                          const float2 *__restrict__ H2, int nyc, int nxc, int nzc,
                                                          double *__restrict__ Ks) {
    constexpr int S = (NQ == 8) ? 2 : 4;
    __shared__ float2 ev[EB][NQ];
    const int64_t nel = (int64_t)nyc * nxc * nzc;
    const int64_t e0 = (int64_t)blockIdx.x * EB;
    const int nyf = S * nyc, nxf = S * nxc;
    for (int idx = threadIdx.x; idx < EB * NQ; idx += blockDim.x) {
        const int k = idx / NQ, q = idx % NQ;
        const int64_t e = e0 + k;
        double v = 0.0;
        if (e < nel && eact_c[e]) {
            const int cy = (int)(e % nyc), cx = (int)((e / nyc) % nxc), cz = (int)(e / ((int64_t)nyc * nxc));
            const int oy = q % S, ox = (q / S) % S, oz = q / (S * S);
            v = E[(int64_t)(S * cy + oy) + (int64_t)nyf * ((S * cx + ox) + (int64_t)nxf * (S * cz + oz))];
        }
        const df d = df_from(v);
        ev[k][q] = make_float2(d.hi, d.lo);
    }
    __syncthreads();
    const int t = threadIdx.x;
    if (t >= 300) return;
    const int r = c_pr[t], c = c_pc[t];
    const int off = r + 24 * c, offt = c + 24 * r;
    dacc acc[EB];
    for (int q = 0; q < NQ; ++q) {
        const float2 h = H2[576 * q + off];
#pragma unroll
        for (int k = 0; k < EB; ++k) acc[k].add(ev[k][q], h);
    }
#pragma unroll
    for (int k = 0; k < EB; ++k) {
        const int64_t e = e0 + k;
        if (e < nel && eact_c[e]) {
            const double v = df_to(acc[k].value());
            Ks[576 * e + off] = v;
            Ks[576 * e + offt] = v;
        }
    }
}

void launch_asm_templates(const Level &coarse, int S, const double *E, const double *H, double *Ks, cudaStream_t s) {
    upload_pairs(s);
    const unsigned nb = (unsigned)((coarse.nel + EB - 1) / EB);
    ++g_launches;
    // the float-pair copy of every template sits (8 + 64) * 576 entries after
    // its FP64 form (setup_templates lays out FP64 span 2, span 4, then the pairs)
    const float2 *H2 = reinterpret_cast<const float2 *>(H + 72 * 576);
    if (S == 2)
        k_asm_templates_df<8><<<nb, 320, 0, s>>>(E, coarse.eact, H2, coarse.ny, coarse.nx, coarse.nz, Ks);
    else
        k_asm_templates_df<64><<<nb, 320, 0, s>>>(E, coarse.eact, H2, coarse.ny, coarse.nx, coarse.nz, Ks);
}

// Jacobi diagonal of a span-2 coarse level without its element matrices:
// diag(N, c) = sum_{coarse elements e around N} sum_q E_q H_q[(3j+c),(3j+c)]
// with j the corner of e at N.
__global__ void k_diag_templates(const double *__restrict__ E, const uint8_t *__restrict__ nflag,
                                 const double *__restrict__ H, int ny, int nx, int nz, double *__restrict__ D) {
    const int NY = ny + 1, NX = nx + 1;
    const int pl = blockIdx.x * blockDim.x + threadIdx.x;
    if (pl >= NY * NX) return;
    const int iy = pl % NY, ix = pl / NY, iz = blockIdx.y;
    const int64_t n = (int64_t)pl + (int64_t)NY * NX * iz;
    double d0 = 0.0, d1 = 0.0, d2 = 0.0;
    if (nflag[n] & NF_ACTIVE) {
        const int cdy[8] = {1, 1, 0, 0, 1, 1, 0, 0}, cdx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cdz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
        const int nyf = 2 * ny, nxf = 2 * nx;
        for (int j = 0; j < 8; ++j) {
            const int ey = iy - cdy[j], ex = ix - cdx[j], ez = iz - cdz[j];
            if (ey < 0 || ex < 0 || ez < 0 || ey >= ny || ex >= nx || ez >= nz) continue;
            for (int q = 0; q < 8; ++q) {
                const int oy = q & 1, ox = (q >> 1) & 1, oz = q >> 2;
                const double ev = E[(int64_t)(2 * ey + oy) + (int64_t)nyf * ((2 * ex + ox) + (int64_t)nxf * (2 * ez + oz))];
                if (ev == 0.0) continue;
                const double *h = H + 576 * q;
                d0 += ev * h[(3 * j) * 25];
                d1 += ev * h[(3 * j + 1) * 25];
                d2 += ev * h[(3 * j + 2) * 25];
            }
        }
    }
    D[3 * n] = d0;
    D[3 * n + 1] = d1;
    D[3 * n + 2] = d2;
}

void launch_diag_templates(const Level &coarse, const double *E, const double *H2, double *diag, cudaStream_t s) {
    const dim3 g((unsigned)(((coarse.ny + 1) * (coarse.nx + 1) + 255) / 256), (unsigned)(coarse.nz + 1));
    ++g_launches;
    k_diag_templates<<<g, 256, 0, s>>>(E, coarse.nflag, H2, coarse.ny, coarse.nx, coarse.nz, diag);
}

// ---- deeper levels: P_q' Ks_q P_q ---------------------------------------------
// W_q[i][a] = trilinear weight of parent corner a at child q's corner i
// (span 2, reference corner order, child q = oy + 2 ox + 4 oz).  Only 27 of
// its 64 entries are nonzero; the kernel walks the nonzeros of each column.
__constant__ unsigned char c_wn[8][8];      // nonzeros in column a of W_q
__constant__ unsigned char c_wi[8][8][8];   // their row indices i
__constant__ double c_ww[8][8][8];          // and weights

__global__ void __launch_bounds__(320) k_asm_coarse(const double *__restrict__ Kf, const uint8_t *__restrict__ eact_f,
                                                    const uint8_t *__restrict__ eact_c, int nyc, int nxc, int nzc,
                                                    double *__restrict__ Ks) {
    const int64_t e = blockIdx.x + (int64_t)gridDim.x * blockIdx.y;
    const int64_t nel = (int64_t)nyc * nxc * nzc;
    if (e >= nel || !eact_c[e]) return;
    __shared__ double sk[576], st[576];
    const int cy = (int)(e % nyc), cx = (int)((e / nyc) % nxc), cz = (int)(e / ((int64_t)nyc * nxc));
    const int nyf = 2 * nyc, nxf = 2 * nxc;
    const int t = threadIdx.x;
    double acc = 0.0;
    for (int q = 0; q < 8; ++q) {
        const int oy = q & 1, ox = (q >> 1) & 1, oz = q >> 2;
        const int64_t f = (int64_t)(2 * cy + oy) + (int64_t)nyf * ((2 * cx + ox) + (int64_t)nxf * (2 * cz + oz));
        if (!eact_f[f]) continue;   // uniform per CTA
        const double *src = Kf + 576 * f;
        for (int i = t; i < 576; i += blockDim.x) sk[i] = src[i];
        __syncthreads();
        // st[r + 24*(3a+d)] = sum_i sk[r + 24*(3i+d)] W[i][a]
        for (int idx = t; idx < 576; idx += blockDim.x) {
            const int r = idx % 24, col = idx / 24, a = col / 3, d = col % 3;
            double v = 0.0;
            const int nz = c_wn[q][a];
            for (int k = 0; k < nz; ++k) v += sk[r + 24 * (3 * c_wi[q][a][k] + d)] * c_ww[q][a][k];
            st[idx] = v;
        }
        __syncthreads();
        // upper triangle of W' st: out[(3b+e), col] = sum_j W[j][b] st[(3j+e) + 24 col]
        if (t < 300) {
            const int row = c_pr[t], col = c_pc[t], b = row / 3, ec = row % 3;
            double v = 0.0;
            const int nz = c_wn[q][b];
            for (int k = 0; k < nz; ++k) v += c_ww[q][b][k] * st[(3 * c_wi[q][b][k] + ec) + 24 * col];
            acc += v;
        }
        __syncthreads();
    }
    if (t < 300) {
        double *o = Ks + 576 * e;
        o[c_pr[t] + 24 * c_pc[t]] = acc;
        o[c_pc[t] + 24 * c_pr[t]] = acc;
    }
}

void launch_asm_coarse(const Level &coarse, const Level &fine, double *Ks, cudaStream_t s) {
    std::atomic<bool> &uploaded = g_weights_done[current_device()];
    upload_pairs(s);
    if (!uploaded) {
        const int cdy[8] = {1, 1, 0, 0, 1, 1, 0, 0}, cdx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cdz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
        unsigned char wn[8][8] = {}, wi[8][8][8] = {};
        double ww[8][8][8] = {};
        for (int q = 0; q < 8; ++q) {
            const int oy = q & 1, ox = (q >> 1) & 1, oz = q >> 2;
            for (int i = 0; i < 8; ++i) {
                // child corner position in parent units: natural coordinates
                const double sn = -1.0 + (ox + cdx[i]), tn = 1.0 - (oy + cdy[i]), pn = -1.0 + (oz + cdz[i]);
                const double N[8] = {(1 - sn) * (1 - tn) * (1 - pn), (1 + sn) * (1 - tn) * (1 - pn),
                                     (1 + sn) * (1 + tn) * (1 - pn), (1 - sn) * (1 + tn) * (1 - pn),
                                     (1 - sn) * (1 - tn) * (1 + pn), (1 + sn) * (1 - tn) * (1 + pn),
                                     (1 + sn) * (1 + tn) * (1 + pn), (1 - sn) * (1 + tn) * (1 + pn)};
                for (int a = 0; a < 8; ++a) {
                    const double w = 0.125 * N[a];
                    if (w != 0.0) {
                        const int k = wn[q][a]++;
                        wi[q][a][k] = (unsigned char)i;
                        ww[q][a][k] = w;
                    }
                }
            }
        }
        cudaMemcpyToSymbolAsync(c_wn, wn, sizeof wn, 0, cudaMemcpyHostToDevice, s);
        cudaMemcpyToSymbolAsync(c_wi, wi, sizeof wi, 0, cudaMemcpyHostToDevice, s);
        cudaMemcpyToSymbolAsync(c_ww, ww, sizeof ww, 0, cudaMemcpyHostToDevice, s);
        uploaded = true;
    }
    const int64_t nel = coarse.nel;
    const unsigned gx = (unsigned)(nel < 65535 ? nel : 65535);
    const unsigned gy = (unsigned)((nel + gx - 1) / gx);
    ++g_launches;
    k_asm_coarse<<<dim3(gx, gy), 320, 0, s>>>(fine.Ks, fine.eact, coarse.eact, coarse.ny, coarse.nx, coarse.nz, Ks);
}

// ---- coarsest level: dense matrix on the free DOFs ---------------------------
__constant__ int c_ady[8] = {1, 1, 0, 0, 1, 1, 0, 0};
__constant__ int c_adx[8] = {0, 1, 1, 0, 0, 1, 1, 0};
__constant__ int c_adz[8] = {0, 0, 0, 0, 1, 1, 1, 1};

// pos[dof] = row of that DOF in the dense matrix or -1; rows[i] = full DOF of row i
__global__ void k_coarse_dense(const double *__restrict__ Ks, const uint8_t *__restrict__ eact, int ny, int nx, int nz,
                               const int *__restrict__ rows, const int *__restrict__ pos, int ncf, double *__restrict__ A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncf) return;
    const int NY = ny + 1, NX = nx + 1;
    const int dof = rows[i];
    const int node = dof / 3, c = dof % 3;
    const int iy = node % NY, ix = (node / NY) % NX, iz = node / (NY * NX);
    for (int j = 0; j < 8; ++j) {
        const int ey = iy - c_ady[j], ex = ix - c_adx[j], ez = iz - c_adz[j];
        if (ey < 0 || ex < 0 || ez < 0 || ey >= ny || ex >= nx || ez >= nz) continue;
        const int64_t e = (int64_t)ey + (int64_t)ny * (ex + (int64_t)nx * ez);
        if (!eact[e]) continue;
        const double *k = Ks + 576 * e;
        for (int kk = 0; kk < 8; ++kk) {
            const int m = (ey + c_ady[kk]) + NY * ((ex + c_adx[kk]) + NX * (ez + c_adz[kk]));
            for (int d = 0; d < 3; ++d) {
                const int p = pos[3 * m + d];
                if (p < 0) continue;
                A[(int64_t)i + (int64_t)ncf * p] += k[(3 * j + c) + 24 * (3 * kk + d)];
            }
        }
    }
}

void launch_coarse_dense(const Level &lc, int ncf, const int *rows_and_pos, double *A, cudaStream_t s) {
    const int *rows = rows_and_pos;
    const int *pos = rows_and_pos + ncf;
    if (ncf == 0) return;   // every coarsest DOF fixed: nothing to factor
    cudaMemsetAsync(A, 0, sizeof(double) * (size_t)ncf * ncf, s);
    ++g_launches;
    k_coarse_dense<<<(ncf + 127) / 128, 128, 0, s>>>(lc.Ks, lc.eact, lc.ny, lc.nx, lc.nz, rows, pos, ncf, A);
}

// ---- blocked band Cholesky, NB x NB tiles, column-major n x n ------------------
constexpr int NB = 32;

// 1/sqrt(d) in double-float: FP32 seed, two Newton steps y += y (1 - d y^2) / 2
__device__ __forceinline__ df df_rsqrt(df d) {
    df y = {rsqrtf(d.hi), 0.f};
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const df h = df_sub({1.f, 0.f}, df_mul(df_mul(d, y), y));
        y = df_add(y, df_mul(df_mul(y, {0.5f, 0.f}), h));
    }
    return y;
}

// One block column of the band Cholesky (4 warps per CTA), in double-float
// arithmetic: GB300's FP64 pipe would serialise the pivot chain (a warp-wide
// FP64 instruction occupies its sub-partition for many cycles).  The matrix
// stays FP64 in memory; tiles are split into (hi, lo) on load.
//   * every CTA factors the 32 x 32 diagonal tile in shared memory (row = lane,
//     the rank-1 update of step j split over the 4 warps by column mod 4; the
//     pivot 1/sqrt(d) is formed by every thread, so it needs no broadcast);
//   * CTA 0 writes the factored tile back;
//   * CTA b > 0 solves CP_RS rows of the band below against it (X = A L^-T):
//     16 lanes per row, two columns per lane in registers, x_q broadcast by a
//     16-wide shuffle.
constexpr int CP_THREADS = 128;
constexpr int CP_RS = 8;

__global__ void __launch_bounds__(CP_THREADS) k_chol_panel(double *A, int n, int k0, int rend, int *info) {
    __shared__ df T[NB][NB + 1];
    __shared__ df rd[NB], ld[NB];
    const int t = threadIdx.x, r = t & 31, w = t >> 5;
    const int m = min(NB, n - k0);
    for (int idx = t; idx < NB * NB; idx += CP_THREADS) {
        const int rr = idx & 31, cc = idx >> 5;
        T[rr][cc] = (rr < m && cc < m && cc <= rr) ? df_from(A[(int64_t)(k0 + rr) + (int64_t)n * (k0 + cc)])
                                                   : df{rr == cc ? 1.f : 0.f, 0.f};
    }
    __syncthreads();
    for (int j = 0; j < NB; ++j) {
        // T[j][j] is read here and never written in the loop (the factor's
        // diagonal goes to ld[]), so no thread can overwrite it early
        df d = T[j][j];
        const bool bad = !(d.hi > 0.f);
        if (bad) d = {1.f, 0.f};
        const df y = df_rsqrt(d);
        if (w == 0 && r > j) T[r][j] = df_mul(T[r][j], y);
        if (t == 0) {
            rd[j] = y;
            ld[j] = df_mul(d, y);
            if (bad && blockIdx.x == 0 && info) atomicExch(info, k0 + j + 1);
        }
        __syncthreads();
        if (r > j) {
            const df lrj = T[r][j];
            for (int q = j + 1 + ((w - j - 1) & 3); q <= r; q += 4) T[r][q] = df_sub(T[r][q], df_mul(lrj, T[q][j]));
        }
        __syncthreads();
    }
    if (blockIdx.x == 0) {
        for (int idx = t; idx < NB * NB; idx += CP_THREADS) {
            const int rr = idx & 31, cc = idx >> 5;
            if (rr < m && cc < m)
                A[(int64_t)(k0 + rr) + (int64_t)n * (k0 + cc)] =
                    rr > cc ? df_to(T[rr][cc]) : (rr == cc ? df_to(ld[rr]) : 0.0);
        }
        return;
    }
    const int rr = t >> 4, g = t & 15;
    const int row = k0 + NB + (blockIdx.x - 1) * CP_RS + rr;
    const bool live = row < rend;
    df a0 = {0.f, 0.f}, a1 = {0.f, 0.f};
    if (live) {
        if (g < m) a0 = df_from(A[(int64_t)row + (int64_t)n * (k0 + g)]);
        if (g + 16 < m) a1 = df_from(A[(int64_t)row + (int64_t)n * (k0 + g + 16)]);
    }
#pragma unroll 4
    for (int q = 0; q < NB; ++q) {
        const df xq = df_shfl(df_mul(q < 16 ? a0 : a1, rd[q]), q & 15, 16);
        if (g == (q & 15)) {
            if (q < 16)
                a0 = xq;
            else
                a1 = xq;
        }
        if (g > q) a0 = df_sub(a0, df_mul(xq, T[g][q]));
        if (g + 16 > q) a1 = df_sub(a1, df_mul(xq, T[g + 16][q]));
    }
    if (live) {
        if (g < m) A[(int64_t)row + (int64_t)n * (k0 + g)] = df_to(a0);
        if (g + 16 < m) A[(int64_t)row + (int64_t)n * (k0 + g + 16)] = df_to(a1);
    }
}


// trailing update A[i,j] -= sum_k A[i,k] A[j,k] over the panel's columns k for
// the band tiles below it: blockIdx.x = tile pair (ii >= jj), blockIdx.y =
// SY_RS-row slice of tile ii (slices spread one pair's work over SMs).  The
// products are summed in double-float; A stays FP64.
constexpr int SY_RS = 8;

__global__ void __launch_bounds__(256) k_syrk_update(double *A, int n, int k0, int jb0, int nbt) {
    int p = blockIdx.x, ii = 0;
    while (p > ii) {
        p -= ii + 1;
        ++ii;
    }
    const int jj = p;
    const int i0 = (jb0 + ii) * NB + blockIdx.y * SY_RS, j0 = (jb0 + jj) * NB;
    __shared__ float2 Ai[SY_RS][NB + 1], Aj[NB][NB + 1];
    const int t = threadIdx.x;
    const int m = min(NB, n - k0);
    for (int idx = t; idx < NB * NB; idx += 256) {
        const int r = idx & 31, c = idx >> 5;
        const df v = df_from((j0 + r < n && c < m) ? A[(int64_t)(j0 + r) + (int64_t)n * (k0 + c)] : 0.0);
        Aj[r][c] = make_float2(v.hi, v.lo);
    }
    {
        const int r = t & (SY_RS - 1), c = t / SY_RS;
        const df v = df_from((i0 + r < n && c < m) ? A[(int64_t)(i0 + r) + (int64_t)n * (k0 + c)] : 0.0);
        Ai[r][c] = make_float2(v.hi, v.lo);
    }
    __syncthreads();
    const int r = t & (SY_RS - 1), c = t / SY_RS;
    const int gi = i0 + r, gj = j0 + c;
    if (gi >= n || gj >= n || gj > gi) return;
    dacc v;
#pragma unroll
    for (int q = 0; q < NB; ++q) v.add(Ai[r][q], Aj[c][q]);
    A[(int64_t)gi + (int64_t)n * gj] -= df_to(v.value());
}

// Band of L by columns in double-float form: LB[k*(b+1) + j] = L[k+j, k]
// (j = 0..b, zero past n), so that the rows of one column are contiguous;
// rd[i] = 1 / L[i,i].
__global__ void k_band_cols(const double *__restrict__ L, int n, int b, float2 *__restrict__ LB,
                            float2 *__restrict__ rd) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < n) {
        const df r = df_from(1.0 / L[t + (int64_t)n * t]);
        rd[t] = make_float2(r.hi, r.lo);
    }
    if (t >= (int64_t)n * (b + 1)) return;
    const int k = (int)(t / (b + 1)), j = (int)(t % (b + 1));
    const df v = df_from(k + j < n ? L[(int64_t)(k + j) + (int64_t)n * k] : 0.0);
    LB[t] = make_float2(v.hi, v.lo);
}

__device__ __forceinline__ float2 band_at(const float2 *__restrict__ LB, int b, int i, int k) {
    return LB[(int64_t)k * (b + 1) + (i - k)];   // requires 0 <= i - k <= b
}

// Inverses of the aligned 32 x 32 diagonal blocks of L (double-float),
// column-major per block: D[kb*1024 + t*32 + r] = (L_kb^-1)[r, t].  One warp
// per block, lane t forms column t by forward substitution (rows past n are
// treated as identity rows).
__global__ void __launch_bounds__(32) k_block_inverse(const float2 *__restrict__ LB, const float2 *__restrict__ rd,
                                                      int n, int b, float2 *__restrict__ D) {
    __shared__ float2 Ls[32][33];   // L_kb[r][k], k < r
    __shared__ float2 X[32][33];    // X[r][t] = column t of the inverse
    const int t = threadIdx.x, i0 = blockIdx.x * 32;
    for (int r = 0; r < 32; ++r) {
        const int i = i0 + r, k = i0 + t;
        Ls[r][t] = (t < r && i < n && i - k <= b) ? band_at(LB, b, i, k) : make_float2(0.f, 0.f);
    }
    __syncwarp();
    auto rdiag = [&](int r) -> df {
        const int i = i0 + r;
        return i < n ? df{rd[i].x, rd[i].y} : df{1.f, 0.f};
    };
    for (int r = 0; r < 32; ++r) {
        df x = {0.f, 0.f};
        if (r == t) {
            x = rdiag(r);
        } else if (r > t) {
            df s = {0.f, 0.f};
            for (int k = t; k < r; ++k) s = df_add(s, df_mul({Ls[r][k].x, Ls[r][k].y}, {X[k][t].x, X[k][t].y}));
            x = df_mul(df_neg(s), rdiag(r));
        }
        X[r][t] = make_float2(x.hi, x.lo);
    }
    __syncwarp();
    for (int tt = 0; tt < 32; ++tt) D[(int64_t)blockIdx.x * 1024 + tt * 32 + t] = X[t][tt];
}

// M = L^-1 in double-float arithmetic, a CTA per group of TI_G columns
// c0..c0+TI_G-1 walking down aligned 32-row blocks i0 (GB300's FP64 issue
// rate would bound the n^2 b / 2 multiply-adds):
//   1. S = L[i0:i0+32, i0-b:i0] * M[i0-b:i0, group]: the band tile is staged
//      in shared memory by TI_KC-column chunks, the group's earlier rows of M
//      sit in a shared ring of R >= b + 32 rows; thread (row r = lane, column
//      pair of its warp) accumulates two entries with no masking (the band
//      tile and the ring hold zeros where L or M vanish);
//   2. M[i0:i0+32, group] = D_blk (E - S) with the block's precomputed
//      inverse, E the identity columns of the group.
// Writes M in FP64 (hi + lo) and in FP32 (the FP32 V-cycle's copy).
// A group is TI_G = 16 columns (8 warps) when the ring fits in shared memory,
// else 8, 4 or 2 (wide coarsest bands, e.g. the reference's default hierarchy).
constexpr int TI_KC = 64;

template <int TI_G>
__global__ void __launch_bounds__(16 * TI_G) k_trinv_tiles(const float2 *__restrict__ LB,
                                                           const float2 *__restrict__ D, int n, int b, int R,
                                                           double *__restrict__ M, float *__restrict__ M32) {
    constexpr int TI_THREADS = 16 * TI_G;
    extern __shared__ float2 tsm[];
    float2 *ring = tsm;                       // [R][TI_G]
    float2 *Lt = ring + (int64_t)R * TI_G;    // [32][TI_KC + 1]
    float2 *rhs = Lt + 32 * (TI_KC + 1);      // [32][TI_G]
    const int t = threadIdx.x, r = t & 31, gp = (t >> 5) * 2;
    const int c0 = blockIdx.x * TI_G;
    for (int idx = t; idx < R * TI_G; idx += TI_THREADS) ring[idx] = make_float2(0.f, 0.f);
    __syncthreads();
    for (int i0 = c0 & ~31; i0 < n; i0 += 32) {
        dacc a0, a1;
        const int kbeg = max(0, i0 - b);
        for (int kc = kbeg; kc < i0; kc += TI_KC) {
            const int kn = min(TI_KC, i0 - kc);
            for (int idx = t; idx < 32 * TI_KC; idx += TI_THREADS) {
                const int rr = idx & 31, kk = idx >> 5, i = i0 + rr, k = kc + kk;
                Lt[rr * (TI_KC + 1) + kk] =
                    (kk < kn && i < n && i - k <= b) ? band_at(LB, b, i, k) : make_float2(0.f, 0.f);
            }
            __syncthreads();
#pragma unroll 4
            for (int kk = 0; kk < kn; ++kk) {
                const float2 l = Lt[r * (TI_KC + 1) + kk];
                const float2 *m = ring + (int64_t)((kc + kk) & (R - 1)) * TI_G + gp;
                a0.add(l, m[0]);
                a1.add(l, m[1]);
            }
            __syncthreads();
        }
        const int i = i0 + r;
        {
            df e0 = df_neg(a0.value()), e1 = df_neg(a1.value());
            if (i == c0 + gp) e0 = df_add(e0, {1.f, 0.f});
            if (i == c0 + gp + 1) e1 = df_add(e1, {1.f, 0.f});
            rhs[r * TI_G + gp] = make_float2(e0.hi, e0.lo);
            rhs[r * TI_G + gp + 1] = make_float2(e1.hi, e1.lo);
        }
        __syncthreads();
        dacc v0, v1;
        const float2 *dblk = D + (int64_t)(i0 >> 5) * 1024 + r;
#pragma unroll 8
        for (int q = 0; q < 32; ++q) {
            const float2 d = q <= r ? dblk[q * 32] : make_float2(0.f, 0.f);
            v0.add(d, rhs[q * TI_G + gp]);
            v1.add(d, rhs[q * TI_G + gp + 1]);
        }
        const df x0 = v0.value(), x1 = v1.value();
        float2 *slot = ring + (int64_t)(i & (R - 1)) * TI_G + gp;
        // rows above a column's start come out as exact zeros
        slot[0] = make_float2(x0.hi, x0.lo);
        slot[1] = make_float2(x1.hi, x1.lo);
        if (i < n) {
            const int ca = c0 + gp, cb = ca + 1;
            if (ca < n && i >= ca) {
                M[(int64_t)i + (int64_t)n * ca] = df_to(x0);
                if (M32) M32[(int64_t)i + (int64_t)n * ca] = x0.hi;
            }
            if (cb < n && i >= cb) {
                M[(int64_t)i + (int64_t)n * cb] = df_to(x1);
                if (M32) M32[(int64_t)i + (int64_t)n * cb] = x1.hi;
            }
        }
        // the transpose into the upper triangle (M^T, column-major), staged
        // through shared memory so that the stores run along the group's columns
        __syncthreads();
        rhs[r * TI_G + gp] = make_float2(x0.hi, x0.lo);
        rhs[r * TI_G + gp + 1] = make_float2(x1.hi, x1.lo);
        __syncthreads();
        for (int idx = t; idx < 32 * TI_G; idx += TI_THREADS) {
            const int g = idx % TI_G, rr = idx / TI_G;
            const int cc = c0 + g, ii = i0 + rr;
            if (ii < n && cc < n && ii > cc) {
                const float2 v = rhs[rr * TI_G + g];
                M[(int64_t)cc + (int64_t)n * ii] = (double)v.x + (double)v.y;
                if (M32) M32[(int64_t)cc + (int64_t)n * ii] = v.x;
            }
        }
        __syncthreads();
    }
}

size_t trinv_smem_bytes(int R, int G) { return sizeof(float2) * ((size_t)R * G + 32 * (TI_KC + 1) + 32 * G); }

// The same column sweep in FP32 (the hi words of the double-float band and
// block inverses, FP32 FMA accumulation), writing only the FP32 copy M32 that
// the FP32 V-cycle of the mixed-precision solves applies.  Its rounding error
// only perturbs that preconditioner: the coarse apply M32' (M32 r) stays
// symmetric positive semi-definite for any M32, and the outer solve still
// converges on the FP64 residual.
template <int TI_G>
__global__ void __launch_bounds__(16 * TI_G) k_trinv_tiles32(const float2 *__restrict__ LB,
                                                             const float2 *__restrict__ D, int n, int b, int R,
                                                             float *__restrict__ M32) {
    constexpr int TI_THREADS = 16 * TI_G;
    extern __shared__ float tsm32[];
    float *ring = tsm32;                      // [R][TI_G]
    float *Lt = ring + (int64_t)R * TI_G;     // [32][TI_KC + 1]
    float *rhs = Lt + 32 * (TI_KC + 1);       // [32][TI_G]
    const int t = threadIdx.x, r = t & 31, gp = (t >> 5) * 2;
    const int c0 = blockIdx.x * TI_G;
    for (int idx = t; idx < R * TI_G; idx += TI_THREADS) ring[idx] = 0.f;
    __syncthreads();
    for (int i0 = c0 & ~31; i0 < n; i0 += 32) {
        float a0 = 0.f, a1 = 0.f;
        const int kbeg = max(0, i0 - b);
        for (int kc = kbeg; kc < i0; kc += TI_KC) {
            const int kn = min(TI_KC, i0 - kc);
            for (int idx = t; idx < 32 * TI_KC; idx += TI_THREADS) {
                const int rr = idx & 31, kk = idx >> 5, i = i0 + rr, k = kc + kk;
                Lt[rr * (TI_KC + 1) + kk] = (kk < kn && i < n && i - k <= b) ? band_at(LB, b, i, k).x : 0.f;
            }
            __syncthreads();
#pragma unroll 8
            for (int kk = 0; kk < kn; ++kk) {
                const float l = Lt[r * (TI_KC + 1) + kk];
                const float2 m = *reinterpret_cast<const float2 *>(ring + (int64_t)((kc + kk) & (R - 1)) * TI_G + gp);
                a0 = fmaf(l, m.x, a0);
                a1 = fmaf(l, m.y, a1);
            }
            __syncthreads();
        }
        const int i = i0 + r;
        {
            float e0 = -a0, e1 = -a1;
            if (i == c0 + gp) e0 += 1.f;
            if (i == c0 + gp + 1) e1 += 1.f;
            rhs[r * TI_G + gp] = e0;
            rhs[r * TI_G + gp + 1] = e1;
        }
        __syncthreads();
        float x0 = 0.f, x1 = 0.f;
        const float2 *dblk = D + (int64_t)(i0 >> 5) * 1024 + r;
#pragma unroll 8
        for (int q = 0; q < 32; ++q) {
            const float d = q <= r ? dblk[q * 32].x : 0.f;
            x0 = fmaf(d, rhs[q * TI_G + gp], x0);
            x1 = fmaf(d, rhs[q * TI_G + gp + 1], x1);
        }
        float *slot = ring + (int64_t)(i & (R - 1)) * TI_G + gp;
        slot[0] = x0;
        slot[1] = x1;
        if (i < n) {
            const int ca = c0 + gp, cb = ca + 1;
            if (ca < n && i >= ca) M32[(int64_t)i + (int64_t)n * ca] = x0;
            if (cb < n && i >= cb) M32[(int64_t)i + (int64_t)n * cb] = x1;
        }
        __syncthreads();
        rhs[r * TI_G + gp] = x0;
        rhs[r * TI_G + gp + 1] = x1;
        __syncthreads();
        for (int idx = t; idx < 32 * TI_G; idx += TI_THREADS) {
            const int g = idx % TI_G, rr = idx / TI_G;
            const int cc = c0 + g, ii = i0 + rr;
            if (ii < n && cc < n && ii > cc) M32[(int64_t)cc + (int64_t)n * ii] = rhs[rr * TI_G + g];
        }
        __syncthreads();
    }
}

size_t trinv32_smem_bytes(int R, int G) { return sizeof(float) * ((size_t)R * G + 32 * (TI_KC + 1) + 32 * G); }

// launches of the two sweeps for the context's column-group width
template <int G>
static void trinv32_launch(const Ctx &c, const float2 *LB, const float2 *D, int n, int b) {
    k_trinv_tiles32<G><<<(n + G - 1) / G, 16 * G, trinv32_smem_bytes(c.trinv_ring, G), c.stream>>>(
        LB, D, n, b, c.trinv_ring, c.d_Ainv32);
}
template <int G>
static void trinv64_launch(const Ctx &c, const float2 *LB, const float2 *D, int n, int b) {
    k_trinv_tiles<G><<<(n + G - 1) / G, 16 * G, trinv_smem_bytes(c.trinv_ring, G), c.stream>>>(
        LB, D, n, b, c.trinv_ring, c.d_Ainv, nullptr);
}
template <int G>
static void trinv_attributes(int R) {
    cudaFuncSetAttribute(k_trinv_tiles<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)trinv_smem_bytes(R, G));
    cudaFuncSetAttribute(k_trinv_tiles32<G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)trinv32_smem_bytes(R, G));
}

// Enqueues the whole factorization (band Cholesky, L^-1, FP32 copy); no host
// synchronisation, so the sequence is captured once into a CUDA graph.
static void factor_enqueue(Ctx &c, int *d_info) {
    const int n = c.ncf;
    const int nblk = (n + NB - 1) / NB;
    const int bw = (c.cband + NB - 1) / NB + 1;   // band in tiles (safety margin of one)
    double *A = c.d_Ac;
    cudaMemsetAsync(d_info, 0, sizeof(int), c.stream);
    for (int kb = 0; kb < nblk; ++kb) {
        const int k0 = kb * NB;
        const int kend = min(nblk - 1, kb + bw);
        const int nbelow = kend - kb;
        const int rend = min(n, (kend + 1) * NB);
        const int ntrsm = rend > k0 + NB ? (rend - k0 - NB + CP_RS - 1) / CP_RS : 0;
        ++g_launches;
        k_chol_panel<<<1 + ntrsm, CP_THREADS, 0, c.stream>>>(A, n, k0, rend, d_info);
        if (nbelow > 0) {
            const int npairs = nbelow * (nbelow + 1) / 2;
            ++g_launches;
            k_syrk_update<<<dim3(npairs, NB / SY_RS), 256, 0, c.stream>>>(A, n, k0, kb + 1, nbelow);
        }
    }
    const int b = c.cband;
    // d_LB (n (b+1) + n + nblk 1024 doubles) holds, as float pairs, the band
    // by columns, 1/diag and the diagonal-block inverses
    float2 *LB = reinterpret_cast<float2 *>(c.d_LB), *rd = LB + (int64_t)n * (b + 1), *D = rd + n;
    ++g_launches;
    k_band_cols<<<(unsigned)(((int64_t)n * (b + 1) + 255) / 256), 256, 0, c.stream>>>(A, n, b, LB, rd);
    ++g_launches;
    k_block_inverse<<<nblk, 32, 0, c.stream>>>(LB, rd, n, b, D);
    cudaMemsetAsync(c.d_Ainv32, 0, sizeof(float) * (size_t)n * n, c.stream);
    ++g_launches;
    switch (c.trinv_g) {
        case 16: trinv32_launch<16>(c, LB, D, n, b); break;
        case 8: trinv32_launch<8>(c, LB, D, n, b); break;
        case 4: trinv32_launch<4>(c, LB, D, n, b); break;
        default: trinv32_launch<2>(c, LB, D, n, b); break;
    }
}

// The FP64 copy M of L^-1 (double-float sweep), for the FP64 V-cycle; made on
// first use after each factorization.
int ensure_coarse_m64(Ctx &c) {
    if (c.m64_valid || c.ncf == 0) return 0;
    const int n = c.ncf, b = c.cband;
    const int nblk = (n + NB - 1) / NB;
    const float2 *LB = reinterpret_cast<const float2 *>(c.d_LB), *D = LB + (int64_t)n * (b + 1) + n;
    (void)nblk;
    if (cudaMemsetAsync(c.d_Ainv, 0, sizeof(double) * (size_t)n * n, c.stream) != cudaSuccess) return -1;
    ++g_launches;
    switch (c.trinv_g) {
        case 16: trinv64_launch<16>(c, LB, D, n, b); break;
        case 8: trinv64_launch<8>(c, LB, D, n, b); break;
        case 4: trinv64_launch<4>(c, LB, D, n, b); break;
        default: trinv64_launch<2>(c, LB, D, n, b); break;
    }
    if (cudaGetLastError() != cudaSuccess) return -1;
    c.m64_valid = true;
    return 0;
}

// Cholesky of the dense coarsest matrix in d_Ac (lower, in place) and
// M = L^-1 in d_Ainv / d_Ainv32.  Returns 0, the 1-based failing pivot, -1 on
// a CUDA error or -2 when the band is too wide for the shared ring.
int coarse_factor_invert(Ctx &c) {
    const int n = c.ncf;
    if (n == 0) return 0;
    int *d_info = c.d_iflag + 8;
    if (!c.factor_graph) {
        int R = 32;
        while (R < c.cband + 32) R <<= 1;
        int G = 16;   // the widest column group whose ring fits
        while (G > 2 && trinv_smem_bytes(R, G) > 220 * 1024) G >>= 1;
        const size_t smem = trinv_smem_bytes(R, G);
        if (smem > 220 * 1024) return -2;
        switch (G) {
            case 16: trinv_attributes<16>(R); break;
            case 8: trinv_attributes<8>(R); break;
            case 4: trinv_attributes<4>(R); break;
            default: trinv_attributes<2>(R); break;
        }
        c.trinv_ring = R;
        c.trinv_g = G;
        c.trinv_smem = smem;
        const int64_t before = g_launches;
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return -1;
        factor_enqueue(c, d_info);
        if (cudaStreamEndCapture(c.stream, &g) != cudaSuccess) return -1;
        c.factor_graph_launches = g_launches - before;
        g_launches = before;
        if (cudaGraphInstantiate(&c.factor_graph, g, 0) != cudaSuccess) {
            cudaGraphDestroy(g);
            return -1;
        }
        cudaGraphDestroy(g);
    }
    if (cudaGraphLaunch(c.factor_graph, c.stream) != cudaSuccess) return -1;
    g_launches += c.factor_graph_launches;
    c.m64_valid = false;
    int info = 0;
    cudaMemcpyAsync(&info, d_info, sizeof(int), cudaMemcpyDeviceToHost, c.stream);
    cudaStreamSynchronize(c.stream);
    return info;
}

// ---- coarse apply: x_L[free] = A^-1 r_L[free] = M' (M r) -------------------------
// The inverse factor is stored square: M (lower triangle, column-major) and
// its transpose in the upper triangle, so that both products are column-major
// GEMVs with coalesced loads.  A CTA covers 32 output rows and one of CSPLIT
// column chunks; each warp takes 32-column blocks of the chunk, lane l holding
// row i0 + l: its 32 loads of a block (one coalesced row segment per column)
// are independent and in flight together.  The 8 warps' sums meet in shared
// memory and the chunk's partial goes to part[chunk * n + row].
//   lower (UPPER = false): y_i = sum_{j <= i} M[i + n j] v[rows[j]]
//   upper (UPPER = true):  x_j = sum_{i >= j} M[j + n i] v[i]   (= (M' v)_j)
constexpr int CL_WARPS = 8;

template <typename T, bool UPPER>
__global__ void __launch_bounds__(32 * CL_WARPS) k_coarse_gemv(const T *__restrict__ M, const int *__restrict__ rows,
                                                              const T *__restrict__ v, int n,
                                                              double *__restrict__ part) {
    __shared__ T red[CL_WARPS][32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i0 = blockIdx.x * 32, i = i0 + lane;
    const int chunk = ((n + CSPLIT - 1) / CSPLIT + 31) & ~31;
    int j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    if (UPPER)
        j0 = max(j0, i0);
    else
        j1 = min(j1, i0 + 32);
    const int ii = min(i, n - 1);
    T acc = T(0);
    for (int jb = j0 + 32 * w; jb < j1; jb += 32 * CL_WARPS) {
        const int jl = jb + lane;
        const T vl = (jl < n) ? (UPPER ? v[jl] : v[rows[jl]]) : T(0);
        T a0 = T(0), a1 = T(0);
#pragma unroll
        for (int q = 0; q < 32; q += 2) {
            const int ja = jb + q, jc = jb + q + 1;
            const T ma = (ja < n) ? M[(int64_t)ja * n + ii] : T(0);
            const T mc = (jc < n) ? M[(int64_t)jc * n + ii] : T(0);
            const T va = __shfl_sync(0xffffffffu, vl, q), vc = __shfl_sync(0xffffffffu, vl, q + 1);
            a0 += (UPPER ? ja >= i : ja <= i) ? ma * va : T(0);
            a1 += (UPPER ? jc >= i : jc <= i) ? mc * vc : T(0);
        }
        acc += a0 + a1;
    }
    red[w][lane] = acc;
    __syncthreads();
    if (w == 0 && i < n) {
        double sum = 0.0;
#pragma unroll
        for (int k = 0; k < CL_WARPS; ++k) sum += (double)red[k][lane];
        part[(int64_t)blockIdx.y * n + i] = sum;
    }
}

// y_i = sum of the chunk partials (compact), or x[rows[i]] = that sum (scatter)
template <typename T, bool SCATTER>
__global__ void k_coarse_sum(const double *__restrict__ part, int n, const int *__restrict__ rows,
                             T *__restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int k = 0; k < CSPLIT; ++k) s += part[(int64_t)k * n + i];
    y[SCATTER ? rows[i] : i] = (T)s;
}

template <typename T>
static void coarse_apply(const Ctx &c, const T *M, const T *rc, T *xc, T *ybuf, cudaStream_t s) {
    const Level &lc = c.lv[c.L - 1];
    cudaMemsetAsync(xc, 0, sizeof(T) * 3 * lc.nnode, s);
    if (c.ncf == 0) return;
    const dim3 g((c.ncf + 31) / 32, CSPLIT);
    const unsigned gs = (unsigned)((c.ncf + 127) / 128);
    g_launches += 4;
    k_coarse_gemv<T, false><<<g, 32 * CL_WARPS, 0, s>>>(M, c.d_cfree, rc, c.ncf, c.d_cpart);
    k_coarse_sum<T, false><<<gs, 128, 0, s>>>(c.d_cpart, c.ncf, c.d_cfree, ybuf);
    k_coarse_gemv<T, true><<<g, 32 * CL_WARPS, 0, s>>>(M, c.d_cfree, ybuf, c.ncf, c.d_cpart);
    k_coarse_sum<T, true><<<gs, 128, 0, s>>>(c.d_cpart, c.ncf, c.d_cfree, xc);
}

void launch_coarse_apply_f64(const Ctx &c, const double *rc, double *xc, cudaStream_t s) {
    coarse_apply<double>(c, c.d_Ainv, rc, xc, c.d_cy, s);
}

void launch_coarse_apply_f32(const Ctx &c, const float *rc, float *xc, cudaStream_t s) {
    coarse_apply<float>(c, c.d_Ainv32, rc, xc, reinterpret_cast<float *>(c.d_cy + c.ncf), s);
}

}  // namespace sgld
