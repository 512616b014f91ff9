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
//    blocked band Cholesky K = L L', explicit inverse A^-1 = L^-T L^-1
//    (two band TRSMs), applied per V-cycle as one dense GEMV.  The reference
//    applies its sparse Cholesky factor with two triangular solves
//    (src/Solving_Vcycle.m:116-118); the inverse gives the same numbers to
//    rounding and turns a sequential solve into a parallel mat-vec.
#include <math.h>

#include <vector>

#include "sgld_internal.cuh"

namespace sgld {

// ---- level 2 from the finest level ------------------------------------------
__global__ void __launch_bounds__(192) k_asm_finest(const double *__restrict__ E, const uint8_t *__restrict__ eact_c,
                                                    const double *__restrict__ H, int nyc, int nxc, int nzc, int s,
                                                    double *__restrict__ Ks) {
    const int64_t e = blockIdx.x + (int64_t)gridDim.x * blockIdx.y;
    const int64_t nel = (int64_t)nyc * nxc * nzc;
    if (e >= nel || !eact_c[e]) return;
    __shared__ double ev[64];
    const int cy = (int)(e % nyc), cx = (int)((e / nyc) % nxc), cz = (int)(e / ((int64_t)nyc * nxc));
    const int nyf = s * nyc, nxf = s * nxc;
    const int nq = s * s * s;
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
        const int oy = q % s, ox = (q / s) % s, oz = q / (s * s);
        ev[q] = E[(int64_t)(s * cy + oy) + (int64_t)nyf * ((s * cx + ox) + (int64_t)nxf * (s * cz + oz))];
    }
    __syncthreads();
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    const int t = threadIdx.x;
    for (int q = 0; q < nq; ++q) {
        const double w = ev[q];
        if (w == 0.0) continue;
        const double *h = H + 576 * q;
        a0 += w * h[t];
        a1 += w * h[t + 192];
        a2 += w * h[t + 384];
    }
    double *o = Ks + 576 * e;
    o[t] = a0;
    o[t + 192] = a1;
    o[t + 384] = a2;
}

void launch_asm_finest(const Level &coarse, const Level &fine, const double *E, const double *H, double *Ks,
                       cudaStream_t s) {
    (void)fine;
    const int64_t nel = coarse.nel;
    const unsigned gx = (unsigned)(nel < 65535 ? nel : 65535);
    const unsigned gy = (unsigned)((nel + gx - 1) / gx);
    ++g_launches;
    k_asm_finest<<<dim3(gx, gy), 192, 0, s>>>(E, coarse.eact, H, coarse.ny, coarse.nx, coarse.nz, coarse.span, Ks);
}

// ---- deeper levels: P_q' Ks_q P_q ---------------------------------------------
__constant__ double c_W[8 * 64];   // W_q[j][a] at c_W[64 q + 8 j + a]

__global__ void __launch_bounds__(192) k_asm_coarse(const double *__restrict__ Kf, const uint8_t *__restrict__ eact_f,
                                                    const uint8_t *__restrict__ eact_c, int nyc, int nxc, int nzc,
                                                    double *__restrict__ Ks) {
    const int64_t e = blockIdx.x + (int64_t)gridDim.x * blockIdx.y;
    const int64_t nel = (int64_t)nyc * nxc * nzc;
    if (e >= nel || !eact_c[e]) return;
    __shared__ double sk[576], st[576];
    const int cy = (int)(e % nyc), cx = (int)((e / nyc) % nxc), cz = (int)(e / ((int64_t)nyc * nxc));
    const int nyf = 2 * nyc, nxf = 2 * nxc;
    const int t = threadIdx.x;
    double acc[3] = {0.0, 0.0, 0.0};
    for (int q = 0; q < 8; ++q) {
        const int oy = q & 1, ox = (q >> 1) & 1, oz = q >> 2;
        const int64_t f = (int64_t)(2 * cy + oy) + (int64_t)nyf * ((2 * cx + ox) + (int64_t)nxf * (2 * cz + oz));
        if (!eact_f[f]) continue;   // uniform per CTA
        const double *src = Kf + 576 * f;
        for (int i = t; i < 576; i += 192) sk[i] = src[i];
        __syncthreads();
        const double *W = c_W + 64 * q;
        // st[r + 24*(3a+d)] = sum_i sk[r + 24*(3i+d)] W[i][a]
        for (int idx = t; idx < 576; idx += 192) {
            const int r = idx % 24, col = idx / 24, a = col / 3, d = col % 3;
            double v = 0.0;
#pragma unroll
            for (int i = 0; i < 8; ++i) v += sk[r + 24 * (3 * i + d)] * W[8 * i + a];
            st[idx] = v;
        }
        __syncthreads();
        // out[(3b+e) + 24*col] += sum_j W[j][b] st[(3j+e) + 24*col]
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int idx = t + 192 * k;
            const int row = idx % 24, col = idx / 24, b = row / 3, ec = row % 3;
            double v = 0.0;
#pragma unroll
            for (int j = 0; j < 8; ++j) v += W[8 * j + b] * st[(3 * j + ec) + 24 * col];
            acc[k] += v;
        }
        __syncthreads();
    }
    double *o = Ks + 576 * e;
    o[t] = acc[0];
    o[t + 192] = acc[1];
    o[t + 384] = acc[2];
}

void launch_asm_coarse(const Level &coarse, const Level &fine, double *Ks, cudaStream_t s) {
    // W_q for span 2, reference corner order, child order y fastest
    static bool uploaded = false;
    if (!uploaded) {
        const int cdy[8] = {1, 1, 0, 0, 1, 1, 0, 0}, cdx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cdz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
        double W[8 * 64];
        for (int q = 0; q < 8; ++q) {
            const int oy = q & 1, ox = (q >> 1) & 1, oz = q >> 2;
            for (int j = 0; j < 8; ++j) {
                // child corner position in the 3x3x3 local block (units of fine cells)
                const int py = oy + cdy[j], px = ox + cdx[j], pz = oz + cdz[j];
                // natural coordinates in the parent: s = -1 + px, t = 1 - py, p = -1 + pz
                const double sn = -1.0 + px, tn = 1.0 - py, pn = -1.0 + pz;
                const double N[8] = {(1 - sn) * (1 - tn) * (1 - pn), (1 + sn) * (1 - tn) * (1 - pn),
                                     (1 + sn) * (1 + tn) * (1 - pn), (1 - sn) * (1 + tn) * (1 - pn),
                                     (1 - sn) * (1 - tn) * (1 + pn), (1 + sn) * (1 - tn) * (1 + pn),
                                     (1 + sn) * (1 + tn) * (1 + pn), (1 - sn) * (1 + tn) * (1 + pn)};
                for (int a = 0; a < 8; ++a) W[64 * q + 8 * j + a] = 0.125 * N[a];
            }
        }
        cudaMemcpyToSymbolAsync(c_W, W, sizeof W, 0, cudaMemcpyHostToDevice, s);
        uploaded = true;
    }
    const int64_t nel = coarse.nel;
    const unsigned gx = (unsigned)(nel < 65535 ? nel : 65535);
    const unsigned gy = (unsigned)((nel + gx - 1) / gx);
    ++g_launches;
    k_asm_coarse<<<dim3(gx, gy), 192, 0, s>>>(fine.Ks, fine.eact, coarse.eact, coarse.ny, coarse.nx, coarse.nz, Ks);
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
    cudaMemsetAsync(A, 0, sizeof(double) * (size_t)ncf * ncf, s);
    ++g_launches;
    k_coarse_dense<<<(ncf + 127) / 128, 128, 0, s>>>(lc.Ks, lc.eact, lc.ny, lc.nx, lc.nz, rows, pos, ncf, A);
}

// ---- blocked band Cholesky, NB x NB tiles, column-major n x n ------------------
constexpr int NB = 32;

// factor the diagonal tile in place (lower), one CTA of NB*NB threads
__global__ void k_potrf_tile(double *A, int n, int k0, int *info) {
    __shared__ double T[NB][NB + 1];
    const int tx = threadIdx.x % NB, ty = threadIdx.x / NB;   // tx = row, ty = col
    const int m = min(NB, n - k0);
    T[tx][ty] = (tx < m && ty < m) ? A[(int64_t)(k0 + tx) + (int64_t)n * (k0 + ty)] : (tx == ty ? 1.0 : 0.0);
    __syncthreads();
    for (int j = 0; j < m; ++j) {
        if (tx == j && ty == j) {
            const double d = T[j][j];
            if (!(d > 0.0)) {
                if (info) atomicExch(info, k0 + j + 1);
                T[j][j] = 1.0;
            } else {
                T[j][j] = sqrt(d);
            }
        }
        __syncthreads();
        if (ty == j && tx > j) T[tx][j] /= T[j][j];
        __syncthreads();
        if (tx > j && ty > j && ty <= tx) T[tx][ty] -= T[tx][j] * T[ty][j];
        __syncthreads();
    }
    if (tx < m && ty < m) A[(int64_t)(k0 + tx) + (int64_t)n * (k0 + ty)] = (ty <= tx) ? T[tx][ty] : 0.0;
}

// A[i-tile, k-tile] <- A[i-tile, k-tile] * L_kk^-T for tiles i = k+1 .. kend
__global__ void k_trsm_panel(double *A, int n, int k0, int iblk0) {
    __shared__ double L[NB][NB + 1];
    const int t = threadIdx.x;   // NB threads: one per row of the panel tile
    const int m = min(NB, n - k0);
    for (int idx = t; idx < NB * NB; idx += NB) {
        const int r = idx % NB, c = idx / NB;
        L[r][c] = (r < m && c < m) ? A[(int64_t)(k0 + r) + (int64_t)n * (k0 + c)] : 0.0;
    }
    __syncthreads();
    const int i0 = (iblk0 + blockIdx.x) * NB;
    const int row = i0 + t;
    if (row >= n) return;
    double x[NB];
#pragma unroll
    for (int j = 0; j < NB; ++j) x[j] = (j < m) ? A[(int64_t)row + (int64_t)n * (k0 + j)] : 0.0;
#pragma unroll
    for (int j = 0; j < NB; ++j) {
        if (j < m) {
            double v = x[j];
            for (int q = 0; q < j; ++q) v -= x[q] * L[j][q];
            x[j] = v / L[j][j];
        }
    }
#pragma unroll
    for (int j = 0; j < NB; ++j)
        if (j < m) A[(int64_t)row + (int64_t)n * (k0 + j)] = x[j];
}

// trailing update A[i,j] -= A[i,k] A[j,k]' for k < j <= i <= kend (tile pairs)
__global__ void k_syrk_update(double *A, int n, int k0, int jb0, int nbt) {
    // map blockIdx.x -> (ii, jj) with 0 <= jj <= ii < nbt
    int p = blockIdx.x, ii = 0;
    while (p > ii) {
        p -= ii + 1;
        ++ii;
    }
    const int jj = p;
    const int i0 = (jb0 + ii) * NB, j0 = (jb0 + jj) * NB;
    __shared__ double Ai[NB][NB + 1], Aj[NB][NB + 1];
    const int t = threadIdx.x;   // 256 threads
    const int m = min(NB, n - k0);
    for (int idx = t; idx < NB * NB; idx += 256) {
        const int r = idx % NB, c = idx / NB;
        Ai[r][c] = (i0 + r < n && c < m) ? A[(int64_t)(i0 + r) + (int64_t)n * (k0 + c)] : 0.0;
        Aj[r][c] = (j0 + r < n && c < m) ? A[(int64_t)(j0 + r) + (int64_t)n * (k0 + c)] : 0.0;
    }
    __syncthreads();
    for (int idx = t; idx < NB * NB; idx += 256) {
        const int r = idx % NB, c = idx / NB;
        if (i0 + r >= n || j0 + c >= n) continue;
        if (ii == jj && c > r) continue;
        double v = 0.0;
#pragma unroll 8
        for (int q = 0; q < NB; ++q) v += Ai[r][q] * Aj[c][q];
        A[(int64_t)(i0 + r) + (int64_t)n * (j0 + c)] -= v;
    }
}

__global__ void k_to_f32(const double *a, float *b, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

// LB[i*(b+1) + d] = L[i, i-b+d], d = 0..b (0 outside the matrix)
__global__ void k_band_rows(const double *__restrict__ L, int n, int b, double *__restrict__ LB) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)n * (b + 1)) return;
    const int i = (int)(t / (b + 1)), d = (int)(t % (b + 1));
    const int k = i - b + d;
    LB[t] = (k >= 0) ? L[(int64_t)i + (int64_t)n * k] : 0.0;
}

// M = L^-1: warp w of the CTA owns column c; for rows i = c..n-1
//   M[i,c] = (delta_ic - sum_{k=max(c,i-b)}^{i-1} L[i,k] M[k,c]) / L[i,i],
// with the last R values of the column kept in a shared ring (R a power of
// two > b, dynamic shared memory of warps * R doubles).
__global__ void k_trinv_cols(const double *__restrict__ LB, int n, int b, int R, double *__restrict__ M) {
    extern __shared__ double ringmem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = blockIdx.x * (blockDim.x >> 5) + w;
    if (c >= n) return;
    double *ring = ringmem + (int64_t)w * R;
    for (int i = c; i < n; ++i) {
        const int k0 = max(c, i - b);
        const double *row = LB + (int64_t)i * (b + 1) - (i - b);   // row[k] = L[i,k]
        double s = 0.0;
        for (int k = k0 + lane; k < i; k += 32) s += row[k] * ring[k & (R - 1)];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        const double v = ((i == c ? 1.0 : 0.0) - s) / row[i];
        if (lane == 0) {
            ring[i & (R - 1)] = v;
            M[(int64_t)i + (int64_t)n * c] = v;
        }
        __syncwarp();
    }
}

int coarse_factor_invert(Ctx &c) {
    const int n = c.ncf;
    if (n == 0) return 0;
    const int nblk = (n + NB - 1) / NB;
    const int bw = (c.cband + NB - 1) / NB + 1;   // band in tiles (safety margin of one)
    int *d_info = c.d_iflag + 8;
    cudaMemsetAsync(d_info, 0, sizeof(int), c.stream);
    double *A = c.d_Ac;
    for (int kb = 0; kb < nblk; ++kb) {
        const int k0 = kb * NB;
        ++g_launches;
        k_potrf_tile<<<1, NB * NB, 0, c.stream>>>(A, n, k0, d_info);
        const int kend = min(nblk - 1, kb + bw);
        const int nbelow = kend - kb;
        if (nbelow > 0) {
            ++g_launches;
            k_trsm_panel<<<nbelow, NB, 0, c.stream>>>(A, n, k0, kb + 1);
            const int npairs = nbelow * (nbelow + 1) / 2;
            ++g_launches;
            k_syrk_update<<<npairs, 256, 0, c.stream>>>(A, n, k0, kb + 1, nbelow);
        }
    }
    // M = L^-1 (dense lower triangular) column by column: one warp per column,
    // rows in order, the band of L read as contiguous rows
    const int b = c.cband;
    ++g_launches;
    k_band_rows<<<(unsigned)(((int64_t)n * (b + 1) + 255) / 256), 256, 0, c.stream>>>(A, n, b, c.d_LB);
    cudaMemsetAsync(c.d_Ainv, 0, sizeof(double) * (size_t)n * n, c.stream);
    int R = 32;
    while (R < b + 1) R <<= 1;
    int warps = 8;
    while (warps > 1 && (size_t)warps * R * sizeof(double) > 200 * 1024) warps >>= 1;
    const size_t smem = (size_t)warps * R * sizeof(double);
    if (smem > 220 * 1024) return -2;   // band too wide for the shared ring
    cudaFuncSetAttribute(k_trinv_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    ++g_launches;
    k_trinv_cols<<<(n + warps - 1) / warps, 32 * warps, smem, c.stream>>>(c.d_LB, n, b, R, c.d_Ainv);
    const int64_t nn = (int64_t)n * n;
    ++g_launches;
    k_to_f32<<<(unsigned)((nn + 255) / 256), 256, 0, c.stream>>>(c.d_Ainv, c.d_Ainv32, nn);
    int info = 0;
    cudaMemcpyAsync(&info, d_info, sizeof(int), cudaMemcpyDeviceToHost, c.stream);
    cudaStreamSynchronize(c.stream);
    return info;
}

// ---- coarse apply: x_L[free] = A^-1 r_L[free] = M' (M r) -------------------------
// y = M r (M lower triangular): rows in threads, columns split into CSPLIT chunks
template <typename T>
__global__ void k_coarse_lower(const T *__restrict__ M, const int *__restrict__ rows, const T *__restrict__ r, int n,
                               double *__restrict__ part) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int chunk = (n + CSPLIT - 1) / CSPLIT;
    const int j0 = blockIdx.y * chunk, j1 = min(min(n, j0 + chunk), i + 1);
    if (i >= n) return;
    T acc = T(0);
    for (int j = j0; j < j1; ++j) acc += M[(int64_t)i + (int64_t)n * j] * r[rows[j]];
    part[(int64_t)blockIdx.y * n + i] = (double)acc;
}

template <typename T>
__global__ void k_coarse_sum(const double *__restrict__ part, int n, T *__restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int k = 0; k < CSPLIT; ++k) s += part[(int64_t)k * n + i];
    y[i] = (T)s;
}

// x_j = sum_{i >= j} M[i,j] y_i: one warp per column (coalesced column reads)
template <typename T>
__global__ void k_coarse_upper(const T *__restrict__ M, const int *__restrict__ rows, const T *__restrict__ y, int n,
                               T *__restrict__ x) {
    const int j = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (j >= n) return;
    const T *col = M + (int64_t)n * j;
    T acc = T(0);
    for (int i = j + lane; i < n; i += 32) acc += col[i] * y[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) x[rows[j]] = acc;
}

template <typename T>
static void coarse_apply(const Ctx &c, const T *M, const T *rc, T *xc, T *ybuf, cudaStream_t s) {
    const Level &lc = c.lv[c.L - 1];
    cudaMemsetAsync(xc, 0, sizeof(T) * 3 * lc.nnode, s);
    if (c.ncf == 0) return;
    dim3 g((c.ncf + 127) / 128, CSPLIT);
    ++g_launches;
    k_coarse_lower<T><<<g, 128, 0, s>>>(M, c.d_cfree, rc, c.ncf, c.d_cpart);
    ++g_launches;
    k_coarse_sum<T><<<(c.ncf + 127) / 128, 128, 0, s>>>(c.d_cpart, c.ncf, ybuf);
    ++g_launches;
    k_coarse_upper<T><<<(unsigned)(((int64_t)c.ncf * 32 + 255) / 256), 256, 0, s>>>(M, c.d_cfree, ybuf, c.ncf, xc);
}

void launch_coarse_apply_f64(const Ctx &c, const double *rc, double *xc, cudaStream_t s) {
    coarse_apply<double>(c, c.d_Ainv, rc, xc, c.d_cy, s);
}

void launch_coarse_apply_f32(const Ctx &c, const float *rc, float *xc, cudaStream_t s) {
    coarse_apply<float>(c, c.d_Ainv32, rc, xc, reinterpret_cast<float *>(c.d_cy + c.ncf), s);
}

}  // namespace sgld
