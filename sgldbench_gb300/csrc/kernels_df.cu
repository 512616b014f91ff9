// FP64-accurate K*u in double-float arithmetic (pairs of FP32 numbers) for
// the outer loop of the mixed-precision solve.
//
// GB300 issues FP64 at about 1/64 of its FP32 rate, and the FP64 K*u
// (kernels_stencil.cu) is bound by that issue rate.  A double-float value
// hi + lo carries 48 significant bits (df_arith.cuh: Knuth's TwoSum, the FMA
// form of Dekker's product; ~11 FP32 operations per add, ~7 per multiply).  The
// result is within a few units of 2^-48 of the FP64 operator (tests compare
// to 1e-12), enough for the FP64 residual recurrence of the outer flexible
// PCG and for its true residual at exit (relative tolerances >= 1e-12).
// The data stay FP64 in HBM; values are split into (hi, lo) when a node
// layer is staged and joined when a node's sum is stored.
#include "sgld_internal.cuh"
#include "df_arith.cuh"

namespace sgld {

__constant__ float c_khh[KH_NNZ], c_khl[KH_NNZ];

void upload_kh_df(const double *Kh, cudaStream_t s) {
    float h[KH_NNZ], l[KH_NNZ];
    for (int i = 0; i < KH_NNZ; ++i) {
        h[i] = (float)Kh[i];
        l[i] = (float)(Kh[i] - (double)h[i]);
    }
    cudaMemcpyToSymbolAsync(c_khh, h, sizeof h, 0, cudaMemcpyHostToDevice, s);
    cudaMemcpyToSymbolAsync(c_khl, l, sizeof l, 0, cudaMemcpyHostToDevice, s);
}

__device__ __forceinline__ df khd(int i) { return {c_khh[i], c_khl[i]}; }

// e * Ke * u for one element in the Hadamard basis (same structure as hex_apply)
__device__ __forceinline__ void hex_apply_df(df (&u)[24], df e) {
#pragma unroll
    for (int ax = 0; ax < 3; ++ax)
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (k & (1 << ax)) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const df lo = u[3 * k + c], hi = u[3 * (k | (1 << ax)) + c];
                u[3 * k + c] = df_add(lo, hi);
                u[3 * (k | (1 << ax)) + c] = df_sub(hi, lo);
            }
        }
    df g[24];
    g[0] = g[1] = g[2] = {0.f, 0.f};
#define D3(i, j, k, o)                                                                                     \
    {                                                                                                      \
        const df a = u[i], b = u[j], d = u[k];                                                             \
        g[i] = df_add(df_add(df_mul(khd(o), a), df_mul(khd(o + 1), b)), df_mul(khd(o + 2), d));            \
        g[j] = df_add(df_add(df_mul(khd(o + 3), a), df_mul(khd(o + 4), b)), df_mul(khd(o + 5), d));        \
        g[k] = df_add(df_add(df_mul(khd(o + 6), a), df_mul(khd(o + 7), b)), df_mul(khd(o + 8), d));        \
    }
#define D2(i, j, o)                                                     \
    {                                                                   \
        const df a = u[i], b = u[j];                                    \
        g[i] = df_add(df_mul(khd(o), a), df_mul(khd(o + 1), b));        \
        g[j] = df_add(df_mul(khd(o + 2), a), df_mul(khd(o + 3), b));    \
    }
    D3(3, 7, 14, 0)
    D2(4, 6, 9)
    D2(5, 12, 13)
    D2(8, 13, 17)
    D2(9, 20, 21)
    D2(10, 17, 25)
    D3(11, 16, 18, 29)
    D2(15, 19, 38)
    g[21] = df_mul(khd(42), u[21]);
    g[22] = df_mul(khd(43), u[22]);
    g[23] = df_mul(khd(44), u[23]);
#undef D3
#undef D2
#pragma unroll
    for (int i = 3; i < 24; ++i) g[i] = df_mul(g[i], e);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax)
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (k & (1 << ax)) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const df a = g[3 * k + c], d = g[3 * (k | (1 << ax)) + c];
                g[3 * k + c] = df_sub(a, d);
                g[3 * (k | (1 << ax)) + c] = df_add(a, d);
            }
        }
#pragma unroll
    for (int i = 0; i < 24; ++i) u[i] = g[i];
}

constexpr int DT_Y = 32, DT_X = 8, DT_THREADS = DT_Y * DT_X;
constexpr int DT_NL = (DT_Y + 1) * (DT_X + 1);
constexpr int DT_ZC = 16;
constexpr int DT_SV = (DT_NL * 3 + DT_THREADS - 1) / DT_THREADS;

// Same tiling as k_kbyu (a CTA owns 31 x 7 node columns and marches in z);
// FP64 in and out, double-float inside.  Optional fused u . y (FP64).
template <bool DOT>
__global__ void __launch_bounds__(DT_THREADS) k_kbyu_df(const double *__restrict__ u, double *__restrict__ y,
                                                        const double *__restrict__ E,
                                                        const uint8_t *__restrict__ nflag, int ny, int nx, int nz,
                                                        double *__restrict__ partial,
                                                        const uint8_t *__restrict__ tiles) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    df *su = reinterpret_cast<df *>(smem_raw);   // [2][DT_NL*3] node layers (hi, lo)
    df *so = su + 2 * DT_NL * 3;                 // [24][DT_THREADS]
    const int tid = threadIdx.x;
    const int ty = tid % DT_Y, tx = tid / DT_Y;
    const int NY = ny + 1, NX = nx + 1, NZ = nz + 1;
    const int y0 = blockIdx.x * (DT_Y - 1), x0 = blockIdx.y * (DT_X - 1), z0 = blockIdx.z * DT_ZC;
    const int zend = min(z0 + DT_ZC, NZ);
    const int gny = y0 + ty, gnx = x0 + tx;
    const bool owner = (ty < DT_Y - 1) && (tx < DT_X - 1) && gny < NY && gnx < NX;
    const int ey = y0 - 1 + ty, ex = x0 - 1 + tx;
    const bool ein = ey >= 0 && ey < ny && ex >= 0 && ex < nx;
    if (tiles && !tiles[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)]) {
        // no active element in the CTA's box: its nodes are inactive, K*u is zero there
        if (owner) {
            const int64_t node0 = (int64_t)gny + (int64_t)NY * gnx;
            for (int z = z0; z < zend; ++z) {
                double *o = y + 3 * (node0 + (int64_t)NY * NX * z);
                o[0] = 0.0;
                o[1] = 0.0;
                o[2] = 0.0;
            }
        }
        if (DOT && tid == 0) partial[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = 0.0;
        return;
    }
    int soff[DT_SV];
#pragma unroll
    for (int k = 0; k < DT_SV; ++k) {
        const int i = tid + k * DT_THREADS;
        soff[k] = -2;
        if (i < DT_NL * 3) {
            const int node = i / 3, c = i - 3 * node;
            const int ly = node % (DT_Y + 1), lx = node / (DT_Y + 1);
            const int gy = y0 - 1 + ly, gx = x0 - 1 + lx;
            soff[k] = (gy >= 0 && gy < NY && gx >= 0 && gx < NX) ? 3 * (gy + NY * gx) + c : -1;
        }
    }
    const int64_t lstride = 3 * (int64_t)NY * NX;
    auto stage = [&](int z, int slot) {
        df *dst = su + slot * DT_NL * 3;
        const bool zin = z >= 0 && z < NZ;
#pragma unroll
        for (int k = 0; k < DT_SV; ++k) {
            const int i = tid + k * DT_THREADS;
            if (soff[k] == -2) continue;
            dst[i] = (zin && soff[k] >= 0) ? df_from(u[(int64_t)z * lstride + soff[k]]) : df{0.f, 0.f};
        }
    };
    df acc[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    double dot = 0.0;
    stage(z0 - 1, (z0 + 1) & 1);
    for (int ez = z0 - 1; ez < zend; ++ez) {
        const int s0 = ez & 1, s1 = (ez + 1) & 1;
        stage(ez + 1, s1);
        __syncthreads();
        df ev = {0.f, 0.f};
        if (ein && ez >= 0 && ez < nz) ev = df_from(E[(int64_t)ey + (int64_t)ny * (ex + (int64_t)nx * ez)]);
        df ue[24];
        if (ev.hi != 0.f) {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int dx = k & 1, dy = 1 - ((k >> 1) & 1), kp = k >> 2;
                const df *src = su + (kp ? s1 : s0) * DT_NL * 3 + 3 * ((ty + dy) + (DT_Y + 1) * (tx + dx));
                ue[3 * k] = src[0];
                ue[3 * k + 1] = src[1];
                ue[3 * k + 2] = src[2];
            }
            hex_apply_df(ue, ev);
        } else {
#pragma unroll
            for (int i = 0; i < 24; ++i) ue[i] = {0.f, 0.f};
        }
#pragma unroll
        for (int i = 0; i < 24; ++i) so[i * DT_THREADS + tid] = ue[i];
        __syncthreads();
        if (owner) {
#pragma unroll
            for (int dy = 0; dy < 2; ++dy)
#pragma unroll
                for (int dx = 0; dx < 2; ++dx) {
                    const int k = dx | ((1 - dy) << 1);
                    const int t = (ty + 1 - dy) + DT_Y * (tx + 1 - dx);
#pragma unroll
                    for (int c = 0; c < 3; ++c) acc[c] = df_add(acc[c], so[(3 * k + c) * DT_THREADS + t]);
                }
            if (ez >= z0) {
                const int64_t node = (int64_t)gny + (int64_t)NY * (gnx + (int64_t)NX * ez);
                const uint8_t f = nflag[node];
                double o[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) o[c] = (f & (NF_FIXX << c)) ? 0.0 : df_to(acc[c]);
                y[3 * node] = o[0];
                y[3 * node + 1] = o[1];
                y[3 * node + 2] = o[2];
                if (DOT) dot += u[3 * node] * o[0] + u[3 * node + 1] * o[1] + u[3 * node + 2] * o[2];
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) acc[c] = {0.f, 0.f};
#pragma unroll
            for (int dy = 0; dy < 2; ++dy)
#pragma unroll
                for (int dx = 0; dx < 2; ++dx) {
                    const int k = 4 | dx | ((1 - dy) << 1);
                    const int t = (ty + 1 - dy) + DT_Y * (tx + 1 - dx);
#pragma unroll
                    for (int c = 0; c < 3; ++c) acc[c] = df_add(acc[c], so[(3 * k + c) * DT_THREADS + t]);
                }
        }
        __syncthreads();
    }
    if (DOT) {
        __shared__ double red[DT_THREADS / 32];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
        if ((tid & 31) == 0) red[tid >> 5] = dot;
        __syncthreads();
        if (tid == 0) {
            double s = 0.0;
            for (int i = 0; i < DT_THREADS / 32; ++i) s += red[i];
            partial[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = s;
        }
    }
}

static constexpr size_t kbyu_df_smem() { return sizeof(df) * (2 * DT_NL * 3 + 24 * DT_THREADS); }

void init_kbyu_df_attributes() {
    cudaFuncSetAttribute(k_kbyu_df<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kbyu_df_smem());
    cudaFuncSetAttribute(k_kbyu_df<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kbyu_df_smem());
}

void launch_kbyu_df(const Level &l0, const double *E, const double *u, double *y, double *partial_dot,
                    int *nblocks_out, cudaStream_t s) {
    const dim3 g((l0.ny + 1 + DT_Y - 2) / (DT_Y - 1), (l0.nx + 1 + DT_X - 2) / (DT_X - 1),
                 (l0.nz + 1 + DT_ZC - 1) / DT_ZC);
    if (nblocks_out) *nblocks_out = (int)(g.x * g.y * g.z);
    ++g_launches;
    if (partial_dot)
        k_kbyu_df<true><<<g, DT_THREADS, kbyu_df_smem(), s>>>(u, y, E, l0.nflag, l0.ny, l0.nx, l0.nz, partial_dot,
                                                             l0.tiles16);
    else
        k_kbyu_df<false><<<g, DT_THREADS, kbyu_df_smem(), s>>>(u, y, E, l0.nflag, l0.ny, l0.nx, l0.nz, nullptr,
                                                              l0.tiles16);
}

}  // namespace sgld
