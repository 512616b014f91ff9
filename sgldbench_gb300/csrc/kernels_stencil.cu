// Element-stencil kernels on the finest level: matrix-free K*u, unit
// compliance and the stress recovery of the solution.
//
// K*u (reference: src/MEXfuncs/Solving_KbyU_MatrixFree_mex.cpp:53-138) is
// restated for a structured grid without colouring.  A CTA owns a tile of
// (TY-1) x (TX-1) node columns and marches through z one element layer at a
// time: the two node layers an element layer touches are staged in shared
// memory, every thread applies E_e*Ke to one element of the (TY x TX)
// element tile (which includes a one-element halo), writes the 24 results to
// shared memory, and every node thread then sums the contributions of its 8
// neighbouring elements.  No atomics, deterministic, every node written once.
//
// The element product uses the 8-corner Hadamard basis in which the
// isotropic hexahedral Ke has 45 nonzeros (instead of 576): forward
// butterflies (72 adds), 45 FMAs, E scaling, inverse butterflies (72 adds).
// FP64 arithmetic is the scarce resource on GB300, so this is the form that
// matters for the FP64 operator.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "sgld_internal.cuh"

namespace sgld {

__constant__ double c_Kh[KH_NNZ];
__constant__ float c_Kh32[KH_NNZ];
// the 8-value form of an element matrix with cubic symmetry (kh_cubic):
// A-B, B, C, D, E, F-G, G, H (KH_CLASS below)
__constant__ float c_Kc32[8];
__constant__ double c_M[48 * 24];   // stress: corner stresses = M * u_e (reference corner order)

// Under the symmetries of the cube (axis permutations and reflections) an
// isotropic hexahedron's Hadamard-basis blocks take 8 values:
//   {3, 7, 14} and {11, 16, 18}: A / F on the diagonal, B / G off it;
//   {4, 6}, {5, 12}, {8, 13}: C in every entry;
//   {9, 20}, {10, 17}, {15, 19}: D on the diagonal, E off it;
//   21, 22, 23: H.
// KH_CLASS gives each of the 45 stored values its letter (A = 0 .. H = 7).
constexpr int KH_CLASS[KH_NNZ] = {0, 1, 1, 1, 0, 1, 1, 1, 0,   // {3, 7, 14}
                                  2, 2, 2, 2,                  // {4, 6}
                                  2, 2, 2, 2,                  // {5, 12}
                                  2, 2, 2, 2,                  // {8, 13}
                                  3, 4, 4, 3,                  // {9, 20}
                                  3, 4, 4, 3,                  // {10, 17}
                                  5, 6, 6, 6, 5, 6, 6, 6, 5,   // {11, 16, 18}
                                  3, 4, 4, 3,                  // {15, 19}
                                  7, 7, 7};                    // 21, 22, 23

bool kh_cubic(const double *Kh) {
    double rep[8], mx = 0.0;
    for (int i = KH_NNZ - 1; i >= 0; --i) {
        rep[KH_CLASS[i]] = Kh[i];   // ends with each letter's first entry
        mx = fmax(mx, fabs(Kh[i]));
    }
    for (int i = 0; i < KH_NNZ; ++i)
        if (fabs(Kh[i] - rep[KH_CLASS[i]]) > 1e-12 * mx) return false;
    return true;
}

void upload_kh(const double *Kh, cudaStream_t s) {
    float f[KH_NNZ];
    for (int i = 0; i < KH_NNZ; ++i) f[i] = (float)Kh[i];
    cudaMemcpyToSymbolAsync(c_Kh, Kh, sizeof(double) * KH_NNZ, 0, cudaMemcpyHostToDevice, s);
    cudaMemcpyToSymbolAsync(c_Kh32, f, sizeof(float) * KH_NNZ, 0, cudaMemcpyHostToDevice, s);
    // A-B, B, C, D, E, F-G, G, H from the letters' first entries (zeros when not cubic;
    // the 8-value kernels then never run)
    float kc[8] = {};
    if (kh_cubic(Kh)) {
        kc[0] = (float)(Kh[0] - Kh[1]);
        kc[1] = (float)Kh[1];
        kc[2] = (float)Kh[9];
        kc[3] = (float)Kh[21];
        kc[4] = (float)Kh[22];
        kc[5] = (float)(Kh[29] - Kh[30]);
        kc[6] = (float)Kh[30];
        kc[7] = (float)Kh[42];
    }
    cudaMemcpyToSymbolAsync(c_Kc32, kc, sizeof kc, 0, cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
}

template <typename T> __device__ __forceinline__ T khv(int i);
template <> __device__ __forceinline__ double khv<double>(int i) { return c_Kh[i]; }
template <> __device__ __forceinline__ float khv<float>(int i) { return c_Kh32[i]; }

// u[3*k + c]: corner bit index k = ks | kt<<1 | kp<<2.  On return u holds
// e * Ke * u in the same layout.
template <typename T>
__device__ __forceinline__ void hex_apply(T (&u)[24], T e) {
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (k & (1 << ax)) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const T lo = u[3 * k + c], hi = u[3 * (k | (1 << ax)) + c];
                u[3 * k + c] = lo + hi;
                u[3 * (k | (1 << ax)) + c] = hi - lo;
            }
        }
    }
    T g[24];
    g[0] = g[1] = g[2] = T(0);
#define KH3(i, j, k, o)                                                          \
    {                                                                            \
        const T a = u[i], b = u[j], d = u[k];                                    \
        g[i] = khv<T>(o) * a + khv<T>(o + 1) * b + khv<T>(o + 2) * d;            \
        g[j] = khv<T>(o + 3) * a + khv<T>(o + 4) * b + khv<T>(o + 5) * d;        \
        g[k] = khv<T>(o + 6) * a + khv<T>(o + 7) * b + khv<T>(o + 8) * d;        \
    }
#define KH2(i, j, o)                                     \
    {                                                    \
        const T a = u[i], b = u[j];                      \
        g[i] = khv<T>(o) * a + khv<T>(o + 1) * b;        \
        g[j] = khv<T>(o + 2) * a + khv<T>(o + 3) * b;    \
    }
    KH3(3, 7, 14, 0)
    KH2(4, 6, 9)
    KH2(5, 12, 13)
    KH2(8, 13, 17)
    KH2(9, 20, 21)
    KH2(10, 17, 25)
    KH3(11, 16, 18, 29)
    KH2(15, 19, 38)
    g[21] = khv<T>(42) * u[21];
    g[22] = khv<T>(43) * u[22];
    g[23] = khv<T>(44) * u[23];
#undef KH3
#undef KH2
#pragma unroll
    for (int i = 3; i < 24; ++i) g[i] *= e;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (k & (1 << ax)) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const T a = g[3 * k + c], d = g[3 * (k | (1 << ax)) + c];
                g[3 * k + c] = a - d;
                g[3 * (k | (1 << ax)) + c] = a + d;
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 24; ++i) u[i] = g[i];
}

// Per-CTA sum of a per-thread partial: the warp stage runs in the kernel's own
// precision T (FP64 issue is scarce on GB300, so FP32 kernels must not do
// their reductions in FP64), the 8 warp sums are added in FP64.
template <typename T>
__device__ __forceinline__ double block_sum_to_double(T v, double *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = (double)v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
    return s;
}

template <typename T>
__device__ __forceinline__ T block_sum(T v, T *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    T s = T(0);
    if (threadIdx.x == 0) {
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
    }
    return s;
}

constexpr int KT_Y = 32, KT_X = 8, KT_THREADS = KT_Y * KT_X;
constexpr int KT_NL = (KT_Y + 1) * (KT_X + 1);   // staged nodes per layer
constexpr int KT_ZC = 16;                        // node layers per CTA

constexpr int KT_SV = (KT_NL * 3 + KT_THREADS - 1) / KT_THREADS;   // staged words per thread and layer

// node layer z lives in ring slot z mod 3 (z may be -1)
__device__ __forceinline__ int kslot(int z) { return (z + 3) % 3; }

// asynchronous global -> shared word copy (cp.async, completes at async_wait_all)
template <typename T>
__device__ __forceinline__ void async_copy(T *dst, const T *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if (sizeof(T) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src));
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src));
}
__device__ __forceinline__ void async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// A CTA whose element box holds no active element: every node it owns is
// inactive and its K*u is exactly zero, so it writes zeros (no loads, no
// element work) and a zero dot partial.  The whole CTA takes this branch.
template <typename T>
__device__ __forceinline__ void skip_tile(T *__restrict__ y, bool owner, int gny, int gnx, int NY, int NX, int z0,
                                          int zend, double *__restrict__ partial) {
    if (owner) {
        const int64_t node0 = (int64_t)gny + (int64_t)NY * gnx;
        for (int z = z0; z < zend; ++z) {
            T *o = y + 3 * (node0 + (int64_t)NY * NX * z);
            o[0] = T(0);
            o[1] = T(0);
            o[2] = T(0);
        }
    }
    if (partial && threadIdx.x == 0) partial[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = 0.0;
}

// Active-tile map of a z-marching K*u grid g whose CTAs own (TY-1) x (TX-1)
// node columns and zc node layers: a CTA is active iff an element of its box
// -- elements y0-1 .. y0+TY-2, x0-1 .. x0+TX-2, z0-1 .. z0+zc (a superset of
// what any of the kernels reads) -- is active.  One warp per CTA.
__global__ void k_tile_map(const uint8_t *__restrict__ eact, int ny, int nx, int nz, int TY, int TX, int zc,
                           dim3 g, uint8_t *__restrict__ out) {
    const int64_t ntile = (int64_t)g.x * g.y * g.z;
    const int64_t t = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (t >= ntile) return;
    const int lane = threadIdx.x & 31;
    const int bx = (int)(t % g.x), by = (int)((t / g.x) % g.y), bz = (int)(t / ((int64_t)g.x * g.y));
    const int y0 = bx * (TY - 1) - 1, x0 = by * (TX - 1) - 1, z0 = bz * zc - 1;
    bool act = false;
    for (int ly = lane; ly < TY; ly += 32) {
        const int ey = y0 + ly;
        if (ey < 0 || ey >= ny) continue;
        for (int ex = max(x0, 0); ex < min(x0 + TX, nx); ++ex)
            for (int ez = max(z0, 0); ez < min(z0 + zc + 2, nz); ++ez)
                act |= eact[ey + (int64_t)ny * (ex + (int64_t)nx * ez)] != 0;
    }
    act = __any_sync(0xffffffffu, act);
    if (lane == 0) out[t] = act ? 1 : 0;
}

static void make_tile_map(const Level &l, int TY, int TX, int zc, dim3 g, uint8_t *out, cudaStream_t s) {
    const int64_t ntile = (int64_t)g.x * g.y * g.z;
    ++g_launches;
    k_tile_map<<<(unsigned)((ntile + 3) / 4), 128, 0, s>>>(l.eact, l.ny, l.nx, l.nz, TY, TX, zc, g, out);
}

// y = K u on the full grid; y at fixed DOFs is 0.  When DOT, also writes
// sum(u .* y) of this CTA's nodes to partial[block].
template <typename T, bool DOT>
__global__ void __launch_bounds__(KT_THREADS) k_kbyu(const T *__restrict__ u, T *__restrict__ y,
                                                     const T *__restrict__ E, const uint8_t *__restrict__ nflag,
                                                     int ny, int nx, int nz, double *__restrict__ partial,
                                                     const uint8_t *__restrict__ tiles) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *su = reinterpret_cast<T *>(smem_raw);      // [3][KT_NL*3] ring of node layers
    T *so = su + 3 * KT_NL * 3;                   // [24][KT_THREADS]
    const int tid = threadIdx.x;
    const int ty = tid % KT_Y, tx = tid / KT_Y;
    const int NY = ny + 1, NX = nx + 1, NZ = nz + 1;
    const int y0 = blockIdx.x * (KT_Y - 1), x0 = blockIdx.y * (KT_X - 1), z0 = blockIdx.z * KT_ZC;
    const int zend = min(z0 + KT_ZC, NZ);
    const int gny = y0 + ty, gnx = x0 + tx;
    const bool owner = (ty < KT_Y - 1) && (tx < KT_X - 1) && gny < NY && gnx < NX;
    const int ey = y0 - 1 + ty, ex = x0 - 1 + tx;
    const bool ein = ey >= 0 && ey < ny && ex >= 0 && ex < nx;
    if (tiles && !tiles[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)]) {
        skip_tile(y, owner, gny, gnx, NY, NX, z0, zend, DOT ? partial : nullptr);
        return;
    }
    T acc0 = T(0), acc1 = T(0), acc2 = T(0);
    T dot = T(0);

    // staging plan: this thread copies up to KT_SV words of every node layer;
    // the in-layer source offsets are fixed, only the layer stride changes
    int soff[KT_SV];
#pragma unroll
    for (int k = 0; k < KT_SV; ++k) {
        const int i = tid + k * KT_THREADS;
        soff[k] = -2;
        if (i < KT_NL * 3) {
            const int node = i / 3, c = i - 3 * node;
            const int ly = node % (KT_Y + 1), lx = node / (KT_Y + 1);
            const int gy = y0 - 1 + ly, gx = x0 - 1 + lx;
            soff[k] = (gy >= 0 && gy < NY && gx >= 0 && gx < NX) ? 3 * (gy + NY * gx) + c : -1;
        }
    }
    const int64_t lstride = 3 * (int64_t)NY * NX;
    auto stage = [&](int z) {
        T *dst = su + kslot(z) * KT_NL * 3;
        const bool zin = z >= 0 && z < NZ;
#pragma unroll
        for (int k = 0; k < KT_SV; ++k) {
            const int i = tid + k * KT_THREADS;
            if (soff[k] == -2) continue;
            if (zin && soff[k] >= 0)
                async_copy(dst + i, u + ((int64_t)z * lstride + soff[k]));
            else
                dst[i] = T(0);
        }
        async_commit();
    };

    stage(z0 - 1);
    stage(z0);
    async_wait_all();
    __syncthreads();
    for (int ez = z0 - 1; ez < zend; ++ez) {
        const int s0 = kslot(ez), s1 = kslot(ez + 1);
        if (ez + 2 <= zend) stage(ez + 2);   // prefetch, overlaps the element work below
        T ev = T(0);
        if (ein && ez >= 0 && ez < nz) ev = E[(int64_t)ey + (int64_t)ny * (ex + (int64_t)nx * ez)];
        T ue[24];
        if (ev != T(0)) {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int dx = k & 1, dy = 1 - ((k >> 1) & 1), kp = k >> 2;
                const T *src = su + (kp ? s1 : s0) * KT_NL * 3 + 3 * ((ty + dy) + (KT_Y + 1) * (tx + dx));
                ue[3 * k + 0] = src[0];
                ue[3 * k + 1] = src[1];
                ue[3 * k + 2] = src[2];
            }
            hex_apply<T>(ue, ev);
        } else {
#pragma unroll
            for (int i = 0; i < 24; ++i) ue[i] = T(0);
        }
#pragma unroll
        for (int i = 0; i < 24; ++i) so[i * KT_THREADS + tid] = ue[i];
        __syncthreads();
        if (owner) {
            // lower corners (kp = 0) of element layer ez complete node layer ez
#pragma unroll
            for (int dy = 0; dy < 2; ++dy)
#pragma unroll
                for (int dx = 0; dx < 2; ++dx) {
                    const int k = dx | ((1 - dy) << 1);
                    const int t = (ty + 1 - dy) + KT_Y * (tx + 1 - dx);
                    acc0 += so[(3 * k + 0) * KT_THREADS + t];
                    acc1 += so[(3 * k + 1) * KT_THREADS + t];
                    acc2 += so[(3 * k + 2) * KT_THREADS + t];
                }
            if (ez >= z0) {
                const int64_t node = (int64_t)gny + (int64_t)NY * (gnx + (int64_t)NX * ez);
                const uint8_t f = nflag[node];
                const T o0 = (f & NF_FIXX) ? T(0) : acc0;
                const T o1 = (f & NF_FIXY) ? T(0) : acc1;
                const T o2 = (f & NF_FIXZ) ? T(0) : acc2;
                y[3 * node + 0] = o0;
                y[3 * node + 1] = o1;
                y[3 * node + 2] = o2;
                if (DOT) {
                    const T *un = su + s0 * KT_NL * 3 + 3 * ((ty + 1) + (KT_Y + 1) * (tx + 1));
                    dot += un[0] * o0 + un[1] * o1 + un[2] * o2;
                }
            }
            acc0 = acc1 = acc2 = T(0);
#pragma unroll
            for (int dy = 0; dy < 2; ++dy)
#pragma unroll
                for (int dx = 0; dx < 2; ++dx) {
                    const int k = 4 | dx | ((1 - dy) << 1);
                    const int t = (ty + 1 - dy) + KT_Y * (tx + 1 - dx);
                    acc0 += so[(3 * k + 0) * KT_THREADS + t];
                    acc1 += so[(3 * k + 1) * KT_THREADS + t];
                    acc2 += so[(3 * k + 2) * KT_THREADS + t];
                }
        }
        async_wait_all();
        __syncthreads();
    }
    if (DOT) {
        __shared__ double red[KT_THREADS / 32];
        const double s = block_sum_to_double<T>(dot, red);
        if (tid == 0) partial[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = s;
    }
}

// ---- paired FP32 arithmetic -----------------------------------------------------
// Blackwell executes FP32 add / multiply / FMA on register pairs (f32x2) at the
// issue cost of one scalar instruction; the FP32 K*u runs all its element
// arithmetic on such pairs.
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 kh2(int i) { return make_float2(c_Kh32[i], c_Kh32[i]); }

// ---- FP32 K*u in sum-factorised Hadamard form, node rows staged by TMA -------
// The Hadamard transform of an element's 8 corners is a product of three
// 2-point butterflies (x, y, z), and neighbouring elements share most of
// them: the y butterfly of a node pair (an edge along y) serves the 4
// elements around that edge, and the x butterfly of two such edges (an element
// face in a node layer) serves the 2 elements above and below the face.
// k_kbyu_tma forms each of them once.  Per node layer a thread forms the 12
// face coefficients of its element column from 4 node columns; per element
// layer it forms the 24 Hadamard coefficients from the faces below and above
// (12 z butterflies), applies E*Kh and undoes the z butterfly.  The transposed
// transform is shared the same way: the two elements of a face add their face
// contributions before the x butterfly is undone, the two faces of an edge
// add before the y butterfly is undone, and the two edges of a node add last.
// Per element that is 12 staged words read instead of 24, about 110 paired
// FP32 operations instead of 170, and an exchange of 6 float2 through shared
// memory (x) and 3 warp shuffles (y) instead of 12 shuffles and 6 float2.
//
// Every thread carries two independent z streams in the lanes of its float2
// registers: node layers [zA, zA+zc) and [zA+zc, zA+2zc) of the CTA's chunk.
// So all arithmetic runs as paired f32x2 instructions with no lane shuffling.
//
// Staging: a node row (33 nodes x 3 words of one x column in one node layer)
// arrives in a ring slot of shared memory by cp.async.bulk.tensor over a
// rank-1 tensor map of the whole vector, one copy per row, completed on the
// slot's mbarrier.  A rank-1 map is used because the rows of a node layer lie
// 12*NY bytes apart, which is not a multiple of 16 bytes as a tensor map's
// strides must be.  Each copy starts at the 16-byte boundary at or below its
// row (the row's first word lands 0..3 words into the slot row), and words
// outside the vector read as zeros (halo rows and layers past the grid).
// Halo values feed only elements outside the grid, whose modulus is 0.
namespace tk {
constexpr int RING = 4;       // ring slots; loads run up to 3 element layers ahead
constexpr int ROWW = 104;     // words per row copy: up to 3 lead words + 99, a multiple of 4
constexpr int ROWP = 128;     // words per slot row: every copy lands on a 128-byte boundary
constexpr unsigned WAIT_LIMIT = 1u << 22;   // mbarrier tries before a CTA gives up
}  // namespace tk

template <int TX>
struct TkTile {
    static constexpr int THREADS = KT_Y * TX;
    static constexpr int ROWS = TX + 1;                     // node x columns staged per layer
    static constexpr int SLOT_WORDS = 2 * ROWS * tk::ROWP;  // both streams
    static constexpr size_t RING_BYTES = sizeof(float) * tk::RING * SLOT_WORDS;
    static constexpr size_t EXCH_BYTES = sizeof(float2) * 2 * 6 * THREADS;   // double-buffered
    static constexpr size_t SMEM = 128 + RING_BYTES + EXCH_BYTES + sizeof(uint64_t) * tk::RING;
    static constexpr uint32_t SLOT_TX_BYTES = 2 * ROWS * tk::ROWW * sizeof(float);
    static_assert(2 * ROWS <= THREADS, "one producer thread per row");
};

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for the completion of phase `parity`; false after WAIT_LIMIT tries
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (unsigned i = 0; i < tk::WAIT_LIMIT; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void tma_load_1d(uint32_t dst, const CUtensorMap *map, int c0, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.1d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2}], [%3];" ::"r"(
            dst),
        "l"((uint64_t)map), "r"(c0), "r"(bar)
        : "memory");
}

// g = Kh h (g[0..2] = 0: the rigid translations), the 11 blocks of the
// Hadamard-basis element matrix on paired lanes
__device__ __forceinline__ void kh_apply_x2(const float2 (&u)[24], float2 (&g)[24]) {
    g[0] = g[1] = g[2] = make_float2(0.f, 0.f);
#define X3(i, j, k, o)                                                                    \
    {                                                                                     \
        const float2 a = u[i], b = u[j], d = u[k];                                        \
        g[i] = f2fma(kh2(o + 2), d, f2fma(kh2(o + 1), b, f2mul(kh2(o), a)));              \
        g[j] = f2fma(kh2(o + 5), d, f2fma(kh2(o + 4), b, f2mul(kh2(o + 3), a)));          \
        g[k] = f2fma(kh2(o + 8), d, f2fma(kh2(o + 7), b, f2mul(kh2(o + 6), a)));          \
    }
#define X2(i, j, o)                                                  \
    {                                                                \
        const float2 a = u[i], b = u[j];                             \
        g[i] = f2fma(kh2(o + 1), b, f2mul(kh2(o), a));               \
        g[j] = f2fma(kh2(o + 3), b, f2mul(kh2(o + 2), a));           \
    }
    X3(3, 7, 14, 0)
    X2(4, 6, 9)
    X2(5, 12, 13)
    X2(8, 13, 17)
    X2(9, 20, 21)
    X2(10, 17, 25)
    X3(11, 16, 18, 29)
    X2(15, 19, 38)
    g[21] = f2mul(kh2(42), u[21]);
    g[22] = f2mul(kh2(43), u[22]);
    g[23] = f2mul(kh2(44), u[23]);
#undef X3
#undef X2
}

// the same product for an element matrix with cubic symmetry, from its 8 values
// k = (A-B, B, C, D, E, F-G, G, H): a 3-block [[A,B,B],[B,A,B],[B,B,A]] is
// (A-B) u_i + B (u_i + u_j + u_k), a C-block maps both entries to C (u_i + u_j);
// 33 paired operations instead of 49, on 8 constants the thread keeps in registers
__device__ __forceinline__ void kh_apply_cubic_x2(const float2 (&u)[24], float2 (&g)[24], const float2 (&k)[8]) {
    g[0] = g[1] = g[2] = make_float2(0.f, 0.f);
#define Y3(i, j, l, a, b)                                           \
    {                                                               \
        const float2 t = f2mul(k[b], f2add(f2add(u[i], u[j]), u[l])); \
        g[i] = f2fma(k[a], u[i], t);                                \
        g[j] = f2fma(k[a], u[j], t);                                \
        g[l] = f2fma(k[a], u[l], t);                                \
    }
#define YC(i, j)                                   \
    {                                              \
        const float2 t = f2mul(k[2], f2add(u[i], u[j])); \
        g[i] = t;                                  \
        g[j] = t;                                  \
    }
#define YD(i, j)                                        \
    {                                                   \
        g[i] = f2fma(k[4], u[j], f2mul(k[3], u[i]));    \
        g[j] = f2fma(k[4], u[i], f2mul(k[3], u[j]));    \
    }
    Y3(3, 7, 14, 0, 1)
    YC(4, 6)
    YC(5, 12)
    YC(8, 13)
    YD(9, 20)
    YD(10, 17)
    Y3(11, 16, 18, 5, 6)
    YD(15, 19)
    g[21] = f2mul(k[7], u[21]);
    g[22] = f2mul(k[7], u[22]);
    g[23] = f2mul(k[7], u[23]);
#undef Y3
#undef YC
#undef YD
}

template <int TX, bool DOT, bool CUBIC>
__global__ void __launch_bounds__(KT_Y * TX, TX == 8 ? 2 : 1)
    k_kbyu_tma(const __grid_constant__ CUtensorMap umap, float *__restrict__ y, const float *__restrict__ E,
               const uint8_t *__restrict__ nflag, int ny, int nx, int nz, int zc, double *__restrict__ partial,
               const uint8_t *__restrict__ tiles, int *__restrict__ err) {
    using G = TkTile<TX>;
    constexpr int THREADS = G::THREADS, ROWS = G::ROWS;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((128u - (smem_addr(smem_raw) & 127u)) & 127u);
    float *ring = reinterpret_cast<float *>(base);
    float2 *exch = reinterpret_cast<float2 *>(base + G::RING_BYTES);
    uint64_t *bars = reinterpret_cast<uint64_t *>(base + G::RING_BYTES + G::EXCH_BYTES);
    __shared__ int s_abort;
    const int tid = threadIdx.x;
    const int ty = tid % KT_Y, tx = tid / KT_Y;
    const int NY = ny + 1, NX = nx + 1, NZ = nz + 1;
    const int y0 = blockIdx.x * (KT_Y - 1), x0 = blockIdx.y * (TX - 1);
    const int zA = blockIdx.z * 2 * zc, zB = zA + zc;
    const int gny = y0 + ty, gnx = x0 + tx;
    const bool owner = ty < KT_Y - 1 && tx < TX - 1 && gny < NY && gnx < NX;
    // the output keeps exact zeros at inactive nodes (it is zeroed when allocated and no
    // launch writes there): a tile without active elements writes nothing
    if (tiles && !tiles[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)]) {
        if (DOT && tid == 0) partial[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = 0.0;
        return;
    }
    const int ey = y0 - 1 + ty, ex = x0 - 1 + tx;
    const bool ein = ey >= 0 && ey < ny && ex >= 0 && ex < nx;
    const int nload = zc + 2;   // node layers zs-1 .. zs+zc of each stream
    const int64_t lwords = 3 * (int64_t)NY * NX;
    if (tid == 0) {
        for (int i = 0; i < tk::RING; ++i) mbar_init(smem_addr(bars + i), 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // row p (row p % ROWS of stream p / ROWS) is copied by lane p / NW of warp p % NW, so that
    // every warp issues 2 or 3 copies
    constexpr int NW = THREADS / 32;
    const int prow = (tid & 31) * NW + (tid >> 5);
    const bool producer = prow < 2 * ROWS;
    int64_t pw = 0;   // word index of the row's first node (y0-1, x0-1+row) in the stream's layer zs-1
    if (producer) {
        const int zs = prow < ROWS ? zA : zB;
        pw = 3 * ((int64_t)(y0 - 1) + (int64_t)NY * (x0 - 1 + prow % ROWS)) + lwords * (zs - 1);
    }
    auto issue = [&](int i) {   // load i: node layer zs-1+i of both streams into slot i % RING
        const int slot = i % tk::RING;
        const uint32_t bar = smem_addr(bars + slot);
        if (tid == 0) mbar_expect_tx(bar, G::SLOT_TX_BYTES);
        if (producer) {
            const int64_t w = pw + lwords * i;
            tma_load_1d(smem_addr(ring + slot * G::SLOT_WORDS + prow * tk::ROWP), &umap,
                        (int)(w & ~(int64_t)3), bar);
        }
    };
    int issued = 0, waited = 0;   // loads issued; loads this thread has waited for
    for (; issued < min(tk::RING, nload); ++issued) issue(issued);
    // every thread waits for a load right before reading it; a wait that gives up raises
    // s_abort, which the CTA acts on after its next barrier
    auto wait_load = [&](int i) -> bool {
        const bool ok = mbar_wait(smem_addr(bars + i % tk::RING), (uint32_t)((i / tk::RING) & 1));
        waited = i + 1;
        return ok;
    };
    // after a wait that gave up: thread 0 lets the copies in flight land and flags the
    // error; the CTA's nodes (and dot partial) read NaN, so that a solve using this
    // product stops and falls back instead of going on with a wrong one
    auto bail = [&]() {
        if (tid == 0) {
            for (int i = waited; i < issued; ++i) wait_load(i);
            if (err) atomicExch(err, 1);
            if (DOT) partial[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = __longlong_as_double(0x7ff8000000000000ll);
        }
        if (owner)
            for (int z = zA; z < min(zA + 2 * zc, NZ); ++z) {
                const int64_t node = (int64_t)gny + (int64_t)NY * (gnx + (int64_t)NX * z);
                if (!(nflag[node] & NF_ACTIVE)) continue;
                float *o = y + 3 * node;
                o[0] = o[1] = o[2] = __int_as_float(0x7fc00000);
            }
    };
    // this thread reads node rows tx and tx+1 of each stream at words 3*ty + lead, where the
    // lead (0..3 words) follows the row's start address modulo 16 bytes
    // (the other rows and the other stream sit at fixed offsets from row tx of stream A, and
    // their leads differ from its lead by per-CTA constants)
    const int roff = tx * tk::ROWP + 3 * ty;
    const int64_t w00 = 3 * ((int64_t)(y0 - 1) + (int64_t)NY * (x0 - 1 + tx)) + lwords * (zA - 1);
    const int lead00 = (int)(w00 & 3);
    const int dr = (3 * NY) & 3, ds = (int)((lwords * zc) & 3);   // lead steps: next row, stream B
    const int lstep = (int)(lwords & 3);                          // lead step: next layer
    // the 12 face coefficients (x, y Hadamard) of node layer zs-1+i, both streams; also the
    // values of node (ey+1, ex+1) in that layer
    auto faces = [&](int i, float2 (&F)[12], float2 (&un)[3]) {
        if (!wait_load(i)) s_abort = 1;
        const float *sl = ring + (i % tk::RING) * G::SLOT_WORDS + roff;
        const int li = lead00 + lstep * i;
        float2 v[2][2][3];   // [row][node ey, ey+1][c]
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const float *pa = sl + r * tk::ROWP + ((li + r * dr) & 3);
            const float *pb = sl + (ROWS + r) * tk::ROWP + ((li + r * dr + ds) & 3);
#pragma unroll
            for (int n = 0; n < 2; ++n)
#pragma unroll
                for (int c = 0; c < 3; ++c) v[r][n][c] = make_float2(pa[3 * n + c], pb[3 * n + c]);
        }
        // y butterfly (bit 1 = node ey): sum and u(ey) - u(ey+1); then x butterfly
        // (bit 0 = column ex+1): sum and v(ex+1) - v(ex)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float2 s0 = f2add(v[0][0][c], v[0][1][c]), d0 = f2sub(v[0][0][c], v[0][1][c]);
            const float2 s1 = f2add(v[1][0][c], v[1][1][c]), d1 = f2sub(v[1][0][c], v[1][1][c]);
            F[c] = f2add(s0, s1);
            F[3 + c] = f2sub(s1, s0);
            F[6 + c] = f2add(d0, d1);
            F[9 + c] = f2sub(d1, d0);
            un[c] = v[1][1][c];
        }
    };
    float2 kc[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) kc[i] = CUBIC ? make_float2(c_Kc32[i], c_Kc32[i]) : make_float2(0.f, 0.f);
    float2 Fp[12], carry[12], uo[3];
    faces(0, Fp, uo);   // a wait that gave up here is acted on after step 0's barrier
#pragma unroll
    for (int i = 0; i < 12; ++i) carry[i] = make_float2(0.f, 0.f);
    float dot = 0.f;
    // moduli of element layer zs-1+j and flags of node layer zs-1+j, loaded a step ahead
    // through pointers that advance one layer per step
    // (32-bit offsets: the launcher keeps every word index of the vector below 2^31)
    const int eplane = ny * nx, nplane = NY * NX;
    int eoA = (ey + ny * ex) + eplane * (zA - 1), eoB = eoA + eplane * zc;
    int noA = (gny + NY * gnx) + nplane * (zA - 1), noB = noA + nplane * zc;
    auto emod = [&](int o, int k) -> float { return (ein && k >= 0 && k < nz) ? E[o] : 0.f; };
    // the raw flag byte, or -1 (not owned, past the grid); nothing uses the loaded byte
    // until the next step, so the load's latency stays hidden
    auto flag = [&](int o, int z) -> int { return (owner && z >= 0 && z < NZ) ? (int)nflag[o] : -1; };
    float2 en = make_float2(emod(eoA, zA - 1), emod(eoB, zB - 1));
    int fnA = -1, fnB = -1;
#pragma unroll 2
    for (int j = 0; j <= zc; ++j) {
        // element layer zs-1+j: faces of node layers zs-1+j (Fp) and zs+j (Ft)
        const float2 ev = en;
        const int fA = fnA, fB = fnB;
        eoA += eplane;
        eoB += eplane;
        if (j < zc) {
            en = make_float2(emod(eoA, zA + j), emod(eoB, zB + j));
            fnA = flag(noA + nplane, zA + j);
            fnB = flag(noB + nplane, zB + j);
        }
        float2 Ft[12], un[3];
        faces(j + 1, Ft, un);
        float2 h[24];
#pragma unroll
        for (int i = 0; i < 12; ++i) {
            h[i] = f2add(Fp[i], Ft[i]);
            h[12 + i] = f2sub(Ft[i], Fp[i]);
            Fp[i] = Ft[i];
        }
        float2 g[24];
        if constexpr (CUBIC)
            kh_apply_cubic_x2(h, g, kc);
        else
            kh_apply_x2(h, g);
        // E scale, z butterfly undone: the face below gets (a - d), the face above (a + d);
        // the face below also takes the carried contribution of the element layer under it
        float2 Lm[6], Rp[6];
#pragma unroll
        for (int by = 0; by < 2; ++by)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float2 phi[2];
#pragma unroll
                for (int bx = 0; bx < 2; ++bx) {
                    const int i = 3 * (bx | (by << 1)) + c;
                    phi[bx] = f2fma(ev, f2sub(g[i], g[12 + i]), carry[i]);
                    carry[i] = f2mul(ev, f2add(g[i], g[12 + i]));
                }
                // x butterfly undone: column ex gets phi0 - phi1, column ex+1 gets phi0 + phi1
                Lm[3 * by + c] = f2sub(phi[0], phi[1]);
                Rp[3 * by + c] = f2add(phi[0], phi[1]);
            }
        float2 *xb = exch + (j & 1) * 6 * THREADS;
#pragma unroll
        for (int v = 0; v < 6; ++v) xb[v * THREADS + tid] = Lm[v];
        __syncthreads();
        if (s_abort) {
            bail();
            return;
        }
        // slots whose loads are consumed take the next ones
        while (issued < nload && issued <= j + 1 + tk::RING) issue(issued++);
        if (j >= 1 && tx < TX - 1) {
            // edge of column ex+1 along y: this element's right face part + the next column's left part;
            // y butterfly undone: node ey+1 gets T0 - T1, node ey gets T0 + T1
            float2 o[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float2 t0 = f2add(Rp[c], xb[c * THREADS + tid + KT_Y]);
                const float2 t1 = f2add(Rp[3 + c], xb[(3 + c) * THREADS + tid + KT_Y]);
                const float2 up = f2add(t0, t1);
                o[c] = f2add(f2sub(t0, t1), make_float2(__shfl_down_sync(0xffffffffu, up.x, 1),
                                                        __shfl_down_sync(0xffffffffu, up.y, 1)));
            }
            // node layer zs-1+j of each stream is complete
            if (fA >= 0 && (fA & NF_ACTIVE)) {   // inactive nodes are never written
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float oc = (fA & (NF_FIXX << c)) ? 0.f : o[c].x;
                    y[3 * noA + c] = oc;
                    if (DOT) dot = fmaf(uo[c].x, oc, dot);
                }
            }
            if (fB >= 0 && (fB & NF_ACTIVE)) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float oc = (fB & (NF_FIXX << c)) ? 0.f : o[c].y;
                    y[3 * noB + c] = oc;
                    if (DOT) dot = fmaf(uo[c].y, oc, dot);
                }
            }
        }
        noA += nplane;
        noB += nplane;
#pragma unroll
        for (int c = 0; c < 3; ++c) uo[c] = un[c];
    }
    if (DOT) {
        __shared__ double red[THREADS / 32];
        const double s = block_sum_to_double<float>(dot, red);
        if (tid == 0) partial[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = s;
    }
}

// node layers per stream of k_kbyu_tma (a CTA covers two streams): about 32
// node layers per CTA, balanced over the z extent
static int kbyu_tma_zc(int NZ) {
    const int chunks = (NZ + 31) / 32;
    return (NZ + 2 * chunks - 1) / (2 * chunks);
}

// sgld_assemble's tuner (tune_kbyu_f32) may set another chunk per level
int kbyu_f32_zc(const Level &l) { return l.kx_zc > 0 ? l.kx_zc : kbyu_tma_zc(l.nz + 1); }
// tile width in x: 8 unless the tuner chose 16
int kbyu_f32_tx(const Level &l) { return l.kx_tx == 16 ? 16 : 8; }
// node layers one CTA of the FP32 K*u covers (two streams)
int kbyu_f32_cta_layers(const Level &l) { return 2 * kbyu_f32_zc(l); }

static dim3 kbyu_f32_grid(const Level &l) {
    const int NZ = l.nz + 1;
    const int zl = kbyu_f32_cta_layers(l), tx = kbyu_f32_tx(l);
    return dim3((l.ny + 1 + KT_Y - 2) / (KT_Y - 1), (l.nx + 1 + tx - 2) / (tx - 1), (NZ + zl - 1) / zl);
}

static dim3 kbyu_grid(const Level &l) {
    return dim3((l.ny + 1 + KT_Y - 2) / (KT_Y - 1), (l.nx + 1 + KT_X - 2) / (KT_X - 1), (l.nz + 1 + KT_ZC - 1) / KT_ZC);
}

template <typename T>
static constexpr size_t kbyu_smem() {
    return sizeof(T) * (3 * KT_NL * 3 + 24 * KT_THREADS);
}

template <int TX, bool DOT, bool CUBIC>
static void tma_attributes() {
    cudaFuncSetAttribute(k_kbyu_tma<TX, DOT, CUBIC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)TkTile<TX>::SMEM);
}

// opt-in shared memory sizes; called once per context before any launch or
// graph capture
void init_kernel_attributes() {
    cudaFuncSetAttribute(k_kbyu<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kbyu_smem<double>());
    cudaFuncSetAttribute(k_kbyu<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kbyu_smem<double>());
    tma_attributes<8, true, false>();
    tma_attributes<8, false, false>();
    tma_attributes<16, true, false>();
    tma_attributes<16, false, false>();
    tma_attributes<8, true, true>();
    tma_attributes<8, false, true>();
    tma_attributes<16, true, true>();
    tma_attributes<16, false, true>();
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library); null when the driver does not provide it
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// Rank-1 tensor map of the n FP32 words at u with boxes of tk::ROWW words;
// words outside [0, n) read as zeros.  TMA coordinates are 32-bit, so n is
// limited to 2^31 - 1 words.
static int vector_tensor_map(CUtensorMap *m, const float *u, int64_t n) {
    const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc || n <= 0 || n > (int64_t)INT32_MAX || (reinterpret_cast<uintptr_t>(u) & 15)) return -1;
    const cuuint64_t dim[1] = {(cuuint64_t)n};
    const cuuint64_t stride[1] = {(cuuint64_t)sizeof(float)};   // no strides at rank 1
    const cuuint32_t box[1] = {(cuuint32_t)tk::ROWW}, estride[1] = {1};
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 1, const_cast<float *>(u), dim, stride, box, estride,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? 0 : -1;
}

template <typename T, bool DOT>
static void kbyu_launch(const Level &l0, const T *E, const T *u, T *y, double *partial, int *nb, cudaStream_t s) {
    const size_t smem = kbyu_smem<T>();
    dim3 g = kbyu_grid(l0);
    if (nb) *nb = (int)(g.x * g.y * g.z);
    ++g_launches;
    k_kbyu<T, DOT><<<g, KT_THREADS, smem, s>>>(u, y, E, l0.nflag, l0.ny, l0.nx, l0.nz, partial, l0.tiles16);
}

void launch_kbyu_f64(const Level &l0, const double *E, const double *u, double *y, double *partial_dot,
                     int *nblocks_out, cudaStream_t s) {
    if (partial_dot)
        kbyu_launch<double, true>(l0, E, u, y, partial_dot, nblocks_out, s);
    else
        kbyu_launch<double, false>(l0, E, u, y, nullptr, nblocks_out, s);
}

template <int TX, bool DOT, bool CUBIC>
static void tma_launch(dim3 g, const CUtensorMap &m, float *y, const float *E, const Level &l0, int zc,
                       double *partial_dot, const uint8_t *tiles, cudaStream_t s) {
    using G = TkTile<TX>;
    k_kbyu_tma<TX, DOT, CUBIC><<<g, G::THREADS, G::SMEM, s>>>(m, y, E, l0.nflag, l0.ny, l0.nx, l0.nz, zc, partial_dot,
                                                              tiles, l0.kerr);
}

int launch_kbyu_f32(const Level &l0, const float *E, const float *u, float *y, double *partial_dot,
                    int *nblocks_out, cudaStream_t s) {
    const dim3 g = kbyu_f32_grid(l0);
    const int zc = kbyu_f32_zc(l0), tx = kbyu_f32_tx(l0);
    if (nblocks_out) *nblocks_out = (int)(g.x * g.y * g.z);
    // the tile map only when it was made for this tile
    const uint8_t *tiles = (l0.tiles_f32 && l0.tiles_f32_tx == tx && l0.tiles_f32_zc == zc) ? l0.tiles_f32 : nullptr;
    // every row coordinate the CTAs form (up to 2 zc + 2 layers past the grid) must fit 32 bits
    const int64_t lw = 3 * (int64_t)(l0.ny + 1) * (l0.nx + 1);
    if (3 * l0.nnode + lw * (2 * (int64_t)zc + 2) >= (int64_t)INT32_MAX) return (int)cudaErrorInvalidValue;
    CUtensorMap m;
    if (vector_tensor_map(&m, u, 3 * l0.nnode)) return (int)cudaErrorInvalidValue;
    ++g_launches;
    const bool cubic = l0.kh_cubic;
    if (tx == 8) {
        if (partial_dot)
            cubic ? tma_launch<8, true, true>(g, m, y, E, l0, zc, partial_dot, tiles, s)
                  : tma_launch<8, true, false>(g, m, y, E, l0, zc, partial_dot, tiles, s);
        else
            cubic ? tma_launch<8, false, true>(g, m, y, E, l0, zc, nullptr, tiles, s)
                  : tma_launch<8, false, false>(g, m, y, E, l0, zc, nullptr, tiles, s);
    } else {
        if (partial_dot)
            cubic ? tma_launch<16, true, true>(g, m, y, E, l0, zc, partial_dot, tiles, s)
                  : tma_launch<16, true, false>(g, m, y, E, l0, zc, partial_dot, tiles, s);
        else
            cubic ? tma_launch<16, false, true>(g, m, y, E, l0, zc, nullptr, tiles, s)
                  : tma_launch<16, false, false>(g, m, y, E, l0, zc, nullptr, tiles, s);
    }
    return 0;
}

int update_kbyu_tiles(Level &l0, cudaStream_t s) {
    cudaError_t e = cudaSuccess;
    const dim3 g16 = kbyu_grid(l0);
    if (!l0.tiles16) {
        e = cudaMalloc((void **)&l0.tiles16, (size_t)g16.x * g16.y * g16.z);
        if (e != cudaSuccess) return (int)e;
        make_tile_map(l0, KT_Y, KT_X, KT_ZC, g16, l0.tiles16, s);
    }
    if (!l0.kerr) {
        e = cudaMalloc((void **)&l0.kerr, sizeof(int));
        if (e != cudaSuccess) return (int)e;
        e = cudaMemsetAsync(l0.kerr, 0, sizeof(int), s);
        if (e != cudaSuccess) return (int)e;
    }
    const int tx = kbyu_f32_tx(l0), zc = kbyu_f32_zc(l0);
    if (l0.tiles_f32 && l0.tiles_f32_tx == tx && l0.tiles_f32_zc == zc) return 0;
    const dim3 g = kbyu_f32_grid(l0);
    const int64_t n = (int64_t)g.x * g.y * g.z;
    if (n > l0.tiles_f32_cap) {
        if (l0.tiles_f32) cudaFree(l0.tiles_f32);
        l0.tiles_f32 = nullptr;
        l0.tiles_f32_cap = 0;
        e = cudaMalloc((void **)&l0.tiles_f32, (size_t)n);
        if (e != cudaSuccess) return (int)e;
        l0.tiles_f32_cap = n;
    }
    make_tile_map(l0, KT_Y, tx, kbyu_f32_cta_layers(l0), g, l0.tiles_f32, s);
    l0.tiles_f32_tx = tx;
    l0.tiles_f32_zc = zc;
    return (int)cudaGetLastError();
}

int kbyu_num_blocks(const Level &l0) {
    dim3 g = kbyu_grid(l0);
    return (int)(g.x * g.y * g.z);
}

// ---------------------------------------------------------------------------
// unit compliance ce_e = u_e' Ke u_e (TopOpti_CmptUnitCompliance_mex.cpp:40-107)
// and the weighted sum c = sum E_e ce_e (FEA_ComputeComplianceVoxel.m:20-22).
// One thread per element; in the Hadamard basis u'Ke u = h' Kh h with h = H u.
// ---------------------------------------------------------------------------
__global__ void k_unit_compliance(const double *__restrict__ u, const double *__restrict__ E,
                                  const uint8_t *__restrict__ eact, int ny, int nx, int nz,
                                  double *__restrict__ ce, double *__restrict__ partial) {
    const int64_t nel = (int64_t)ny * nx * nz;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double cs = 0.0;
    if (e < nel && eact[e]) {
        const int ey = (int)(e % ny), ex = (int)((e / ny) % nx), ez = (int)(e / ((int64_t)ny * nx));
        const int NY = ny + 1, NX = nx + 1;
        double ue[24], h[24];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int dx = k & 1, dy = 1 - ((k >> 1) & 1), dz = k >> 2;
            const int64_t n = (int64_t)(ey + dy) + (int64_t)NY * ((ex + dx) + (int64_t)NX * (ez + dz));
            ue[3 * k] = u[3 * n];
            ue[3 * k + 1] = u[3 * n + 1];
            ue[3 * k + 2] = u[3 * n + 2];
            h[3 * k] = ue[3 * k];
            h[3 * k + 1] = ue[3 * k + 1];
            h[3 * k + 2] = ue[3 * k + 2];
        }
        hex_apply<double>(h, 1.0);
        double q = 0.0;
#pragma unroll
        for (int i = 0; i < 24; ++i) q += ue[i] * h[i];
        ce[e] = q;
        cs = E[e] * q;
    } else if (e < nel) {
        ce[e] = 0.0;
    }
    __shared__ double red[8];
    const double s = block_sum<double>(cs, red);
    if (threadIdx.x == 0 && partial) partial[blockIdx.x] = s;
}

void launch_unit_compliance(const Level &l0, const double *u, const double *E, double *ce_full, double *partial,
                            int *nblocks_out, cudaStream_t s) {
    const int64_t nel = l0.nel;
    const int nb = (int)((nel + 255) / 256);
    if (nblocks_out) *nblocks_out = nb;
    ++g_launches;
    k_unit_compliance<<<nb, 256, 0, s>>>(u, E, l0.eact, l0.ny, l0.nx, l0.nz, ce_full, partial);
}

// ---------------------------------------------------------------------------
// stress recovery (src/FEA_StressAnalysis.m:29-60): per element, corner
// stresses = E_e * inv(sFM) * D * B * u_e (48 values); nodal stress = sum
// over the elements sharing the node / their count; nodal von Mises.
// Node-centric gather: each node thread recomputes the corner stresses of its
// (at most 8) elements restricted to its own corner -> deterministic.
// ---------------------------------------------------------------------------
__global__ void k_nodal_stress(const double *__restrict__ u, const double *__restrict__ E,
                               const uint8_t *__restrict__ nflag, const uint8_t *__restrict__ eact, int ny, int nx,
                               int nz, double *__restrict__ s6,
                               double *__restrict__ vm) {
    const int NY = ny + 1, NX = nx + 1, NZ = nz + 1;
    const int64_t nn = (int64_t)NY * NX * NZ;
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const int iy = (int)(n % NY), ix = (int)((n / NY) % NX), iz = (int)(n / ((int64_t)NY * NX));
    double acc[6] = {0, 0, 0, 0, 0, 0};
    int cnt = 0;
    if (nflag[n] & NF_ACTIVE) {
        // reference corner order j: offsets (dy, dx, dz)
        const int cdy[8] = {1, 1, 0, 0, 1, 1, 0, 0}, cdx[8] = {0, 1, 1, 0, 0, 1, 1, 0},
                  cdz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
        for (int j = 0; j < 8; ++j) {
            const int ey = iy - cdy[j], ex = ix - cdx[j], ez = iz - cdz[j];
            if (ey < 0 || ex < 0 || ez < 0 || ey >= ny || ex >= nx || ez >= nz) continue;
            const int64_t eidx = (int64_t)ey + (int64_t)ny * (ex + (int64_t)nx * ez);
            if (!eact[eidx]) continue;
            const double ev = E[eidx];
            ++cnt;
            double ue[24];
            for (int k = 0; k < 8; ++k) {
                const int64_t m = (int64_t)(ey + cdy[k]) + (int64_t)NY * ((ex + cdx[k]) + (int64_t)NX * (ez + cdz[k]));
                ue[3 * k] = u[3 * m];
                ue[3 * k + 1] = u[3 * m + 1];
                ue[3 * k + 2] = u[3 * m + 2];
            }
            for (int c = 0; c < 6; ++c) {
                const double *row = c_M + (6 * j + c);   // column-major 48 x 24
                double sacc = 0.0;
                for (int i = 0; i < 24; ++i) sacc += row[48 * i] * ue[i];
                acc[c] += sacc * ev;
            }
        }
    }
    double v[6];
    for (int c = 0; c < 6; ++c) v[c] = cnt ? acc[c] / (double)cnt : 0.0;
    for (int c = 0; c < 6; ++c) s6[6 * n + c] = v[c];
    const double a = v[0] - v[1], b = v[1] - v[2], d = v[2] - v[0];
    vm[n] = cnt ? sqrt(0.5 * (a * a + b * b + d * d) + 3.0 * (v[5] * v[5] + v[3] * v[3] + v[4] * v[4])) : 0.0;
}

void launch_stress(const Level &l0, const double *E, const double *u, const double *M48x24, double *nodal6,
                   double *vm_node, cudaStream_t s) {
    cudaMemcpyToSymbolAsync(c_M, M48x24, sizeof(double) * 48 * 24, 0, cudaMemcpyHostToDevice, s);
    const int64_t nn = l0.nnode;
    ++g_launches;
    k_nodal_stress<<<(unsigned)((nn + 127) / 128), 128, 0, s>>>(u, E, l0.nflag, l0.eact, l0.ny, l0.nx, l0.nz, nodal6, vm_node);
}

// per-element: centroid stress = mean of the 8 nodal stresses, von Mises,
// then the reference's extra square root (FEA_ComputePerElementVonMisesStress.m:10-19).
__global__ void k_elem_vm(const double *__restrict__ s6, const uint8_t *__restrict__ eact, int ny, int nx, int nz,
                          double *__restrict__ vme) {
    const int64_t nel = (int64_t)ny * nx * nz;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= nel) return;
    if (!eact[e]) {
        vme[e] = 0.0;
        return;
    }
    const int ey = (int)(e % ny), ex = (int)((e / ny) % nx), ez = (int)(e / ((int64_t)ny * nx));
    const int NY = ny + 1, NX = nx + 1;
    const int cdy[8] = {1, 1, 0, 0, 1, 1, 0, 0}, cdx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cdz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    double v[6] = {0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 8; ++k) {
        const int64_t m = (int64_t)(ey + cdy[k]) + (int64_t)NY * ((ex + cdx[k]) + (int64_t)NX * (ez + cdz[k]));
        for (int c = 0; c < 6; ++c) v[c] += 0.125 * s6[6 * m + c];
    }
    const double a = v[0] - v[1], b = v[1] - v[2], d = v[2] - v[0];
    vme[e] = sqrt(sqrt(0.5 * (a * a + b * b + d * d) + 3.0 * (v[5] * v[5] + v[3] * v[3] + v[4] * v[4])));
}

void launch_elem_vm(const Level &l0, const double *nodal6, double *vm_elem_full, cudaStream_t s) {
    const int64_t nel = l0.nel;
    ++g_launches;
    k_elem_vm<<<(unsigned)((nel + 255) / 256), 256, 0, s>>>(nodal6, l0.eact, l0.ny, l0.nx, l0.nz, vm_elem_full);
}

}  // namespace sgld
