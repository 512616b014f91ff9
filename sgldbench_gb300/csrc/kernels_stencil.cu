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
#include "sgld_internal.cuh"

namespace sgld {

__constant__ double c_Kh[KH_NNZ];
__constant__ float c_Kh32[KH_NNZ];
__constant__ double c_M[48 * 24];   // stress: corner stresses = M * u_e (reference corner order)

void upload_kh(const double *Kh, cudaStream_t s) {
    float f[KH_NNZ];
    for (int i = 0; i < KH_NNZ; ++i) f[i] = (float)Kh[i];
    cudaMemcpyToSymbolAsync(c_Kh, Kh, sizeof(double) * KH_NNZ, 0, cudaMemcpyHostToDevice, s);
    cudaMemcpyToSymbolAsync(c_Kh32, f, sizeof(float) * KH_NNZ, 0, cudaMemcpyHostToDevice, s);
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

// ---- FP32 K*u on packed pairs of element layers -------------------------------
// Blackwell executes FP32 add / multiply / FMA on register pairs (f32x2) at the
// issue cost of one scalar instruction.  k_kbyu_x2 gives every thread two
// elements, (ez, ez+1) of the same (y, x) column, packed as float2 lanes, so
// the Hadamard butterflies, the Kh blocks and the modulus scaling all run as
// paired instructions; the shared-memory exchange moves float2 as well.
// Pair p of a CTA covers element layers z0-1+2p and z0+2p and completes node
// layers z0-1+2p and z0+2p: node layer ez takes the lower corners of element
// ez plus the upper corners of element ez-1 (carried from the previous pair).
// The corner sums are gathered in two steps: along y inside the warp (lanes
// are consecutive y, so the neighbour's corner arrives by a shuffle), then
// along x through shared memory (the next warp is the next x column), which
// leaves 6 float2 per thread in shared memory instead of 24.
// The tile is 32 (y) x TX (x) elements; a CTA owns 31 x (TX-1) node columns,
// so a wider tile recomputes fewer halo elements (15 % at TX = 8, 9 % at 16)
// and stages fewer halo nodes, at the same 1024 threads per SM.
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 kh2(int i) { return make_float2(c_Kh32[i], c_Kh32[i]); }

__device__ __forceinline__ void hex_apply_x2(float2 (&u)[24], float2 e) {
#pragma unroll
    for (int ax = 0; ax < 3; ++ax)
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (k & (1 << ax)) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float2 lo = u[3 * k + c], hi = u[3 * (k | (1 << ax)) + c];
                u[3 * k + c] = f2add(lo, hi);
                u[3 * (k | (1 << ax)) + c] = f2sub(hi, lo);
            }
        }
    float2 g[24];
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
#pragma unroll
    for (int i = 3; i < 24; ++i) g[i] = f2mul(g[i], e);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax)
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (k & (1 << ax)) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float2 a = g[3 * k + c], d = g[3 * (k | (1 << ax)) + c];
                g[3 * k + c] = f2sub(a, d);
                g[3 * (k | (1 << ax)) + c] = f2add(a, d);
            }
        }
#pragma unroll
    for (int i = 0; i < 24; ++i) u[i] = g[i];
}

constexpr int KX_RING = 5;   // node-layer slots: 3 in use + 2 in flight

// geometry of the 32 x TX tile
template <int TX>
struct KxTile {
    static constexpr int THREADS = KT_Y * TX;
    static constexpr int NL = (KT_Y + 1) * (TX + 1);             // staged nodes per layer
    static constexpr int SV = (NL * 3 + THREADS - 1) / THREADS;  // staged words per thread and layer
    // floats of the ring, rounded up to 16 bytes so that the float2 exchange
    // area behind it is aligned (5 * 891 floats alone would leave it 4 bytes off)
    static constexpr int RING_FLOATS = ((KX_RING * NL * 3 + 3) / 4) * 4;
    static constexpr size_t SMEM = sizeof(float) * RING_FLOATS + sizeof(float2) * 6 * THREADS;
    static_assert((RING_FLOATS * sizeof(float)) % 16 == 0, "float2 exchange area must be aligned");
};

__device__ __forceinline__ int xslot(int z) { return (z + KX_RING) % KX_RING; }

template <int TX, bool DOT>
__global__ void __launch_bounds__(KT_Y * TX, 1024 / (KT_Y * TX))
    k_kbyu_x2(const float *__restrict__ u, float *__restrict__ y, const float *__restrict__ E,
              const uint8_t *__restrict__ nflag, int ny, int nx, int nz, int zc, double *__restrict__ partial,
              const uint8_t *__restrict__ tiles) {
    using G = KxTile<TX>;
    constexpr int KT_X = TX, KT_THREADS = G::THREADS, KT_NL = G::NL, KT_SV = G::SV;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *su = reinterpret_cast<float *>(smem_raw);                  // [KX_RING][KT_NL*3]
    float2 *so = reinterpret_cast<float2 *>(su + G::RING_FLOATS);   // [6][KT_THREADS]
    const int tid = threadIdx.x;
    const int ty = tid % KT_Y, tx = tid / KT_Y;
    const int NY = ny + 1, NX = nx + 1, NZ = nz + 1;
    const int y0 = blockIdx.x * (KT_Y - 1), x0 = blockIdx.y * (KT_X - 1), z0 = blockIdx.z * zc;
    const int zend = min(z0 + zc, NZ);
    const int npair = (zend - z0 + 2) / 2;   // element layers z0-1 .. zend-1
    const int zlast = z0 + 2 * npair - 1;    // highest node layer the pairs read
    const int gny = y0 + ty, gnx = x0 + tx;
    const bool owner = (ty < KT_Y - 1) && (tx < KT_X - 1) && gny < NY && gnx < NX;
    const int ey = y0 - 1 + ty, ex = x0 - 1 + tx;
    const bool ein = ey >= 0 && ey < ny && ex >= 0 && ex < nx;
    if (tiles && !tiles[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)]) {
        skip_tile(y, owner, gny, gnx, NY, NX, z0, zend, DOT ? partial : nullptr);
        return;
    }
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
        float *dst = su + xslot(z) * KT_NL * 3;
        const bool zin = z >= 0 && z < NZ;
#pragma unroll
        for (int k = 0; k < KT_SV; ++k) {
            const int i = tid + k * KT_THREADS;
            if (soff[k] == -2) continue;
            if (zin && soff[k] >= 0)
                async_copy(dst + i, u + ((int64_t)z * lstride + soff[k]));
            else
                dst[i] = 0.f;
        }
    };
    stage(z0 - 1);
    stage(z0);
    stage(z0 + 1);
    async_commit();
    async_wait_all();
    __syncthreads();
    float carry[3] = {0.f, 0.f, 0.f};
    float dot = 0.f;
    const int64_t eplane = (int64_t)ny * nx;
    const int64_t ecol = (int64_t)ey + (int64_t)ny * ex;
    // moduli of the next pair are loaded one step ahead (register double buffer)
    auto emod = [&](int z) -> float { return (ein && z >= 0 && z < nz) ? E[ecol + eplane * z] : 0.f; };
    float en0 = emod(z0 - 1), en1 = emod(z0);
    for (int p = 0; p < npair; ++p) {
        const int ez = z0 - 1 + 2 * p;
        if (ez + 3 <= zlast) stage(ez + 3);
        if (ez + 4 <= zlast) stage(ez + 4);
        async_commit();
        const float e0 = en0, e1 = en1;
        en0 = emod(ez + 2);
        en1 = emod(ez + 3);
        float2 ue[24];
        if (e0 != 0.f || e1 != 0.f) {
            const float *l0 = su + xslot(ez) * KT_NL * 3, *l1 = su + xslot(ez + 1) * KT_NL * 3,
                        *l2 = su + xslot(ez + 2) * KT_NL * 3;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int dx = k & 1, dy = 1 - ((k >> 1) & 1), kp = k >> 2;
                const int o = 3 * ((ty + dy) + (KT_Y + 1) * (tx + dx));
                const float *a = kp ? l1 : l0, *b = kp ? l2 : l1;
#pragma unroll
                for (int c = 0; c < 3; ++c) ue[3 * k + c] = make_float2(a[o + c], b[o + c]);
            }
            hex_apply_x2(ue, make_float2(e0, e1));
        } else {
#pragma unroll
            for (int i = 0; i < 24; ++i) ue[i] = make_float2(0.f, 0.f);
        }
        // y step: Y_dx = corner (dx, dy=1) of this element + corner (dx, dy=0)
        // of the element one lane up (corner k = dx | (1-dy) << 1 | kp << 2)
        float2 y1[2][3];   // dx = 1: stays in this thread (the owner's own column)
#pragma unroll
        for (int kp = 0; kp < 2; ++kp)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float2 a1 = ue[3 * (1 | (kp << 2)) + c], b1 = ue[3 * (1 | 2 | (kp << 2)) + c];
                const float2 a0 = ue[3 * (kp << 2) + c], b0 = ue[3 * (2 | (kp << 2)) + c];
                y1[kp][c] = f2add(a1, make_float2(__shfl_down_sync(0xffffffffu, b1.x, 1),
                                                  __shfl_down_sync(0xffffffffu, b1.y, 1)));
                so[(3 * kp + c) * KT_THREADS + tid] =
                    f2add(a0, make_float2(__shfl_down_sync(0xffffffffu, b0.x, 1),
                                          __shfl_down_sync(0xffffffffu, b0.y, 1)));
            }
        __syncthreads();
        if (owner) {
            // x step: dx = 0 comes from the next column (the next warp)
            float2 lo[3], up[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                lo[c] = f2add(y1[0][c], so[c * KT_THREADS + tid + KT_Y]);
                up[c] = f2add(y1[1][c], so[(3 + c) * KT_THREADS + tid + KT_Y]);
            }
            const int64_t node0 = (int64_t)gny + (int64_t)NY * gnx;
            const int on = 3 * ((ty + 1) + (KT_Y + 1) * (tx + 1));
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int z = ez + h;
                float o[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) o[c] = h == 0 ? carry[c] + lo[c].x : lo[c].y + up[c].x;
                if (z >= z0 && z < zend) {
                    const int64_t node = node0 + (int64_t)NY * NX * z;
                    const uint8_t f = nflag[node];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        if (f & (NF_FIXX << c)) o[c] = 0.f;
                        y[3 * node + c] = o[c];
                    }
                    if (DOT) {
                        const float *un = su + xslot(z) * KT_NL * 3 + on;
                        dot += un[0] * o[0] + un[1] * o[1] + un[2] * o[2];
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) carry[c] = up[c].y;
        }
        async_wait_all();
        __syncthreads();
    }
    if (DOT) {
        __shared__ double red[KT_THREADS / 32];
        const double s = block_sum_to_double<float>(dot, red);
        if (tid == 0) partial[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = s;
    }
}

// node layers per CTA of k_kbyu_x2: an odd count (so that the element layers
// z0-1 .. z0+zc-1 form whole pairs).  Default: near 15, balanced over the z
// extent; sgld_assemble's tuner (tune_kbyu_f32) may set another per level.
static int kbyu_x2_zc(int NZ) {
    const int chunks = (NZ + 14) / 15;
    int zc = (NZ + chunks - 1) / chunks;
    if (!(zc & 1)) ++zc;
    return zc;
}

int kbyu_f32_zc(const Level &l) { return l.kx_zc > 0 ? l.kx_zc : kbyu_x2_zc(l.nz + 1); }
// tile width in x: 8 unless the tuner chose 16
int kbyu_f32_tx(const Level &l) { return l.kx_tx == 16 ? 16 : 8; }

static dim3 kbyu_x2_grid(const Level &l) {
    const int NZ = l.nz + 1;
    const int zc = kbyu_f32_zc(l), tx = kbyu_f32_tx(l);
    return dim3((l.ny + 1 + KT_Y - 2) / (KT_Y - 1), (l.nx + 1 + tx - 2) / (tx - 1), (NZ + zc - 1) / zc);
}

static dim3 kbyu_grid(const Level &l) {
    return dim3((l.ny + 1 + KT_Y - 2) / (KT_Y - 1), (l.nx + 1 + KT_X - 2) / (KT_X - 1), (l.nz + 1 + KT_ZC - 1) / KT_ZC);
}

template <typename T>
static constexpr size_t kbyu_smem() {
    return sizeof(T) * (3 * KT_NL * 3 + 24 * KT_THREADS);
}

// opt-in shared memory sizes; called once per context before any launch or
// graph capture
void init_kernel_attributes() {
    cudaFuncSetAttribute(k_kbyu<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kbyu_smem<double>());
    cudaFuncSetAttribute(k_kbyu<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kbyu_smem<double>());
    cudaFuncSetAttribute(k_kbyu_x2<8, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)KxTile<8>::SMEM);
    cudaFuncSetAttribute(k_kbyu_x2<8, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)KxTile<8>::SMEM);
    cudaFuncSetAttribute(k_kbyu_x2<16, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)KxTile<16>::SMEM);
    cudaFuncSetAttribute(k_kbyu_x2<16, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)KxTile<16>::SMEM);
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

void launch_kbyu_f32(const Level &l0, const float *E, const float *u, float *y, double *partial_dot,
                     int *nblocks_out, cudaStream_t s) {
    const dim3 g = kbyu_x2_grid(l0);
    const int zc = kbyu_f32_zc(l0), tx = kbyu_f32_tx(l0);
    if (nblocks_out) *nblocks_out = (int)(g.x * g.y * g.z);
    ++g_launches;
    // the tile map only when it was made for this tile
    const uint8_t *tiles = (l0.tiles_x2 && l0.tiles_x2_tx == tx && l0.tiles_x2_zc == zc) ? l0.tiles_x2 : nullptr;
    if (tx == 8) {
        using G = KxTile<8>;
        if (partial_dot)
            k_kbyu_x2<8, true><<<g, G::THREADS, G::SMEM, s>>>(u, y, E, l0.nflag, l0.ny, l0.nx, l0.nz, zc, partial_dot,
                                                              tiles);
        else
            k_kbyu_x2<8, false><<<g, G::THREADS, G::SMEM, s>>>(u, y, E, l0.nflag, l0.ny, l0.nx, l0.nz, zc, nullptr,
                                                               tiles);
    } else {
        using G = KxTile<16>;
        if (partial_dot)
            k_kbyu_x2<16, true><<<g, G::THREADS, G::SMEM, s>>>(u, y, E, l0.nflag, l0.ny, l0.nx, l0.nz, zc,
                                                               partial_dot, tiles);
        else
            k_kbyu_x2<16, false><<<g, G::THREADS, G::SMEM, s>>>(u, y, E, l0.nflag, l0.ny, l0.nx, l0.nz, zc, nullptr,
                                                                tiles);
    }
}

int update_kbyu_tiles(Level &l0, cudaStream_t s) {
    cudaError_t e = cudaSuccess;
    const dim3 g16 = kbyu_grid(l0);
    if (!l0.tiles16) {
        e = cudaMalloc((void **)&l0.tiles16, (size_t)g16.x * g16.y * g16.z);
        if (e != cudaSuccess) return (int)e;
        make_tile_map(l0, KT_Y, KT_X, KT_ZC, g16, l0.tiles16, s);
    }
    const int tx = kbyu_f32_tx(l0), zc = kbyu_f32_zc(l0);
    if (l0.tiles_x2 && l0.tiles_x2_tx == tx && l0.tiles_x2_zc == zc) return 0;
    const dim3 g = kbyu_x2_grid(l0);
    const int64_t n = (int64_t)g.x * g.y * g.z;
    if (n > l0.tiles_x2_cap) {
        if (l0.tiles_x2) cudaFree(l0.tiles_x2);
        l0.tiles_x2 = nullptr;
        l0.tiles_x2_cap = 0;
        e = cudaMalloc((void **)&l0.tiles_x2, (size_t)n);
        if (e != cudaSuccess) return (int)e;
        l0.tiles_x2_cap = n;
    }
    make_tile_map(l0, KT_Y, tx, zc, g, l0.tiles_x2, s);
    l0.tiles_x2_tx = tx;
    l0.tiles_x2_zc = zc;
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
