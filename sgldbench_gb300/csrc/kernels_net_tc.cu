// The U-Net's 3x3x3 convolutions (forward, data gradient and weight gradient)
// on the tensor cores; the forward and data gradient are an implicit GEMM per CTA of 128 output voxels x all output channels,
// reduced over 27 taps x input channels with tcgen05.mma (BF16 operands, FP32
// accumulation in tensor memory).  Same operands and epilogues as the
// CUDA-core convolution k_conv (kernels_net.cu): BF16 activations, FP32
// gradients rounded to BF16 when staged as an operand, BF16 weights.
//
// Per tap t a CTA of 4 warps
//   * gathers A = the 128 voxels' neighbours at tap t (cin channels each,
//     zero outside the grid or past cin) into shared memory in the MMA's
//     K-major core-matrix layout, one 16-byte chunk per 8 channels,
//   * copies B = the tap's weight image (cout rows x cin, the same layout,
//     prepared once per call by k_wimage) from global memory,
//   * and one thread issues cin/16 MMAs of 128 x cout x 16 into the TMEM
//     accumulator, then commits them to the buffer's mbarrier.
// A and B are double-buffered: tap t+1 is gathered while tap t's MMAs run;
// before a buffer is refilled the threads wait (bounded) for the commit of
// the tap that last used it.  The epilogue reads the accumulator with
// tcgen05.ld (warp w holds voxel rows 32w .. 32w+31).
#include <cuda_bf16.h>

#include "sgld_net.cuh"
#include "tc_ptx.cuh"

namespace sgld {

namespace {
constexpr int TC_BM = 128;   // output voxels per CTA (the MMA's M)
constexpr int TC_CMAX = 64;  // channels on either side (K and N padded to 16)

__device__ __forceinline__ uint16_t bf16_bits(bf16 v) { return __bfloat16_as_ushort(v); }
__device__ __forceinline__ uint16_t bf16_bits(float v) { return __bfloat16_as_ushort(__float2bfloat16_rn(v)); }

// neighbour of voxel (y, x, z) at tap t (t = (dy+1) + 3(dx+1) + 9(dz+1)), or -1
__device__ __forceinline__ int64_t tc_tap_nb(int y, int x, int z, int t, int taps, int ny, int nx, int nz) {
    if (taps == 1) return (int64_t)y + (int64_t)ny * (x + (int64_t)nx * z);
    const int yy = y + t % 3 - 1, xx = x + (t / 3) % 3 - 1, zz = z + t / 9 - 1;
    if (yy < 0 || yy >= ny || xx < 0 || xx >= nx || zz < 0 || zz >= nz) return -1;
    return (int64_t)yy + (int64_t)ny * (xx + (int64_t)nx * zz);
}
}  // namespace

// img[t] = the B operand of tap t: row n, column k holds W[t][k][n] (K x N
// weights, k < K and n < N), zero elsewhere, in the K-major core-matrix layout
// of an NP x KP operand
__global__ void k_wimage(const bf16 *__restrict__ W, int taps, int K, int N, int KP, int NP, bf16 *__restrict__ img) {
    const int64_t per = (int64_t)NP * KP;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= per * taps) return;
    const int t = (int)(i / per), rem = (int)(i - t * per), n = rem / KP, k = rem - n * KP;
    const bf16 v = (k < K && n < N) ? W[((int64_t)t * K + k) * N + n] : __float2bfloat16_rn(0.f);
    img[t * per + tc::canon_off(n, k, KP) / 2] = v;
}

// MODE 0: BF16 out = relu(. + bias)     MODE 1: FP32 out = . + bias (linear head)
// MODE 2: FP32 out (=/+=) mask(.)      (gradient of a ReLU output when mask != null)
template <typename TIn, int MODE>
__global__ void __launch_bounds__(TC_BM) k_conv_tc(const TIn *__restrict__ in, int cin, const bf16 *__restrict__ wimg,
                                                   int KP, int NP, const float *__restrict__ bias, int cout, int taps,
                                                   int ny, int nx, int nz, void *__restrict__ outp,
                                                   const bf16 *__restrict__ mask, int accumulate,
                                                   int *__restrict__ err) {
    extern __shared__ __align__(128) unsigned char tsm[];
    const int abytes = TC_BM * KP * 2, bbytes = NP * KP * 2;
    unsigned char *Abuf = tsm;                   // [2][abytes]
    unsigned char *Bbuf = tsm + 2 * abytes;      // [2][bbytes]
    uint64_t *bars = reinterpret_cast<uint64_t *>(tsm + 2 * abytes + 2 * bbytes);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 2);
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t ncols = NP <= 32 ? 32u : 64u;
    if (warp == 0) {
        tc::tmem_alloc(tc::saddr(tslot), ncols);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(tc::saddr(bars), 1);
        tc::mbar_init(tc::saddr(bars + 1), 1);
        tc::mbar_init_fence();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t taddr = *tslot;
    const int64_t V = (int64_t)ny * nx * nz;
    const int64_t v = (int64_t)blockIdx.x * TC_BM + tid;   // this thread's voxel = row tid of A
    int y = 0, x = 0, z = 0;
    if (v < V) {
        y = (int)(v % ny);
        x = (int)((v / ny) % nx);
        z = (int)(v / ((int64_t)ny * nx));
    }
    const uint32_t idesc = tc::idesc_bf16(TC_BM, NP);
    const uint32_t lbo = 128, sbo = (uint32_t)(KP / 8) * 128;
    bool ok = true;
    for (int t = 0; t < taps; ++t) {
        const int buf = t & 1;
        // the MMAs of tap t-2 read this buffer: wait for their commit
        if (t >= 2) ok = tc::mbar_wait(tc::saddr(bars + buf), (uint32_t)(((t - 2) >> 1) & 1)) && ok;
        unsigned char *A = Abuf + buf * abytes, *B = Bbuf + buf * bbytes;
        const int64_t nb = v < V ? tc_tap_nb(y, x, z, t, taps, ny, nx, nz) : -1;
        for (int kc = 0; kc < KP / 8; ++kc) {
            uint16_t h[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int k = 8 * kc + j;
                h[j] = (nb >= 0 && k < cin) ? bf16_bits(in[nb * cin + k]) : (uint16_t)0;
            }
            uint4 q;
            q.x = (uint32_t)h[0] | ((uint32_t)h[1] << 16);
            q.y = (uint32_t)h[2] | ((uint32_t)h[3] << 16);
            q.z = (uint32_t)h[4] | ((uint32_t)h[5] << 16);
            q.w = (uint32_t)h[6] | ((uint32_t)h[7] << 16);
            *reinterpret_cast<uint4 *>(A + tc::canon_off(tid, 8 * kc, KP)) = q;
        }
        const uint4 *src = reinterpret_cast<const uint4 *>(wimg + (int64_t)t * NP * KP);
        for (int i = tid; i < bbytes / 16; i += TC_BM) reinterpret_cast<uint4 *>(B)[i] = src[i];
        tc::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc::tc_fence_after();
            const uint32_t a0 = tc::saddr(A), b0 = tc::saddr(B);
            for (int kk = 0; kk < KP / 16; ++kk)
                tc::mma_bf16(taddr, tc::smem_desc(a0 + 256 * kk, lbo, sbo), tc::smem_desc(b0 + 256 * kk, lbo, sbo),
                             idesc, (t > 0 || kk > 0) ? 1u : 0u);
            tc::mma_commit(tc::saddr(bars + buf));
        }
    }
    // the last commit covers every MMA issued before it
    ok = tc::mbar_wait(tc::saddr(bars + ((taps - 1) & 1)), (uint32_t)(((taps - 1) >> 1) & 1)) && ok;
    tc::tc_fence_after();
    if (__syncthreads_or(!ok)) {
        // a wait gave up: wait once more (bounded) so that no MMA is in flight, free TMEM, flag it
        tc::mbar_wait(tc::saddr(bars + ((taps - 1) & 1)), (uint32_t)(((taps - 1) >> 1) & 1));
        tc::tc_fence_before();
        __syncthreads();
        if (warp == 0) tc::tmem_dealloc(taddr, ncols);
        if (tid == 0 && err) atomicExch(err, 1);
        return;
    }
    for (int c0 = 0; c0 < NP; c0 += 16) {
        float r[16];
        tc::tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
        if (v >= V) continue;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int co = c0 + j;
            if (co >= cout) continue;
            const int64_t o = v * cout + co;
            float val = r[j] + ((MODE != 2 && bias) ? bias[co] : 0.f);
            if (MODE == 0) {
                static_cast<bf16 *>(outp)[o] = __float2bfloat16_rn(fmaxf(val, 0.f));
            } else if (MODE == 1) {
                static_cast<float *>(outp)[o] = val;
            } else {
                if (mask && !(__bfloat162float(mask[o]) > 0.f)) val = 0.f;
                float *out = static_cast<float *>(outp);
                out[o] = accumulate ? out[o] + val : val;
            }
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, ncols);
}

// Weight and bias gradients of one convolution on the tensor cores, split over
// voxel ranges like the FP32-pipe k_conv_wgrad:
//   part[s][t][ci][co] = sum_{v in range s} in[nb(v,t)][ci] * g[v][co]
//   bpart[s][co]       = sum_{v in range s} g[v][co]     (centre tap only)
// as D = A B^T with A = 128 channel rows (ci, zero-padded; for the centre tap
// row cin holds ones, so that D's row cin is the bias sum) x 128 voxels, B = cout
// rows x the same voxels, K = the voxels of the CTA's range, 128 per block, all
// accumulated in one TMEM tile.  Operands are BF16 (g rounded as in k_conv_wgrad).
template <typename TIn>
__global__ void __launch_bounds__(TC_BM) k_conv_wgrad_tc(const TIn *__restrict__ in, int cin,
                                                         const float *__restrict__ g, int cout, int NP, int taps,
                                                         int ny, int nx, int nz, int64_t vchunk,
                                                         float *__restrict__ part, float *__restrict__ bpart,
                                                         int *__restrict__ err) {
    extern __shared__ __align__(128) unsigned char tsm[];
    constexpr int KB = TC_BM;                     // voxels per block (the K of 8 MMAs)
    const int abytes = TC_BM * KB * 2, bbytes = NP * KB * 2;
    unsigned char *Abuf = tsm, *Bbuf = tsm + 2 * abytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(tsm + 2 * abytes + 2 * bbytes);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 2);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int t = blockIdx.x, s = blockIdx.y;
    const bool centre = taps == 1 || t == 13;
    const uint32_t ncols = NP <= 32 ? 32u : 64u;
    // padding rows stay zero: clear both buffers once
    for (int i = tid; i < (2 * abytes + 2 * bbytes) / 16; i += TC_BM) reinterpret_cast<uint4 *>(tsm)[i] = make_uint4(0, 0, 0, 0);
    if (warp == 0) {
        tc::tmem_alloc(tc::saddr(tslot), ncols);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(tc::saddr(bars), 1);
        tc::mbar_init(tc::saddr(bars + 1), 1);
        tc::mbar_init_fence();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t taddr = *tslot;
    const int64_t V = (int64_t)ny * nx * nz;
    const int64_t vb = (int64_t)s * vchunk, ve = min(V, vb + vchunk);
    const int nblk = ve > vb ? (int)((ve - vb + KB - 1) / KB) : 0;
    const uint32_t idesc = tc::idesc_bf16(TC_BM, NP);
    const uint32_t lbo = 128, sbo = (KB / 8) * 128;
    const uint16_t one = __bfloat16_as_ushort(__float2bfloat16_rn(1.f));
    // 16-byte loads of 8 activation channels / 4 gradient channels where rows allow them
    const bool vec_in = (cin & 7) == 0 && (reinterpret_cast<uintptr_t>(in) & 15) == 0;
    const bool vec_g = (cout & 3) == 0 && (reinterpret_cast<uintptr_t>(g) & 15) == 0;
    bool ok = true;
    for (int b = 0; b < nblk; ++b) {
        const int buf = b & 1;
        if (b >= 2) ok = tc::mbar_wait(tc::saddr(bars + buf), (uint32_t)(((b - 2) >> 1) & 1)) && ok;
        unsigned char *A = Abuf + buf * abytes, *B = Bbuf + buf * bbytes;
        const int64_t v = vb + (int64_t)b * KB + tid;   // this thread's voxel = column tid
        const bool valid = v < ve;
        int64_t nb = -1;
        if (valid) {
            const int y = (int)(v % ny), x = (int)((v / ny) % nx), z = (int)(v / ((int64_t)ny * nx));
            nb = tc_tap_nb(y, x, z, t, taps, ny, nx, nz);
        }
        // column tid of A (channels of the neighbour) and of B (gradient channels)
        if (vec_in) {
            for (int c8 = 0; c8 < cin; c8 += 8) {
                const uint4 q = nb >= 0 ? *reinterpret_cast<const uint4 *>(in + nb * cin + c8) : make_uint4(0, 0, 0, 0);
                const uint32_t w4[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    *reinterpret_cast<uint16_t *>(A + tc::canon_off(c8 + j, tid, KB)) =
                        (uint16_t)(w4[j >> 1] >> (16 * (j & 1)));
            }
        } else {
            for (int ci = 0; ci < cin; ++ci)
                *reinterpret_cast<uint16_t *>(A + tc::canon_off(ci, tid, KB)) =
                    nb >= 0 ? bf16_bits(in[nb * cin + ci]) : (uint16_t)0;
        }
        if (centre) *reinterpret_cast<uint16_t *>(A + tc::canon_off(cin, tid, KB)) = valid ? one : (uint16_t)0;
        if (vec_g) {
            for (int c4 = 0; c4 < cout; c4 += 4) {
                const float4 q = valid ? *reinterpret_cast<const float4 *>(g + v * cout + c4) : make_float4(0, 0, 0, 0);
                const float f4[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    *reinterpret_cast<uint16_t *>(B + tc::canon_off(c4 + j, tid, KB)) = bf16_bits(f4[j]);
            }
        } else {
            for (int co = 0; co < cout; ++co)
                *reinterpret_cast<uint16_t *>(B + tc::canon_off(co, tid, KB)) =
                    valid ? bf16_bits(g[v * cout + co]) : (uint16_t)0;
        }
        tc::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc::tc_fence_after();
            const uint32_t a0 = tc::saddr(A), b0 = tc::saddr(B);
            for (int kk = 0; kk < KB / 16; ++kk)
                tc::mma_bf16(taddr, tc::smem_desc(a0 + 256 * kk, lbo, sbo), tc::smem_desc(b0 + 256 * kk, lbo, sbo),
                             idesc, (b > 0 || kk > 0) ? 1u : 0u);
            tc::mma_commit(tc::saddr(bars + buf));
        }
    }
    if (nblk > 0) ok = tc::mbar_wait(tc::saddr(bars + ((nblk - 1) & 1)), (uint32_t)(((nblk - 1) >> 1) & 1)) && ok;
    tc::tc_fence_after();
    if (__syncthreads_or(!ok)) {
        if (nblk > 0) tc::mbar_wait(tc::saddr(bars + ((nblk - 1) & 1)), (uint32_t)(((nblk - 1) >> 1) & 1));
        tc::tc_fence_before();
        __syncthreads();
        if (warp == 0) tc::tmem_dealloc(taddr, ncols);
        if (tid == 0 && err) atomicExch(err, 1);
        return;
    }
    const int row = tid;   // TMEM lane = channel row (warp w holds rows 32w .. 32w+31)
    float *outw = part + ((int64_t)s * taps + t) * cin * cout;
    for (int c0 = 0; c0 < NP; c0 += 16) {
        float r[16];
        tc::tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int co = c0 + j;
            if (co >= cout) continue;
            const float val = nblk > 0 ? r[j] : 0.f;
            if (row < cin)
                outw[row * cout + co] = val;
            else if (centre && row == cin)
                bpart[(int64_t)s * cout + co] = val;
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, ncols);
}

static inline int pad16(int c) { return (c + 15) & ~15; }
static inline int nblk_tc(int64_t n, int b) { return (int)((n + b - 1) / b); }
static size_t tc_smem(int KP, int NP) { return 2 * (size_t)TC_BM * KP * 2 + 2 * (size_t)NP * KP * 2 + 32; }

bool net_conv_tc_fits(int cin, int cout) { return cin <= TC_CMAX && cout <= TC_CMAX; }

static size_t tc_wgrad_smem(int NP) { return 2 * (size_t)TC_BM * TC_BM * 2 + 2 * (size_t)NP * TC_BM * 2 + 32; }

bool net_wgrad_tc_fits(int cin, int cout) { return cin < TC_BM && cout <= TC_CMAX; }

void net_conv_wgrad_tc(const bf16 *in, int cin, const float *gout, int cout, int taps, int ny, int nx, int nz, int S,
                       int64_t vchunk, float *part, float *bpart, int *err, cudaStream_t s) {
    const int NP = pad16(cout);
    ++g_launches;
    k_conv_wgrad_tc<bf16><<<dim3(taps, S), TC_BM, tc_wgrad_smem(NP), s>>>(in, cin, gout, cout, NP, taps, ny, nx, nz,
                                                                          vchunk, part, bpart, err);
}

void net_tc_init_attributes() {
    cudaFuncSetAttribute(k_conv_wgrad_tc<bf16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)tc_wgrad_smem(TC_CMAX));
    const int mx = (int)tc_smem(TC_CMAX, TC_CMAX);
    cudaFuncSetAttribute(k_conv_tc<bf16, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_conv_tc<bf16, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_conv_tc<float, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
}

void net_conv_fwd_tc(const bf16 *in, int cin, const bf16 *w, const float *b, int cout, int taps, int ny, int nx,
                     int nz, bool relu_bf16_out, void *out, bf16 *wimg, int *err, cudaStream_t s) {
    const int64_t V = (int64_t)ny * nx * nz;
    const int KP = pad16(cin), NP = pad16(cout);
    g_launches += 2;
    k_wimage<<<nblk_tc((int64_t)taps * NP * KP, 256), 256, 0, s>>>(w, taps, cin, cout, KP, NP, wimg);
    if (relu_bf16_out)
        k_conv_tc<bf16, 0><<<nblk_tc(V, TC_BM), TC_BM, tc_smem(KP, NP), s>>>(in, cin, wimg, KP, NP, b, cout, taps, ny,
                                                                          nx, nz, out, nullptr, 0, err);
    else
        k_conv_tc<bf16, 1><<<nblk_tc(V, TC_BM), TC_BM, tc_smem(KP, NP), s>>>(in, cin, wimg, KP, NP, b, cout, taps, ny,
                                                                          nx, nz, out, nullptr, 0, err);
}

// data gradient: gin (=/+=) mask(conv(gout, wt)) with wt[t'][co][ci] = w[T-1-t'][ci][co]
// (made by the caller), i.e. K = cout input channels and N = cin output channels
void net_conv_bwd_data_tc(const float *gout, int cout, const bf16 *wt, int cin, int taps, int ny, int nx, int nz,
                          const bf16 *mask, float *gin, bool accumulate, bf16 *wimg, int *err, cudaStream_t s) {
    const int64_t V = (int64_t)ny * nx * nz;
    const int KP = pad16(cout), NP = pad16(cin);
    g_launches += 2;
    k_wimage<<<nblk_tc((int64_t)taps * NP * KP, 256), 256, 0, s>>>(wt, taps, cout, cin, KP, NP, wimg);
    k_conv_tc<float, 2><<<nblk_tc(V, TC_BM), TC_BM, tc_smem(KP, NP), s>>>(gout, cout, wimg, KP, NP, nullptr, cin,
                                                                        taps, ny, nx, nz, gin, mask,
                                                                        accumulate ? 1 : 0, err);
}

}  // namespace sgld
