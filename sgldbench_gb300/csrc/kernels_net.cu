// Kernels of the learned warm start: a small 3D convolutional U-Net that runs
// on the node grid of one multigrid level and is trained on the GPU by the
// solver itself (no counterpart in the reference, whose solves always start
// from the previous displacement, src/Solving_CG_GMGS.m:7).
//
// Tensors are channels-last on a structured node grid: element [v][c] with
// v = y + NY*(x + NX*z), the layout of the solver's own nodal vectors, so a
// 3-component level vector is already a 3-channel tensor.
//   * activations: BF16 (stored after the epilogue, round to nearest even);
//   * gradients of activations: FP32, rounded to BF16 when they are staged as
//     an operand of a convolution;
//   * weights: FP32 master copy, BF16 shadow used by every convolution;
//   * every product accumulates in FP32.
// A 3x3x3 convolution ("same", zero padding) is an implicit GEMM: output
// voxels x output channels, reduced over 27 taps x input channels.  The work
// is small (about 4 GFLOP forward at 65x33x33 nodes).  The forward and data-
// gradient convolutions run on the tensor cores (kernels_net_tc.cu); k_conv
// below is their FP32-pipe form (SGLD_NET_CUDA_CORES=1, and channel counts
// above 64), and the weight gradient stays on the FP32 pipes.
#include <cuda_bf16.h>

#include "sgld_internal.cuh"
#include "sgld_net.cuh"

namespace sgld {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ float ld_op(const bf16 *p, int64_t i) { return __bfloat162float(p[i]); }
// an FP32 gradient staged as an operand takes BF16 precision
__device__ __forceinline__ float ld_op(const float *p, int64_t i) {
    return __bfloat162float(__float2bfloat16_rn(p[i]));
}

// neighbour of voxel v at tap t of a 3x3x3 stencil (t = (dy+1) + 3(dx+1) + 9(dz+1)),
// or -1 outside the grid; a 1-tap convolution is the centre only
__device__ __forceinline__ int64_t tap_nb(int y, int x, int z, int t, int taps, int ny, int nx, int nz) {
    if (taps == 1) return (int64_t)y + (int64_t)ny * (x + (int64_t)nx * z);
    const int dy = t % 3 - 1, dx = (t / 3) % 3 - 1, dz = t / 9 - 1;
    const int yy = y + dy, xx = x + dx, zz = z + dz;
    if (yy < 0 || yy >= ny || xx < 0 || xx >= nx || zz < 0 || zz >= nz) return -1;
    return (int64_t)yy + (int64_t)ny * (xx + (int64_t)nx * zz);
}

constexpr int CV_BM = 128;          // output voxels per CTA
constexpr int CV_AS = CV_BM + 4;    // row stride of the staged input tile (16-byte rows)
constexpr int CV_CMAX = 64;         // channels per side

// out[v][co] = epilogue(sum_t sum_ci in[nb(v,t)][ci] * w[t][ci][co] + bias[co])
// MODE 0: BF16 out = relu(.)            MODE 1: FP32 out = (.)  (linear head)
// MODE 2: FP32 out (=/+=) mask(.)      (gradient of a ReLU output when mask != null)
// blockDim = 32 * cp/4 with cp = cout rounded up to 4; thread (vg, cg) owns
// voxels v0 + 4vg .. +3 and channels 4cg .. 4cg+3.
template <typename TIn, int MODE>
__global__ void __launch_bounds__(512) k_conv(const TIn *__restrict__ in, int cin, const bf16 *__restrict__ w,
                                              const float *__restrict__ bias, int cout, int taps, int ny, int nx,
                                              int nz, void *__restrict__ outp, const bf16 *__restrict__ mask,
                                              int accumulate) {
    extern __shared__ __align__(16) float cv_smem[];
    const int cp = (cout + 3) & ~3;
    float *As = cv_smem;              // [cin][CV_AS]
    float *Ws = cv_smem + cin * CV_AS;  // [cin][cp]
    const int tid = threadIdx.x, vg = tid & 31, cg = tid >> 5;
    const int64_t V = (int64_t)ny * nx * nz;
    const int64_t v0 = (int64_t)blockIdx.x * CV_BM;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int t = 0; t < taps; ++t) {
        for (int idx = tid; idx < CV_BM * cin; idx += blockDim.x) {
            const int vl = idx / cin, ci = idx - vl * cin;
            const int64_t v = v0 + vl;
            float a = 0.f;
            if (v < V) {
                const int y = (int)(v % ny), x = (int)((v / ny) % nx), z = (int)(v / ((int64_t)ny * nx));
                const int64_t nb = tap_nb(y, x, z, t, taps, ny, nx, nz);
                if (nb >= 0) a = ld_op(in, nb * cin + ci);
            }
            As[ci * CV_AS + vl] = a;
        }
        for (int idx = tid; idx < cin * cp; idx += blockDim.x) {
            const int ci = idx / cp, co = idx - ci * cp;
            Ws[idx] = co < cout ? __bfloat162float(w[((int64_t)t * cin + ci) * cout + co]) : 0.f;
        }
        __syncthreads();
        for (int ci = 0; ci < cin; ++ci) {
            const float4 a = *reinterpret_cast<const float4 *>(&As[ci * CV_AS + 4 * vg]);
            const float4 b = *reinterpret_cast<const float4 *>(&Ws[ci * cp + 4 * cg]);
            const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t v = v0 + 4 * vg + i;
        if (v >= V) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int co = 4 * cg + j;
            if (co >= cout) continue;
            const int64_t o = v * cout + co;
            float r = acc[i][j] + (bias ? bias[co] : 0.f);
            if (MODE == 0) {
                static_cast<bf16 *>(outp)[o] = __float2bfloat16_rn(fmaxf(r, 0.f));
            } else if (MODE == 1) {
                static_cast<float *>(outp)[o] = r;
            } else {
                if (mask && !(__bfloat162float(mask[o]) > 0.f)) r = 0.f;
                float *out = static_cast<float *>(outp);
                out[o] = accumulate ? out[o] + r : r;
            }
        }
    }
}

// Weight and bias gradients of one convolution, split over voxel ranges:
//   part[s][t][ci][co] = sum_{v in range s} in[nb(v,t)][ci] * g[v][co]
//   bpart[s][co]       = sum_{v in range s} g[v][co]          (t = centre only)
// grid (taps, S).  Thread p < (cin/4)(cp/4) owns a 4x4 block (ci, co); the
// remaining factor of the block size splits the voxels of each staged chunk.
constexpr int WG_BV = 64;

template <typename TIn>
__global__ void __launch_bounds__(256, 1) k_conv_wgrad(const TIn *__restrict__ in, int cin,
                                                    const float *__restrict__ g, int cout, int taps, int ny, int nx,
                                                    int nz, int64_t vchunk, float *__restrict__ part,
                                                    float *__restrict__ bpart) {
    __shared__ __align__(16) float Xs[WG_BV * (CV_CMAX + 4)];
    __shared__ __align__(16) float Gs[WG_BV * (CV_CMAX + 4)];
    __shared__ float red[256 * 4];
    const int cp = (cout + 3) & ~3, ci4n = cin / 4, co4n = cp / 4;
    const int npair = ci4n * co4n;
    const int vsplit = max(1, (int)blockDim.x / npair);
    const int tid = threadIdx.x;
    const int pr = tid % npair, vs = tid / npair;
    const bool active = tid < npair * vsplit;
    const int ci4 = pr / co4n, co4 = pr % co4n;
    const int t = blockIdx.x, s = blockIdx.y;
    const int xs = cin + 4, gs = cp + 4;
    const int64_t V = (int64_t)ny * nx * nz;
    const int64_t vb = (int64_t)s * vchunk, ve = min(V, vb + vchunk);
    const bool centre = (taps == 1) || t == 13;
    float acc[4][4], bacc[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        bacc[i] = 0.f;
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    }
    for (int64_t c0 = vb; c0 < ve; c0 += WG_BV) {
        for (int idx = tid; idx < WG_BV * cin; idx += blockDim.x) {
            const int vl = idx / cin, ci = idx - vl * cin;
            const int64_t v = c0 + vl;
            float a = 0.f;
            if (v < ve) {
                const int y = (int)(v % ny), x = (int)((v / ny) % nx), z = (int)(v / ((int64_t)ny * nx));
                const int64_t nb = tap_nb(y, x, z, t, taps, ny, nx, nz);
                if (nb >= 0) a = ld_op(in, nb * cin + ci);
            }
            Xs[vl * xs + ci] = a;
        }
        for (int idx = tid; idx < WG_BV * cp; idx += blockDim.x) {
            const int vl = idx / cp, co = idx - vl * cp;
            const int64_t v = c0 + vl;
            Gs[vl * gs + co] = (v < ve && co < cout) ? ld_op(g, v * cout + co) : 0.f;
        }
        __syncthreads();
        if (active) {
            for (int vl = vs; vl < WG_BV; vl += vsplit) {
                const float4 a = *reinterpret_cast<const float4 *>(&Xs[vl * xs + 4 * ci4]);
                const float4 b = *reinterpret_cast<const float4 *>(&Gs[vl * gs + 4 * co4]);
                const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
                if (centre && ci4 == 0)
#pragma unroll
                    for (int j = 0; j < 4; ++j) bacc[j] += bv[j];
            }
        }
        __syncthreads();
    }
    // sum the vsplit groups of each (ci, co) block: 16 + 4 values per thread
    float *outw = part + ((int64_t)s * taps + t) * cin * cout;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        __syncthreads();
        if (active)
#pragma unroll
            for (int j = 0; j < 4; ++j) red[tid * 4 + j] = q < 4 ? acc[q][j] : bacc[j];
        __syncthreads();
        if (active && vs == 0) {
            float sum[4] = {0.f, 0.f, 0.f, 0.f};
            for (int k = 0; k < vsplit; ++k)
#pragma unroll
                for (int j = 0; j < 4; ++j) sum[j] += red[(pr + k * npair) * 4 + j];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int co = 4 * co4 + j;
                if (co >= cout) continue;
                if (q < 4)
                    outw[(4 * ci4 + q) * cout + co] = sum[j];
                else if (centre && ci4 == 0)
                    bpart[(int64_t)s * cout + co] = sum[j];
            }
        }
    }
}

// out[i] = sum_s part[s][i] (fixed order)
__global__ void k_sum_parts(const float *__restrict__ part, int64_t n, int S, float *__restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float a = 0.f;
    for (int s = 0; s < S; ++s) a += part[(int64_t)s * n + i];
    out[i] = a;
}

// weights of the data gradient: wt[t'][co][ci] = w[T-1-t'][ci][co]
__global__ void k_wflip(const bf16 *__restrict__ w, int taps, int cin, int cout, bf16 *__restrict__ wt) {
    const int64_t n = (int64_t)taps * cin * cout;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int ci = (int)(i % cin), co = (int)((i / cin) % cout), t = (int)(i / ((int64_t)cin * cout));
    wt[i] = w[((int64_t)(taps - 1 - t) * cin + ci) * cout + co];
}

// child (fine) -> parent (coarse) on grids with coarse = ceil(fine / 2)
__device__ __forceinline__ int64_t parent_of(int64_t vf, int fy, int fx, int cy, int cx) {
    const int y = (int)(vf % fy), x = (int)((vf / fy) % fx), z = (int)(vf / ((int64_t)fy * fx));
    return (int64_t)(y >> 1) + (int64_t)cy * ((x >> 1) + (int64_t)cx * (z >> 1));
}
__device__ __forceinline__ int child_count(int64_t vc, int cy, int cx, int fy, int fx, int fz) {
    const int y = (int)(vc % cy), x = (int)((vc / cy) % cx), z = (int)(vc / ((int64_t)cy * cx));
    return (min(2, fy - 2 * y)) * (min(2, fx - 2 * x)) * (min(2, fz - 2 * z));
}

// average pooling over the existing children
__global__ void k_pool(const bf16 *__restrict__ f, int C, int fy, int fx, int fz, int cy, int cx, int cz,
                       bf16 *__restrict__ c) {
    const int64_t n = (int64_t)cy * cx * cz * C;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int ch = (int)(i % C);
    const int64_t vc = i / C;
    const int y = (int)(vc % cy), x = (int)((vc / cy) % cx), z = (int)(vc / ((int64_t)cy * cx));
    float s = 0.f;
    int k = 0;
    for (int dz = 0; dz < 2; ++dz)
        for (int dx = 0; dx < 2; ++dx)
            for (int dy = 0; dy < 2; ++dy) {
                const int yy = 2 * y + dy, xx = 2 * x + dx, zz = 2 * z + dz;
                if (yy >= fy || xx >= fx || zz >= fz) continue;
                s += __bfloat162float(f[((int64_t)yy + (int64_t)fy * (xx + (int64_t)fx * zz)) * C + ch]);
                ++k;
            }
    c[i] = __float2bfloat16_rn(s / (float)k);
}

// gf (=/+=) mask_f(gc[parent] / count(parent))
__global__ void k_pool_bwd(const float *__restrict__ gc, int C, int fy, int fx, int fz, int cy, int cx,
                           const bf16 *__restrict__ maskf, float *__restrict__ gf, int accumulate) {
    const int64_t n = (int64_t)fy * fx * fz * C;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int ch = (int)(i % C);
    const int64_t vf = i / C;
    const int64_t vc = parent_of(vf, fy, fx, cy, cx);
    float r = gc[vc * C + ch] / (float)child_count(vc, cy, cx, fy, fx, fz);
    if (maskf && !(__bfloat162float(maskf[i]) > 0.f)) r = 0.f;
    gf[i] = accumulate ? gf[i] + r : r;
}

// out = up(c) + skip  (nearest-neighbour upsampling)
__global__ void k_up_add(const bf16 *__restrict__ c, const bf16 *__restrict__ skip, int C, int fy, int fx, int fz,
                         int cy, int cx, bf16 *__restrict__ out) {
    const int64_t n = (int64_t)fy * fx * fz * C;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int ch = (int)(i % C);
    const int64_t vc = parent_of(i / C, fy, fx, cy, cx);
    out[i] = __float2bfloat16_rn(__bfloat162float(c[vc * C + ch]) + __bfloat162float(skip[i]));
}

// backward of k_up_add: gc = mask_c(sum over children of gs), gskip (=/+=) mask_skip(gs)
__global__ void k_up_add_bwd(const float *__restrict__ gs, int C, int fy, int fx, int fz, int cy, int cx, int cz,
                             const bf16 *__restrict__ maskc, float *__restrict__ gc,
                             const bf16 *__restrict__ maskskip, float *__restrict__ gskip, int acc_skip) {
    const int64_t nf = (int64_t)fy * fx * fz * C, nc = (int64_t)cy * cx * cz * C;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < nf) {
        float r = gs[i];
        if (maskskip && !(__bfloat162float(maskskip[i]) > 0.f)) r = 0.f;
        gskip[i] = acc_skip ? gskip[i] + r : r;
    }
    if (i < nc) {
        const int ch = (int)(i % C);
        const int64_t vc = i / C;
        const int y = (int)(vc % cy), x = (int)((vc / cy) % cx), z = (int)(vc / ((int64_t)cy * cx));
        float s = 0.f;
        for (int dz = 0; dz < 2; ++dz)
            for (int dx = 0; dx < 2; ++dx)
                for (int dy = 0; dy < 2; ++dy) {
                    const int yy = 2 * y + dy, xx = 2 * x + dx, zz = 2 * z + dz;
                    if (yy >= fy || xx >= fx || zz >= fz) continue;
                    s += gs[((int64_t)yy + (int64_t)fy * (xx + (int64_t)fx * zz)) * C + ch];
                }
        if (maskc && !(__bfloat162float(maskc[i]) > 0.f)) s = 0.f;
        gc[i] = s;
    }
}

// masked mean-square loss over C channels: partial sums of m (y - t)^2 and of m,
// and gy = m (y - t) (scaled on the host side of the next kernel by 2 / (C sum m))
__global__ void k_mse(const float *__restrict__ y, const float *__restrict__ t, const float *__restrict__ m,
                      int C, int64_t V, float *__restrict__ gy, double *__restrict__ part) {
    double se = 0.0, sm = 0.0;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
        const float mv = m[v];
        sm += mv;
        for (int c = 0; c < C; ++c) {
            const float d = y[v * C + c] - t[v * C + c];
            se += (double)(mv * d * d);
            gy[v * C + c] = mv * d;
        }
    }
    __shared__ double r1[256], r2[256];
    r1[threadIdx.x] = se;
    r2[threadIdx.x] = sm;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            r1[threadIdx.x] += r1[threadIdx.x + s];
            r2[threadIdx.x] += r2[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = r1[0];
        part[2 * blockIdx.x + 1] = r2[0];
    }
}

// loss = sum se / (C sum m); gy *= 2 / (C sum m)
__global__ void k_mse_finish(const double *__restrict__ part, int nb, int C, int64_t n, float *__restrict__ gy,
                             double *__restrict__ loss) {
    __shared__ double sc;
    if (threadIdx.x == 0) {
        double se = 0.0, sm = 0.0;
        for (int b = 0; b < nb; ++b) {
            se += part[2 * b];
            sm += part[2 * b + 1];
        }
        const double den = (double)C * (sm > 0.0 ? sm : 1.0);
        sc = 2.0 / den;
        if (blockIdx.x == 0) *loss = se / den;
    }
    __syncthreads();
    const float f = (float)sc;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        gy[i] *= f;
}

// Adam (Kingma & Ba 2015) on the FP32 master weights; c1 = 1/(1-b1^k),
// c2 = 1/(1-b2^k); refreshes the BF16 shadow
__global__ void k_adam(float *__restrict__ w, float *__restrict__ m, float *__restrict__ v,
                       const float *__restrict__ g, bf16 *__restrict__ wb, int64_t n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    w[i] = wi;
    wb[i] = __float2bfloat16_rn(wi);
}

__global__ void k_to_bf16(const float *__restrict__ a, bf16 *__restrict__ b, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = __float2bfloat16_rn(a[i]);
}

// ---- launchers -------------------------------------------------------------
static inline int nblk(int64_t n, int b = 256) { return (int)((n + b - 1) / b); }

static size_t conv_smem(int cin, int cout) { return sizeof(float) * (size_t)cin * (CV_AS + ((cout + 3) & ~3)); }

// opt-in shared memory of the convolution (64 x 64 channels need 49 KB)
void net_init_attributes() {
    net_tc_init_attributes();
    const int mx = (int)conv_smem(CV_CMAX, CV_CMAX);
    cudaFuncSetAttribute(k_conv<bf16, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_conv<bf16, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_conv<float, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
}

// the CUDA-core convolutions instead of the tensor-core ones (environment
// SGLD_NET_CUDA_CORES=1, read once; for comparisons)
static bool net_cuda_cores() {
    static const bool v = [] {
        const char *e = getenv("SGLD_NET_CUDA_CORES");
        return e && e[0] == '1';
    }();
    return v;
}

void net_conv_fwd(const bf16 *in, int cin, const bf16 *w, const float *b, int cout, int taps, int ny, int nx, int nz,
                  bool relu_bf16_out, void *out, bf16 *wimg, int *err, cudaStream_t s) {
    if (wimg && net_conv_tc_fits(cin, cout) && !net_cuda_cores()) {
        net_conv_fwd_tc(in, cin, w, b, cout, taps, ny, nx, nz, relu_bf16_out, out, wimg, err, s);
        return;
    }
    const int64_t V = (int64_t)ny * nx * nz;
    const int threads = 32 * (((cout + 3) & ~3) / 4);
    ++g_launches;
    if (relu_bf16_out)
        k_conv<bf16, 0><<<nblk(V, CV_BM), threads, conv_smem(cin, cout), s>>>(in, cin, w, b, cout, taps, ny, nx, nz,
                                                                             out, nullptr, 0);
    else
        k_conv<bf16, 1><<<nblk(V, CV_BM), threads, conv_smem(cin, cout), s>>>(in, cin, w, b, cout, taps, ny, nx, nz,
                                                                             out, nullptr, 0);
}

// data gradient: gin (=/+=) mask(conv(gout, flipped w)); wt is scratch of taps*cin*cout
void net_conv_bwd_data(const float *gout, int cout, const bf16 *w, bf16 *wt, int cin, int taps, int ny, int nx,
                       int nz, const bf16 *mask, float *gin, bool accumulate, bf16 *wimg, int *err, cudaStream_t s) {
    const int64_t V = (int64_t)ny * nx * nz;
    const int64_t nw = (int64_t)taps * cin * cout;
    ++g_launches;
    k_wflip<<<nblk(nw), 256, 0, s>>>(w, taps, cin, cout, wt);
    if (wimg && net_conv_tc_fits(cout, cin) && !net_cuda_cores()) {
        net_conv_bwd_data_tc(gout, cout, wt, cin, taps, ny, nx, nz, mask, gin, accumulate, wimg, err, s);
        return;
    }
    ++g_launches;
    const int threads = 32 * (((cin + 3) & ~3) / 4);
    k_conv<float, 2><<<nblk(V, CV_BM), threads, conv_smem(cout, cin), s>>>(gout, cout, wt, nullptr, cin, taps, ny, nx,
                                                                           nz, gin, mask, accumulate ? 1 : 0);
}

int net_wgrad_splits(int64_t V) {
    const int64_t s = V / 2048;
    return (int)(s < 1 ? 1 : (s > 64 ? 64 : s));
}

// gw = dL/dw [taps][cin][cout], gb = dL/db [cout]; part holds S*(taps*cin*cout + cout) floats
void net_conv_wgrad(const bf16 *in, int cin, const float *gout, int cout, int taps, int ny, int nx, int nz,
                    float *part, float *gw, float *gb, int *err, cudaStream_t s) {
    const int64_t V = (int64_t)ny * nx * nz;
    const int S = net_wgrad_splits(V);
    const int64_t vchunk = (V + S - 1) / S;
    const int64_t nw = (int64_t)taps * cin * cout;
    float *bpart = part + (int64_t)S * nw;
    g_launches += 2;
    if (err && net_wgrad_tc_fits(cin, cout) && !net_cuda_cores()) {
        net_conv_wgrad_tc(in, cin, gout, cout, taps, ny, nx, nz, S, vchunk, part, bpart, err, s);
    } else {
        ++g_launches;
        k_conv_wgrad<bf16><<<dim3(taps, S), 256, 0, s>>>(in, cin, gout, cout, taps, ny, nx, nz, vchunk, part, bpart);
    }
    k_sum_parts<<<nblk(nw), 256, 0, s>>>(part, nw, S, gw);
    k_sum_parts<<<nblk(cout), 256, 0, s>>>(bpart, cout, S, gb);
}

void net_pool(const bf16 *f, int C, const int fd[3], const int cd[3], bf16 *c, cudaStream_t s) {
    const int64_t n = (int64_t)cd[0] * cd[1] * cd[2] * C;
    ++g_launches;
    k_pool<<<nblk(n), 256, 0, s>>>(f, C, fd[0], fd[1], fd[2], cd[0], cd[1], cd[2], c);
}

void net_pool_bwd(const float *gc, int C, const int fd[3], const int cd[3], const bf16 *maskf, float *gf,
                  bool accumulate, cudaStream_t s) {
    const int64_t n = (int64_t)fd[0] * fd[1] * fd[2] * C;
    ++g_launches;
    k_pool_bwd<<<nblk(n), 256, 0, s>>>(gc, C, fd[0], fd[1], fd[2], cd[0], cd[1], maskf, gf, accumulate ? 1 : 0);
}

void net_up_add(const bf16 *c, const bf16 *skip, int C, const int fd[3], const int cd[3], bf16 *out,
                cudaStream_t s) {
    const int64_t n = (int64_t)fd[0] * fd[1] * fd[2] * C;
    ++g_launches;
    k_up_add<<<nblk(n), 256, 0, s>>>(c, skip, C, fd[0], fd[1], fd[2], cd[0], cd[1], out);
}

void net_up_add_bwd(const float *gs, int C, const int fd[3], const int cd[3], const bf16 *maskc, float *gc,
                    const bf16 *maskskip, float *gskip, bool acc_skip, cudaStream_t s) {
    const int64_t n = (int64_t)fd[0] * fd[1] * fd[2] * C;
    ++g_launches;
    k_up_add_bwd<<<nblk(n), 256, 0, s>>>(gs, C, fd[0], fd[1], fd[2], cd[0], cd[1], cd[2], maskc, gc, maskskip, gskip,
                                         acc_skip ? 1 : 0);
}

int net_mse_blocks(int64_t V) {
    const int64_t b = (V + 255) / 256;
    return (int)(b < 304 ? (b > 0 ? b : 1) : 304);
}

void net_mse(const float *y, const float *t, const float *m, int C, int64_t V, float *gy, double *part,
             double *loss, cudaStream_t s) {
    const int nb = net_mse_blocks(V);
    g_launches += 2;
    k_mse<<<nb, 256, 0, s>>>(y, t, m, C, V, gy, part);
    k_mse_finish<<<nb, 256, 0, s>>>(part, nb, C, V * C, gy, loss);
}

void net_adam(float *w, float *m, float *v, const float *g, bf16 *wb, int64_t n, float lr, float b1, float b2,
              float eps, float c1, float c2, cudaStream_t s) {
    ++g_launches;
    k_adam<<<nblk(n), 256, 0, s>>>(w, m, v, g, wb, n, lr, b1, b2, eps, c1, c2);
}

void net_to_bf16(const float *a, bf16 *b, int64_t n, cudaStream_t s) {
    ++g_launches;
    k_to_bf16<<<nblk(n), 256, 0, s>>>(a, b, n);
}

}  // namespace sgld

// ---- the warm start's bridge between the solver's level vectors and the network ----
namespace sgld {

// coarse node (y, x, z) of a level with cumulative span S sits on fine node (Sy, Sx, Sz)
__global__ void k_net_inject(const double *__restrict__ fine, int NYf, int NXf, int S, int NYc, int NXc, int NZc,
                             double *__restrict__ out) {
    const int64_t Vc = (int64_t)NYc * NXc * NZc;
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= Vc) return;
    const int y = (int)(v % NYc), x = (int)((v / NYc) % NXc), z = (int)(v / ((int64_t)NYc * NXc));
    const int64_t f = (int64_t)S * y + (int64_t)NYf * ((int64_t)S * x + (int64_t)NXf * ((int64_t)S * z));
#pragma unroll
    for (int c = 0; c < 3; ++c) out[3 * v + c] = fine[3 * f + c];
}

// log-modulus field on the network's nodes: mean over the fine elements within
// half a coarse cell (at least one element) of g(E) = clamp(1 + log10(E/E0)/9, 0, 1), 0 for void
__global__ void k_net_logE(const double *__restrict__ E, int ny, int nx, int nz, int S, int NYc, int NXc, int NZc,
                           double E0, float *__restrict__ fe) {
    const int64_t Vc = (int64_t)NYc * NXc * NZc;
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= Vc) return;
    const int y = (int)(v % NYc), x = (int)((v / NYc) % NXc), z = (int)(v / ((int64_t)NYc * NXc));
    const int h = S / 2 > 1 ? S / 2 : 1;
    float s = 0.f;
    int n = 0;
    for (int ez = S * z - h; ez < S * z + h; ++ez)
        for (int ex = S * x - h; ex < S * x + h; ++ex)
            for (int ey = S * y - h; ey < S * y + h; ++ey) {
                ++n;
                if (ey < 0 || ey >= ny || ex < 0 || ex >= nx || ez < 0 || ez >= nz) continue;
                const double e = E[(int64_t)ey + (int64_t)ny * (ex + (int64_t)nx * ez)];
                if (e > 0.0) s += fminf(fmaxf(1.f + (float)log10(e / E0) / 9.f, 0.f), 1.f);
            }
    fe[v] = s / (float)n;
}

// network input [v][8]: restricted residual (3) * sr, previous change (3) * sd,
// log-modulus field, active-node indicator
__global__ void k_net_pack(const double *__restrict__ rc, const double *__restrict__ dc,
                           const float *__restrict__ fe, const uint8_t *__restrict__ nflag, int64_t Vc, double sr,
                           double sd, bf16 *__restrict__ X) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= Vc) return;
    const bool act = nflag[v] & NF_ACTIVE;
    bf16 *o = X + 8 * v;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        o[c] = __float2bfloat16_rn(act ? (float)(rc[3 * v + c] * sr) : 0.f);
        o[3 + c] = __float2bfloat16_rn(act ? (float)(dc[3 * v + c] * sd) : 0.f);
    }
    o[6] = __float2bfloat16_rn(act ? fe[v] : 0.f);
    o[7] = __float2bfloat16_rn(act ? 1.f : 0.f);
}

// training target: the change of the displacement, injected and scaled; mask = active nodes
__global__ void k_net_target(const double *__restrict__ ec, const uint8_t *__restrict__ nflag, int64_t Vc,
                             double se, float *__restrict__ T, float *__restrict__ M) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= Vc) return;
    const bool act = nflag[v] & NF_ACTIVE;
#pragma unroll
    for (int c = 0; c < 3; ++c) T[3 * v + c] = act ? (float)(ec[3 * v + c] * se) : 0.f;
    M[v] = act ? 1.f : 0.f;
}

// network output [v][3] -> level vector, zero on inactive nodes
__global__ void k_net_unpack(const float *__restrict__ Y, const uint8_t *__restrict__ nflag, int64_t Vc,
                             double *__restrict__ out) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= Vc) return;
    const bool act = nflag[v] & NF_ACTIVE;
#pragma unroll
    for (int c = 0; c < 3; ++c) out[3 * v + c] = act ? (double)Y[3 * v + c] : 0.0;
}

// y = a x + b y
__global__ void k_net_axpby(double *__restrict__ y, const double *__restrict__ x, double a, double b, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = a * x[i] + b * y[i];
}

void net_inject(const double *fine, const int fnodes[3], int S, const int cnodes[3], double *out, cudaStream_t s) {
    const int64_t Vc = (int64_t)cnodes[0] * cnodes[1] * cnodes[2];
    ++g_launches;
    k_net_inject<<<nblk(Vc), 256, 0, s>>>(fine, fnodes[0], fnodes[1], S, cnodes[0], cnodes[1], cnodes[2], out);
}

void net_logE(const double *E, const int felems[3], int S, const int cnodes[3], double E0, float *fe,
              cudaStream_t s) {
    const int64_t Vc = (int64_t)cnodes[0] * cnodes[1] * cnodes[2];
    ++g_launches;
    k_net_logE<<<nblk(Vc), 256, 0, s>>>(E, felems[0], felems[1], felems[2], S, cnodes[0], cnodes[1], cnodes[2], E0,
                                        fe);
}

void net_pack(const double *rc, const double *dc, const float *fe, const uint8_t *nflag, int64_t Vc, double sr,
              double sd, bf16 *X, cudaStream_t s) {
    ++g_launches;
    k_net_pack<<<nblk(Vc), 256, 0, s>>>(rc, dc, fe, nflag, Vc, sr, sd, X);
}

void net_target(const double *ec, const uint8_t *nflag, int64_t Vc, double se, float *T, float *M, cudaStream_t s) {
    ++g_launches;
    k_net_target<<<nblk(Vc), 256, 0, s>>>(ec, nflag, Vc, se, T, M);
}

void net_unpack(const float *Y, const uint8_t *nflag, int64_t Vc, double *out, cudaStream_t s) {
    ++g_launches;
    k_net_unpack<<<nblk(Vc), 256, 0, s>>>(Y, nflag, Vc, out);
}

void net_axpby(double *y, const double *x, double a, double b, int64_t n, cudaStream_t s) {
    ++g_launches;
    const int64_t nb = (n + 255) / 256;
    k_net_axpby<<<(int)(nb < 152 * 8 ? (nb > 0 ? nb : 1) : 152 * 8), 256, 0, s>>>(y, x, a, b, n);
}

}  // namespace sgld
