// Kernels of the load-case basis (sgld_cases.cu): dot products of a nodal
// vector with every stored basis vector in one pass, linear combinations of
// the basis, and storing a new basis vector.
//
// The basis lives in the compact DOF order (active nodes only, node-major
// [ux uy uz]) in FP64, so a model with 30 % active voxels stores 3.5x less
// than on the full grid; nodal vectors of the solver live on the full grid,
// and DOF n of the compact order is full-grid entry 3 map[n / 3] + n % 3.
// FP64, because a start rounded to FP32 leaves a high-frequency residual near
// 1e-3 of ||F|| that the solve must then remove.  Every pass reads each basis
// vector once (HBM-bound: 8 bytes per DOF per basis vector plus the solver
// vector's 8 bytes per DOF).
#include "sgld_internal.cuh"

namespace sgld {

constexpr int CB_THREADS = 256;
constexpr int CB_MAXK = 32;   // basis vectors per pass

__device__ __forceinline__ int64_t full_index(const int64_t *map, int64_t n) {
    const int64_t node = n / 3;
    return 3 * map[node] + (n - 3 * node);
}

// part[i * gridDim.x + block] = sum over this block's DOFs of W_i[n] v(n)
__global__ void __launch_bounds__(CB_THREADS) k_basis_dots(const double *__restrict__ W, int k, int64_t nd,
                                                           const double *__restrict__ v,
                                                           const int64_t *__restrict__ map,
                                                           double *__restrict__ part) {
    double acc[CB_MAXK];
#pragma unroll
    for (int i = 0; i < CB_MAXK; ++i) acc[i] = 0.0;
    for (int64_t n = blockIdx.x * (int64_t)CB_THREADS + threadIdx.x; n < nd; n += (int64_t)gridDim.x * CB_THREADS) {
        const double vn = v[full_index(map, n)];
#pragma unroll
        for (int i = 0; i < CB_MAXK; ++i)
            if (i < k) acc[i] += W[(int64_t)i * nd + n] * vn;
    }
    __shared__ double red[CB_THREADS / 32][CB_MAXK];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
    for (int i = 0; i < CB_MAXK; ++i) {
        if (i >= k) break;
        double s = acc[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (l == 0) red[w][i] = s;
    }
    __syncthreads();
    if (threadIdx.x < k) {
        double s = 0.0;
        for (int j = 0; j < CB_THREADS / 32; ++j) s += red[j][threadIdx.x];
        part[(int64_t)threadIdx.x * gridDim.x + blockIdx.x] = s;
    }
}

// out[i] = scale * sum_b part[i * nb + b], in a fixed order (one warp per i)
__global__ void k_basis_finalize(const double *__restrict__ part, int nb, int k, double scale,
                                 double *__restrict__ out) {
    const int i = blockIdx.x;
    if (i >= k) return;
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += 32) s += part[(int64_t)i * nb + b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) out[i] = scale * s;
}

// x(n) = beta x(n) + alpha sum_i coef[i] W_i[n] on the full grid
__global__ void __launch_bounds__(CB_THREADS) k_basis_combine(const double *__restrict__ W, int k, int64_t nd,
                                                              const double *__restrict__ coef, double alpha,
                                                              double beta, double *__restrict__ x,
                                                              const int64_t *__restrict__ map) {
    __shared__ double c[CB_MAXK];
    if (threadIdx.x < k) c[threadIdx.x] = coef[threadIdx.x];
    __syncthreads();
    for (int64_t n = blockIdx.x * (int64_t)CB_THREADS + threadIdx.x; n < nd; n += (int64_t)gridDim.x * CB_THREADS) {
        double s = 0.0;
        for (int i = 0; i < k; ++i) s += c[i] * W[(int64_t)i * nd + n];
        const int64_t f = full_index(map, n);
        x[f] = (beta == 0.0 ? 0.0 : beta * x[f]) + alpha * s;
    }
}

// Wk[n] = scale * w(n)
__global__ void k_basis_store(const double *__restrict__ w, const int64_t *__restrict__ map, int64_t nd,
                              double scale, double *__restrict__ Wk) {
    for (int64_t n = blockIdx.x * (int64_t)CB_THREADS + threadIdx.x; n < nd; n += (int64_t)gridDim.x * CB_THREADS)
        Wk[n] = scale * w[full_index(map, n)];
}

static int basis_blocks(int64_t nd) {
    int64_t nb = (nd + CB_THREADS - 1) / CB_THREADS;
    return (int)(nb < 1216 ? (nb < 1 ? 1 : nb) : 1216);   // 152 SMs x 8 CTAs
}

int basis_max() { return CB_MAXK; }
int basis_partials(int64_t nd) { return basis_blocks(nd); }

// out[0..k) = scale * W_i . v  (part: k * basis_partials(nd) doubles)
void launch_basis_dots(const double *W, int k, int64_t nd, const double *v, const int64_t *map, double *part,
                       double scale, double *out, cudaStream_t s) {
    if (k <= 0) return;
    const int nb = basis_blocks(nd);
    g_launches += 2;
    k_basis_dots<<<nb, CB_THREADS, 0, s>>>(W, k, nd, v, map, part);
    k_basis_finalize<<<k, 32, 0, s>>>(part, nb, k, scale, out);
}

void launch_basis_combine(const double *W, int k, int64_t nd, const double *coef, double alpha, double beta,
                          double *x, const int64_t *map, cudaStream_t s) {
    ++g_launches;
    k_basis_combine<<<basis_blocks(nd), CB_THREADS, 0, s>>>(W, k, nd, coef, alpha, beta, x, map);
}

void launch_basis_store(const double *w, const int64_t *map, int64_t nd, double scale, double *Wk, cudaStream_t s) {
    ++g_launches;
    k_basis_store<<<basis_blocks(nd), CB_THREADS, 0, s>>>(w, map, nd, scale, Wk);
}

}  // namespace sgld
