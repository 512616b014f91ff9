// BLAS-1 style kernels of the preconditioned CG loop
// (reference: src/Solving_PreconditionedConjugateGradientSolver.m:7-36).
// Scalars live on the device; reductions are two-stage (per-CTA partials,
// then one CTA sums them in a fixed order), so results are deterministic.
// Once the convergence flag is set, the kernels that would change x, r or
// the iteration count return immediately.
#include "sgld_internal.cuh"

namespace sgld {

constexpr int VB = 256;
constexpr int VGRID = 152 * 8;   // persistent grid: 8 CTAs per SM

int reduce_blocks(int64_t n) {
    const int64_t b = (n + VB - 1) / VB;
    return (int)(b < VGRID ? (b > 0 ? b : 1) : VGRID);
}

__device__ __forceinline__ double block_reduce(double v) {
    __shared__ double red[VB / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < VB / 32; ++i) s += red[i];
    return s;
}

__global__ void k_dot(const double *__restrict__ a, const double *__restrict__ b, int64_t n, double *__restrict__ part) {
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)VB + threadIdx.x; i < n; i += (int64_t)gridDim.x * VB) s += a[i] * b[i];
    s = block_reduce(s);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

void launch_dot(const double *a, const double *b, int64_t n, double *partial, int nb, cudaStream_t s) {
    ++g_launches;
    k_dot<<<nb, VB, 0, s>>>(a, b, n, partial);
}

// fixed-order sum of nb partials (single CTA)
__device__ double sum_partials(const double *__restrict__ part, int nb) {
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += VB) s += part[i];
    return block_reduce(s);
}

__global__ void k_finalize_sum(const double *__restrict__ part, int nb, double *__restrict__ out) {
    const double s = sum_partials(part, nb);
    if (threadIdx.x == 0) out[0] = s;
}
void launch_finalize_sum(const double *partial, int nb, double *out, cudaStream_t s) {
    ++g_launches;
    k_finalize_sum<<<1, VB, 0, s>>>(partial, nb, out);
}

// scalar slots
enum { S_NORMB = 0, S_X1 = 1, S_LAM = 2, S_RES = 3, S_BETA = 4, S_PQ = 5, S_RR = 6, S_TOL = 15 };
enum { I_ITS = 0, I_DONE = 1, I_STOP = 2 };

// op: 0 normB = sqrt(sum); 1 x1 = sum; 2 lambda = x1 / sum;
//     3 residual test; 4 beta = sum / x1, x1 = sum; 5 reset iteration state
__global__ void k_pcg_scalar(int op, double *__restrict__ scal, int *__restrict__ iflag,
                             const double *__restrict__ part, int nb, double tol, int maxit) {
    double s = 0.0;
    if (op != 5) s = sum_partials(part, nb);
    if (threadIdx.x != 0) return;
    switch (op) {
        case 0:
            scal[S_NORMB] = sqrt(s);
            scal[S_TOL] = tol;
            break;
        case 1: scal[S_X1] = s; break;
        case 2:
            if (iflag[I_STOP]) return;
            scal[S_PQ] = s;
            scal[S_LAM] = scal[S_X1] / s;
            break;
        case 3: {
            if (iflag[I_STOP]) return;
            scal[S_RR] = s;
            const double res = sqrt(s) / scal[S_NORMB];
            scal[S_RES] = res;
            const int its = iflag[I_ITS] + 1;
            iflag[I_ITS] = its;
            if (res < tol) {
                iflag[I_DONE] = 1;
                iflag[I_STOP] = 1;
            } else if (its >= maxit || !(res == res)) {
                iflag[I_STOP] = 1;
            }
            break;
        }
        case 4:
            if (iflag[I_STOP]) return;
            scal[S_BETA] = s / scal[S_X1];
            scal[S_X1] = s;
            break;
        case 5:
            iflag[I_ITS] = 0;
            iflag[I_DONE] = 0;
            iflag[I_STOP] = 0;
            scal[S_RES] = 1.0;
            break;
    }
}

void launch_pcg_scalar(int op, double *scal, int *iflag, const double *partial, int nb, double tol, int maxit,
                       cudaStream_t s) {
    ++g_launches;
    k_pcg_scalar<<<1, VB, 0, s>>>(op, scal, iflag, partial, nb, tol, maxit);
}

// x += lambda p; r -= lambda q; partial sums of r.r
__global__ void k_pcg_update(double *__restrict__ x, double *__restrict__ r, const double *__restrict__ p,
                             const double *__restrict__ q, int64_t n, const double *__restrict__ scal,
                             const int *__restrict__ iflag, double *__restrict__ part) {
    if (iflag[I_STOP]) return;
    const double lam = scal[S_LAM];
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)VB + threadIdx.x; i < n; i += (int64_t)gridDim.x * VB) {
        x[i] = x[i] + lam * p[i];
        const double ri = r[i] - lam * q[i];
        r[i] = ri;
        s += ri * ri;
    }
    s = block_reduce(s);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

void launch_pcg_update(double *x, double *r, const double *p, const double *q, int64_t n, const double *scal,
                       int *iflag, double *partial, int nb, cudaStream_t s) {
    ++g_launches;
    k_pcg_update<<<nb, VB, 0, s>>>(x, r, p, q, n, scal, iflag, partial);
}

// p = z + beta p
__global__ void k_pcg_pupdate(double *__restrict__ p, const double *__restrict__ z, int64_t n,
                              const double *__restrict__ scal, const int *__restrict__ iflag) {
    if (iflag[I_STOP]) return;
    const double beta = scal[S_BETA];
    for (int64_t i = blockIdx.x * (int64_t)VB + threadIdx.x; i < n; i += (int64_t)gridDim.x * VB)
        p[i] = z[i] + beta * p[i];
}

void launch_pcg_pupdate(double *p, const double *z, int64_t n, const double *scal, const int *iflag, cudaStream_t s) {
    ++g_launches;
    k_pcg_pupdate<<<reduce_blocks(n), VB, 0, s>>>(p, z, n, scal, iflag);
}

// r = b - Ax
__global__ void k_residual(double *__restrict__ r, const double *__restrict__ b, const double *__restrict__ Ax,
                           int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)VB + threadIdx.x; i < n; i += (int64_t)gridDim.x * VB) r[i] = b[i] - Ax[i];
}
void launch_residual(double *r, const double *b, const double *Ax, int64_t n, cudaStream_t s) {
    ++g_launches;
    k_residual<<<reduce_blocks(n), VB, 0, s>>>(r, b, Ax, n);
}

__global__ void k_scale(double *__restrict__ x, double a, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)VB + threadIdx.x; i < n; i += (int64_t)gridDim.x * VB) x[i] *= a;
}
void launch_scale(double *x, double a, int64_t n, cudaStream_t s) {
    ++g_launches;
    k_scale<<<reduce_blocks(n), VB, 0, s>>>(x, a, n);
}

__global__ void k_cast_f32(const double *__restrict__ a, float *__restrict__ b, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)VB + threadIdx.x; i < n; i += (int64_t)gridDim.x * VB) b[i] = (float)a[i];
}
__global__ void k_cast_f64(const float *__restrict__ a, double *__restrict__ b, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)VB + threadIdx.x; i < n; i += (int64_t)gridDim.x * VB) b[i] = (double)a[i];
}
void launch_cast_f32(const double *a, float *b, int64_t n, cudaStream_t s) {
    ++g_launches;
    k_cast_f32<<<reduce_blocks(n), VB, 0, s>>>(a, b, n);
}
void launch_cast_f64(const float *a, double *b, int64_t n, cudaStream_t s) {
    ++g_launches;
    k_cast_f64<<<reduce_blocks(n), VB, 0, s>>>(a, b, n);
}

}  // namespace sgld
