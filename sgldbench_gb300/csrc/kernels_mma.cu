// MMA update for one constraint on the device (src/MEXfuncs/MMA_mex.cpp:6-54
// with src/MEXfuncs/MMAseq.cpp, Svanberg's method of moving asymptotes with a
// dual interior-point subproblem solver).
//
// MMA_mex builds a fresh MMAseq(n, 1, a=0, c=100, d=0) per call, so the
// asymptotes are the initial ones, L = x - 0.5 (xmax - xmin) and
// U = x + 0.5 (xmax - xmin) (MMAseq.cpp:460-466), and the subproblem
// coefficients (MMAseq.cpp:503-545) are functions of the element's own inputs.
// Every kernel therefore recomputes them from (x, xmin, xmax, df0dx, dfdx)
// instead of storing eight n-vectors; the dual variables (lambda, mu) and the
// interior-point iteration are scalar and run on the host, which reads two
// reduced sums per Newton step.
#include "sgld_internal.cuh"

namespace sgld {

struct MmaCoef {
    double L, U, alpha, beta, p0, q0, p1, q1;
};

__device__ __forceinline__ MmaCoef mma_coef(double x, double xmin, double xmax, double df0, double dg) {
    MmaCoef c;
    c.L = x - 0.5 * (xmax - xmin);
    c.U = x + 0.5 * (xmax - xmin);
    c.alpha = fmax(xmin, 0.9 * c.L + 0.1 * x);
    c.beta = fmin(xmax, 0.9 * c.U + 0.1 * x);
    const double feps = 1.0e-6;
    const double ux = c.U - x, xl = x - c.L, ul = c.U - c.L;
    c.p0 = ux * ux * (fmax(0.0, df0) + 0.001 * fabs(df0) + 0.5 * feps / ul);
    c.q0 = xl * xl * (fmax(0.0, -df0) + 0.001 * fabs(df0) + 0.5 * feps / ul);
    c.p1 = ux * ux * fmax(0.0, dg);
    c.q1 = xl * xl * fmax(0.0, -dg);
    return c;
}

__device__ __forceinline__ void block_sum2(double a, double b, double *pa, double *pb) {
    __shared__ double ra[8], rb[8];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
        ra[threadIdx.x >> 5] = a;
        rb[threadIdx.x >> 5] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double sa = 0.0, sb = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            sa += ra[i];
            sb += rb[i];
        }
        *pa = sa;
        *pb = sb;
    }
}

// lam < 0: partial sums of p1/(U-x) + q1/(x-L) at x = xval (the constant b).
// lam >= 0: x(lam) = (sqrt(pl) L + sqrt(ql) U) / (sqrt(pl) + sqrt(ql)) clamped to
// [alpha, beta] (XYZofLAMBDA) into xout, with partial sums of
// p1/(U-x) + q1/(x-L) (DualGrad / DualResidual) and of PQ^2 df2 (DualHess).
__global__ void k_mma_eval(const double *__restrict__ xv, const double *__restrict__ xmin,
                           const double *__restrict__ xmax, const double *__restrict__ df0,
                           const double *__restrict__ dg, int64_t n, double lam, double *__restrict__ xout,
                           double *__restrict__ part1, double *__restrict__ part2) {
    double s1 = 0.0, s2 = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double x0 = xv[i];
        const MmaCoef c = mma_coef(x0, xmin[i], xmax[i], df0[i], dg[i]);
        if (lam < 0.0) {
            s1 += c.p1 / (c.U - x0) + c.q1 / (x0 - c.L);
            continue;
        }
        const double pl = c.p0 + c.p1 * lam, ql = c.q0 + c.q1 * lam;
        const double sp = sqrt(pl), sq = sqrt(ql);
        const double xp = (sp * c.L + sq * c.U) / (sp + sq);
        const double x = fmin(fmax(xp, c.alpha), c.beta);
        xout[i] = x;
        const double ux = c.U - x, xl = x - c.L;
        s1 += c.p1 / ux + c.q1 / xl;
        const double pq = c.p1 / (ux * ux) - c.q1 / (xl * xl);
        double df2 = -1.0 / (2.0 * pl / (ux * ux * ux) + 2.0 * ql / (xl * xl * xl));
        if (xp < c.alpha || xp > c.beta) df2 = 0.0;
        s2 += pq * pq * df2;
    }
    block_sum2(s1, s2, part1 + blockIdx.x, part2 + blockIdx.x);
}

__global__ void k_mma_finalize(const double *__restrict__ p1, const double *__restrict__ p2, int nb,
                               double *__restrict__ out) {
    __shared__ double r1[256], r2[256];
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        a += p1[i];
        b += p2[i];
    }
    r1[threadIdx.x] = a;
    r2[threadIdx.x] = b;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            r1[threadIdx.x] += r1[threadIdx.x + s];
            r2[threadIdx.x] += r2[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = r1[0];
        out[1] = r2[0];
    }
}

int mma_blocks(int64_t n) {
    const int64_t b = (n + 255) / 256;
    return (int)(b < 152 * 8 ? (b > 0 ? b : 1) : 152 * 8);
}

void launch_mma_eval(const double *xv, const double *xmin, const double *xmax, const double *df0, const double *dg,
                     int64_t n, double lam, double *xout, double *part1, double *part2, double *sums2,
                     cudaStream_t s) {
    const int nb = mma_blocks(n);
    g_launches += 2;
    k_mma_eval<<<nb, 256, 0, s>>>(xv, xmin, xmax, df0, dg, n, lam, xout, part1, part2);
    k_mma_finalize<<<1, 256, 0, s>>>(part1, part2, nb, sums2);
}

}  // namespace sgld
