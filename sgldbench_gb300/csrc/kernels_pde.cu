// PDE (Helmholtz) density filter (src/TopOpti_PDEFiltering_matrixFree.m:1-56,
// src/TopOpti_BuildPDEfilter_matrixFree.m:1-43): the element field is spread
// to the nodes (x_e / 8 to each corner), K_pde t = src is solved by the
// reference's Jacobi-preconditioned CG with the scalar 8 x 8 element matrix
// K_pde = r^2 dN'dN + N'WN shared by all active elements, and the nodal
// solution is averaged back to the elements.
//
// Kernels are node-centric gathers on the full grid (deterministic: every
// output is written by one thread summing in a fixed order).  The element
// matrix Kp (row-major 8 x 8, in the context's own device buffer, since it
// depends on the call's radius) is in the reference's corner order j (offsets
// (dy, dx, dz) = (1,0,0),(1,1,0),(0,1,0),(0,0,0),(1,0,1),(1,1,1),(0,1,1),(0,0,1)).
#include "sgld_internal.cuh"

namespace sgld {

__constant__ int c_pdy[8] = {1, 1, 0, 0, 1, 1, 0, 0};
__constant__ int c_pdx[8] = {0, 1, 1, 0, 0, 1, 1, 0};
__constant__ int c_pdz[8] = {0, 0, 0, 0, 1, 1, 1, 1};

void upload_kpde(const double *K, double *d_kp, cudaStream_t s) {
    cudaMemcpyAsync(d_kp, K, sizeof(double) * 64, cudaMemcpyHostToDevice, s);
}

// node n is corner j of element (iy - dy_j, ix - dx_j, iz - dz_j)
__device__ __forceinline__ int64_t corner_elem(int iy, int ix, int iz, int j, int ny, int nx, int nz) {
    const int ey = iy - c_pdy[j], ex = ix - c_pdx[j], ez = iz - c_pdz[j];
    if (ey < 0 || ex < 0 || ez < 0 || ey >= ny || ex >= nx || ez >= nz) return -1;
    return (int64_t)ey + (int64_t)ny * (ex + (int64_t)nx * ez);
}

// src_n = sum over corners j (ascending) of x_e * (1/8), active elements only
// (the accumarray over eNodMat columns of TopOpti_PDEFiltering_matrixFree.m:8-17)
__global__ void k_pde_e2n(const double *__restrict__ xe, const uint8_t *__restrict__ eact, int ny, int nx, int nz,
                          double *__restrict__ yn) {
    const int NY = ny + 1, NX = nx + 1;
    const int64_t nn = (int64_t)NY * NX * (nz + 1);
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const int iy = (int)(n % NY), ix = (int)((n / NY) % NX), iz = (int)(n / ((int64_t)NY * NX));
    double s = 0.0;
    for (int j = 0; j < 8; ++j) {
        const int64_t e = corner_elem(iy, ix, iz, j, ny, nx, nz);
        if (e >= 0 && eact[e]) s += xe[e] * (1.0 / 8.0);
    }
    yn[n] = s;
}

// y = K_pde u (scalar field), optional partial sums of u.y per CTA
__global__ void k_pde_kbyu(const double *__restrict__ u, const uint8_t *__restrict__ eact, int ny, int nx, int nz,
                           const double *__restrict__ Kp, double *__restrict__ y, double *__restrict__ partial) {
    const int NY = ny + 1, NX = nx + 1;
    const int64_t nn = (int64_t)NY * NX * (nz + 1);
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double acc = 0.0, dot = 0.0;
    if (n < nn) {
        const int iy = (int)(n % NY), ix = (int)((n / NY) % NX), iz = (int)(n / ((int64_t)NY * NX));
        for (int j = 0; j < 8; ++j) {
            const int64_t e = corner_elem(iy, ix, iz, j, ny, nx, nz);
            if (e < 0 || !eact[e]) continue;
            const int ey = iy - c_pdy[j], ex = ix - c_pdx[j], ez = iz - c_pdz[j];
            double s = 0.0;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int64_t m = (int64_t)(ey + c_pdy[k]) + (int64_t)NY * ((ex + c_pdx[k]) + (int64_t)NX * (ez + c_pdz[k]));
                s += Kp[8 * j + k] * u[m];
            }
            acc += s;
        }
        y[n] = acc;
        dot = u[n] * acc;
    }
    if (partial) {
        __shared__ double red[8];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dot;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[i];
            partial[blockIdx.x] = t;
        }
    }
}

// dinv_n = 1 / sum of diag(K_pde) over the active elements at n (0 where none)
__global__ void k_pde_diag(const uint8_t *__restrict__ eact, int ny, int nx, int nz, const double *__restrict__ Kp,
                           double *__restrict__ dinv) {
    const int NY = ny + 1, NX = nx + 1;
    const int64_t nn = (int64_t)NY * NX * (nz + 1);
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const int iy = (int)(n % NY), ix = (int)((n / NY) % NX), iz = (int)(n / ((int64_t)NY * NX));
    double d = 0.0;
    for (int j = 0; j < 8; ++j) {
        const int64_t e = corner_elem(iy, ix, iz, j, ny, nx, nz);
        if (e >= 0 && eact[e]) d += Kp[9 * j];
    }
    dinv[n] = d > 0.0 ? 1.0 / d : 0.0;
}

// z = dinv .* r with partial sums of z.r
__global__ void k_pde_jacobi(const double *__restrict__ r, const double *__restrict__ dinv, int64_t n,
                             double *__restrict__ z, double *__restrict__ partial) {
    double dot = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = dinv[i] * r[i];
        z[i] = v;
        dot += v * r[i];
    }
    __shared__ double red[8];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dot;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[i];
        partial[blockIdx.x] = t;
    }
}

// x_e = (sum over the 8 corners k of t) * (1/8) for active elements
__global__ void k_pde_n2e(const double *__restrict__ t, const uint8_t *__restrict__ eact, int ny, int nx, int nz,
                          double *__restrict__ xe) {
    const int64_t nel = (int64_t)ny * nx * nz;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= nel) return;
    double s = 0.0;
    if (eact[e]) {
        const int ey = (int)(e % ny), ex = (int)((e / ny) % nx), ez = (int)(e / ((int64_t)ny * nx));
        const int NY = ny + 1, NX = nx + 1;
        for (int k = 0; k < 8; ++k)
            s += t[(int64_t)(ey + c_pdy[k]) + (int64_t)NY * ((ex + c_pdx[k]) + (int64_t)NX * (ez + c_pdz[k]))];
        s *= (1.0 / 8.0);
    }
    xe[e] = s;
}

static unsigned nblk(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

void launch_pde_e2n(const Level &l0, const double *xe, double *yn, cudaStream_t s) {
    ++g_launches;
    k_pde_e2n<<<nblk(l0.nnode, 256), 256, 0, s>>>(xe, l0.eact, l0.ny, l0.nx, l0.nz, yn);
}
int launch_pde_kbyu(const Level &l0, const double *Kp, const double *u, double *y, double *partial, cudaStream_t s) {
    ++g_launches;
    const unsigned nb = nblk(l0.nnode, 256);
    k_pde_kbyu<<<nb, 256, 0, s>>>(u, l0.eact, l0.ny, l0.nx, l0.nz, Kp, y, partial);
    return (int)nb;
}
void launch_pde_diag(const Level &l0, const double *Kp, double *dinv, cudaStream_t s) {
    ++g_launches;
    k_pde_diag<<<nblk(l0.nnode, 256), 256, 0, s>>>(l0.eact, l0.ny, l0.nx, l0.nz, Kp, dinv);
}
void launch_pde_jacobi(const double *r, const double *dinv, int64_t n, double *z, double *partial, int nb,
                       cudaStream_t s) {
    ++g_launches;
    k_pde_jacobi<<<nb, 256, 0, s>>>(r, dinv, n, z, partial);
}
void launch_pde_n2e(const Level &l0, const double *t, double *xe, cudaStream_t s) {
    ++g_launches;
    k_pde_n2e<<<nblk(l0.nel, 256), 256, 0, s>>>(t, l0.eact, l0.ny, l0.nx, l0.nz, xe);
}

}  // namespace sgld
