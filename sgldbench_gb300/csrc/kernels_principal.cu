// Principal stresses (src/FEA_ComputePrincipalStress.m:1-8) and the dominant
// principal direction per element
// (src/Common_ExtractDominantDirectionsFromPrincipalStressDirections.m:1-39).
//
// The reference assembles A = [xx xy zx; xy yy yz; zx yz zz] from a Cartesian
// stress [xx yy zz yz zx xy] and calls MATLAB eig (ascending eigenvalues for
// a symmetric matrix); its output row is [l1 v1 l2 v2 l3 v3].  Here the 3x3
// symmetric eigenproblem is solved per node / element with the cyclic Jacobi
// method (Golub & Van Loan, Matrix Computations, sec. 8.5: 2x2 symmetric Schur
// rotations applied to the off-diagonal pairs until they vanish), the pairs
// sorted ascending, and every eigenvector signed so that its entry of largest
// magnitude is positive (eig leaves the sign open; this fixes one).
#include "sgld_internal.cuh"

namespace sgld {

// A (row-major 3x3, symmetric) -> eigenvalues w (ascending), eigenvectors as
// columns of V (row-major, V[3*i + k] = component i of vector k)
__device__ void sym3_eig(const double (&Ain)[9], double (&w)[3], double (&V)[9]) {
    double A[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) A[i] = Ain[i];
#pragma unroll
    for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
    const double fro = sqrt(A[0] * A[0] + A[4] * A[4] + A[8] * A[8] + 2.0 * (A[1] * A[1] + A[2] * A[2] + A[5] * A[5]));
    for (int sweep = 0; sweep < 16; ++sweep) {
        const double off = sqrt(2.0 * (A[1] * A[1] + A[2] * A[2] + A[5] * A[5]));
        if (!(off > 1e-17 * fro)) break;
#pragma unroll
        for (int pq = 0; pq < 3; ++pq) {
            const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
            const double apq = A[3 * p + q];
            if (apq == 0.0) continue;
            // symmetric Schur: c, s zeroing A[p][q]
            const double theta = (A[3 * q + q] - A[3 * p + p]) / (2.0 * apq);
            const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
            const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
            // A <- J' A J with J = rotation in the (p, q) plane
#pragma unroll
            for (int k = 0; k < 3; ++k) {   // columns p, q
                const double akp = A[3 * k + p], akq = A[3 * k + q];
                A[3 * k + p] = c * akp - s * akq;
                A[3 * k + q] = s * akp + c * akq;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {   // rows p, q
                const double apk = A[3 * p + k], aqk = A[3 * q + k];
                A[3 * p + k] = c * apk - s * aqk;
                A[3 * q + k] = s * apk + c * aqk;
            }
            A[3 * p + q] = A[3 * q + p] = 0.0;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const double vkp = V[3 * k + p], vkq = V[3 * k + q];
                V[3 * k + p] = c * vkp - s * vkq;
                V[3 * k + q] = s * vkp + c * vkq;
            }
        }
    }
    w[0] = A[0];
    w[1] = A[4];
    w[2] = A[8];
    // ascending order (stable for ties)
    int o[3] = {0, 1, 2};
    if (w[o[1]] < w[o[0]]) { const int t = o[0]; o[0] = o[1]; o[1] = t; }
    if (w[o[2]] < w[o[1]]) { const int t = o[1]; o[1] = o[2]; o[2] = t; }
    if (w[o[1]] < w[o[0]]) { const int t = o[0]; o[0] = o[1]; o[1] = t; }
    double ws[3], Vs[9];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        ws[k] = w[o[k]];
        int big = 0;
        double bm = -1.0;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const double a = fabs(V[3 * i + o[k]]);
            if (a > bm) { bm = a; big = i; }
        }
        const double sg = V[3 * big + o[k]] < 0.0 ? -1.0 : 1.0;
#pragma unroll
        for (int i = 0; i < 3; ++i) Vs[3 * i + k] = sg * V[3 * i + o[k]];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) w[k] = ws[k];
#pragma unroll
    for (int i = 0; i < 9; ++i) V[i] = Vs[i];
}

__device__ __forceinline__ void stress_matrix3(const double *s6, double (&A)[9]) {
    // [xx yy zz yz zx xy] -> [xx xy zx; xy yy yz; zx yz zz]
    A[0] = s6[0]; A[1] = s6[5]; A[2] = s6[4];
    A[3] = s6[5]; A[4] = s6[1]; A[5] = s6[3];
    A[6] = s6[4]; A[7] = s6[3]; A[8] = s6[2];
}

// per node: [l1 v1 l2 v2 l3 v3] (12 doubles), zeros at inactive nodes
__global__ void k_principal_nodes(const double *__restrict__ s6, const uint8_t *__restrict__ nflag, int64_t nn,
                                  double *__restrict__ ps) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= nn) return;
    double out[12];
#pragma unroll
    for (int i = 0; i < 12; ++i) out[i] = 0.0;
    if (nflag[n] & NF_ACTIVE) {
        double A[9], w[3], V[9];
        stress_matrix3(s6 + 6 * n, A);
        sym3_eig(A, w, V);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            out[4 * k] = w[k];
#pragma unroll
            for (int i = 0; i < 3; ++i) out[4 * k + 1 + i] = V[3 * i + k];
        }
    }
#pragma unroll
    for (int i = 0; i < 12; ++i) ps[12 * n + i] = out[i];
}

// per element: centroid stress (mean of the 8 nodal stresses, the shape
// functions at the centroid), principal directions, the direction of the
// principal stress of largest magnitude (first of equal maxima, as max does)
__global__ void k_dominant_dir(const double *__restrict__ s6, const uint8_t *__restrict__ eact, int ny, int nx,
                               int nz, double *__restrict__ dir) {
    const int64_t nel = (int64_t)ny * nx * nz;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= nel) return;
    double d[3] = {0.0, 0.0, 0.0};
    if (eact[e]) {
        const int ey = (int)(e % ny), ex = (int)((e / ny) % nx), ez = (int)(e / ((int64_t)ny * nx));
        const int NY = ny + 1, NX = nx + 1;
        const int cdy[8] = {1, 1, 0, 0, 1, 1, 0, 0}, cdx[8] = {0, 1, 1, 0, 0, 1, 1, 0},
                  cdz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
        double v[6] = {0, 0, 0, 0, 0, 0};
        for (int k = 0; k < 8; ++k) {
            const int64_t m = (int64_t)(ey + cdy[k]) + (int64_t)NY * ((ex + cdx[k]) + (int64_t)NX * (ez + cdz[k]));
            for (int c = 0; c < 6; ++c) v[c] += 0.125 * s6[6 * m + c];
        }
        double A[9], w[3], V[9];
        stress_matrix3(v, A);
        sym3_eig(A, w, V);
        int best = 0;
        double bm = fabs(w[0]);
#pragma unroll
        for (int k = 1; k < 3; ++k)
            if (fabs(w[k]) > bm) { bm = fabs(w[k]); best = k; }
#pragma unroll
        for (int i = 0; i < 3; ++i) d[i] = V[3 * i + best];
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) dir[3 * e + i] = d[i];
}

void launch_principal(const Level &l0, const double *s6, double *ps_node, double *dir_elem, cudaStream_t s) {
    if (ps_node) {
        ++g_launches;
        k_principal_nodes<<<(unsigned)((l0.nnode + 127) / 128), 128, 0, s>>>(s6, l0.nflag, l0.nnode, ps_node);
    }
    if (dir_elem) {
        ++g_launches;
        k_dominant_dir<<<(unsigned)((l0.nel + 127) / 128), 128, 0, s>>>(s6, l0.eact, l0.ny, l0.nx, l0.nz,
                                                                        dir_elem);
    }
}

}  // namespace sgld
