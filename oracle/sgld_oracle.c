/*
 * sgld_oracle.c -- CPU restatement (C + OpenMP) of SGLDBench's MEX kernels.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle's element-kernel layer:
 * the product never links it.  It is used by tests/, by the smoke check and
 * as the CPU baseline ("port") that bench.py times on the host cores.  Each
 * function restates one reference MEX kernel (SGLDBench src/MEXfuncs/, file
 * and lines cited per function) in the reference's own data formats:
 * 1-based int32 index tables stored column-major, node-major interleaved DOF
 * vectors for K*u, n-by-3 column-major arrays for the transfer operators, and
 * the 8-colour element partition for race-free parallel scatter.
 *
 * Colour lists are passed flattened: `cidx` holds the concatenated 1-based
 * element lists and `coff[c]..coff[c+1]` delimits colour c.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t i64;
typedef int32_t i32;

/* y = sum_e E_e * Ke * u_e  (Solving_KbyU_MatrixFree_mex.cpp:53-102, 105-138). */
void orc_kbyu(const double *U, const i32 *eNodMat, i64 numEl, const double *Ke, const double *E,
              const i32 *cidx, const i64 *coff, int ncol, double *Y, i64 numDOFs) {
#pragma omp parallel for schedule(static)
    for (i64 i = 0; i < numDOFs; ++i) Y[i] = 0.0;
    for (int c = 0; c < ncol; ++c) {
#pragma omp parallel for schedule(static)
        for (i64 k = coff[c]; k < coff[c + 1]; ++k) {
            i64 e = (i64)cidx[k] - 1;
            double ue[24], ye[24];
            i64 nd[8];
            for (int j = 0; j < 8; ++j) {
                nd[j] = (i64)eNodMat[e + j * numEl] - 1;
                for (int d = 0; d < 3; ++d) ue[3 * j + d] = U[3 * nd[j] + d];
            }
            for (int r = 0; r < 24; ++r) ye[r] = 0.0;
            for (int col = 0; col < 24; ++col) {   /* column-major Ke, as the MEX does */
                const double uc = ue[col];
                const double *kc = Ke + 24 * col;
                for (int r = 0; r < 24; ++r) ye[r] += kc[r] * uc;
            }
            for (int r = 0; r < 24; ++r) ye[r] *= E[e];
            for (int j = 0; j < 8; ++j)
                for (int d = 0; d < 3; ++d) Y[3 * nd[j] + d] += ye[3 * j + d];
        }
    }
}

/* r_c = R r_f  (Solving_Restriction_MatrixFree_mex.cpp:52-121, 182-210).
 * rF: nFine x 3, transferMat: m x Mc (m = 27 or 125), RI: m x 8 (the
 * reference passes RI' as 8 x m; here the m x 8 table is read directly),
 * eNodMat: Mc x 8, out rC: nCoarse x 3. */
void orc_restriction(const double *rF, i64 nFine, const i32 *transferMat, int m, const double *RI,
                     const i32 *eNodMat, i64 Mc, i64 nCoarse, i64 nGhost, const i32 *solidMap,
                     const double *coeffi, const i32 *cidx, const i64 *coff, int ncol, double *rC) {
    double *g = (double *)calloc((size_t)(3 * nGhost), sizeof(double));
    for (i64 i = 0; i < 3 * nCoarse; ++i) rC[i] = 0.0;
    for (int d = 0; d < 3; ++d) {
#pragma omp parallel for schedule(static)
        for (i64 j = 0; j < nFine; ++j) {
            i64 gj = (i64)solidMap[j] - 1;
            g[gj + d * nGhost] = rF[j + d * nFine] / coeffi[gj];
        }
    }
    for (int c = 0; c < ncol; ++c) {
#pragma omp parallel for schedule(static)
        for (i64 k = coff[c]; k < coff[c + 1]; ++k) {
            i64 e = (i64)cidx[k] - 1;
            double acc[3][8];
            memset(acc, 0, sizeof acc);
            for (int q = 0; q < m; ++q) {
                i64 gn = (i64)transferMat[(i64)m * e + q] - 1;
                for (int d = 0; d < 3; ++d) {
                    const double v = g[gn + d * nGhost];
                    for (int a = 0; a < 8; ++a) acc[d][a] += RI[q + a * m] * v;
                }
            }
            for (int a = 0; a < 8; ++a) {
                i64 cn = (i64)eNodMat[e + a * Mc] - 1;
                for (int d = 0; d < 3; ++d) rC[cn + d * nCoarse] += acc[d][a];
            }
        }
    }
    free(g);
}

/* x_f = P x_c  (Solving_Interpolation_MatrixFree_mex.cpp:55-129, 182-219). */
void orc_interpolation(const double *xC, i64 nCoarse, const i32 *transferMat, int m, const double *RI,
                       const i32 *eNodMat, i64 Mc, i64 nFine, i64 nGhost, const i32 *solidMap,
                       const double *coeffi, const i32 *cidx, const i64 *coff, int ncol, double *xF) {
    double *g = (double *)calloc((size_t)(3 * nGhost), sizeof(double));
    for (int c = 0; c < ncol; ++c) {
#pragma omp parallel for schedule(static)
        for (i64 k = coff[c]; k < coff[c + 1]; ++k) {
            i64 e = (i64)cidx[k] - 1;
            double xe[3][8];
            for (int a = 0; a < 8; ++a) {
                i64 cn = (i64)eNodMat[e + a * Mc] - 1;
                for (int d = 0; d < 3; ++d) xe[d][a] = xC[cn + d * nCoarse];
            }
            for (int q = 0; q < m; ++q) {
                i64 gn = (i64)transferMat[(i64)m * e + q] - 1;
                for (int d = 0; d < 3; ++d) {
                    double s = 0.0;
                    for (int a = 0; a < 8; ++a) s += RI[q + a * m] * xe[d][a];
                    g[gn + d * nGhost] += s;
                }
            }
        }
    }
    for (int d = 0; d < 3; ++d) {
#pragma omp parallel for schedule(static)
        for (i64 j = 0; j < nFine; ++j) {
            i64 gj = (i64)solidMap[j] - 1;
            xF[j + d * nFine] = g[gj + d * nGhost] / coeffi[gj];
        }
    }
    free(g);
}

/* ce_e = u_e' Ke u_e  (TopOpti_CmptUnitCompliance_mex.cpp:40-58, 61-88). */
void orc_unit_compliance(const double *U, const i32 *eNodMat, i64 numEl, const double *Ke, double *ce) {
#pragma omp parallel for schedule(static)
    for (i64 e = 0; e < numEl; ++e) {
        double ue[24], y[24];
        for (int j = 0; j < 8; ++j) {
            i64 n = (i64)eNodMat[e + j * numEl] - 1;
            for (int d = 0; d < 3; ++d) ue[3 * j + d] = U[3 * n + d];
        }
        for (int r = 0; r < 24; ++r) y[r] = 0.0;
        for (int col = 0; col < 24; ++col)
            for (int r = 0; r < 24; ++r) y[r] += Ke[r + 24 * col] * ue[col];
        double q = 0.0;
        for (int r = 0; r < 24; ++r) q += ue[r] * y[r];
        ce[e] = q;
    }
}

/* Galerkin coarse element matrix from per-child 24x24 matrices:
 *   tmpK (nd x nd) = sum_q scatter(child_q) via localMapping;  Kc = P' tmpK P.
 * Shared by the two assembly kernels below.  P: nd x 24 dense, column-major. */
static void galerkin_one(const double *const *child, int nq, const i32 *lmap, const double *P, int nd,
                         double *tmpK, double *B, double *Kc) {
    memset(tmpK, 0, sizeof(double) * (size_t)nd * nd);
    for (int q = 0; q < nq; ++q) {
        if (!child[q]) continue;
        for (int k = 0; k < 576; ++k) tmpK[lmap[k + 576 * q] - 1] += child[q][k];
    }
    /* B (24 x nd) = P' tmpK */
    memset(B, 0, sizeof(double) * 24 * (size_t)nd);
    for (int col = 0; col < nd; ++col)
        for (int r = 0; r < nd; ++r) {
            const double t = tmpK[r + (i64)nd * col];
            if (t == 0.0) continue;
            for (int a = 0; a < 24; ++a) B[a + 24 * col] += P[r + (i64)nd * a] * t;
        }
    /* Kc (24 x 24) = B P */
    for (int b = 0; b < 24; ++b)
        for (int a = 0; a < 24; ++a) {
            double s = 0.0;
            for (int r = 0; r < nd; ++r) s += B[a + 24 * r] * P[r + (i64)nd * b];
            Kc[a + 24 * b] = s;
        }
}

/* Level-2 stencils from the finest level: Ks_E = sum_q E_q H_q with the
 * templates H_q = P' scatter_q(Ke) P  (Solving_AssembleCmptStencilFromFinestLevel.cpp:71-169). */
void orc_assemble_finest(const double *Ke, const double *E, const i32 *eum, i64 Mc, int nq, const double *P,
                         const i32 *lmap, int nProjNodes, double *Ks) {
    const int nd = 3 * nProjNodes;
    double *H = (double *)malloc(sizeof(double) * 576 * (size_t)nq);
    double *tmpK = (double *)malloc(sizeof(double) * (size_t)nd * nd);
    double *B = (double *)malloc(sizeof(double) * 24 * (size_t)nd);
    const double **child = (const double **)calloc((size_t)nq, sizeof(double *));
    for (int q = 0; q < nq; ++q) {
        for (int j = 0; j < nq; ++j) child[j] = (j == q) ? Ke : NULL;
        galerkin_one(child, nq, lmap, P, nd, tmpK, B, H + 576 * (i64)q);
    }
    free(child);
    free(tmpK);
    free(B);
#pragma omp parallel for schedule(static)
    for (i64 i = 0; i < Mc; ++i) {
        double *out = Ks + 576 * i;
        for (int t = 0; t < 576; ++t) out[t] = 0.0;
        for (int q = 0; q < nq; ++q) {
            i32 ch = eum[i + q * Mc];
            if (ch == 0) continue;
            const double ev = E[ch - 1];
            const double *hq = H + 576 * (i64)q;
            for (int t = 0; t < 576; ++t) out[t] += ev * hq[t];
        }
    }
    free(H);
}

/* Deeper levels: Ks_E = P' (sum_q scatter_q(Ks_child)) P
 * (Solving_AssembleCmptStencilFromNonFinestLevel.cpp:248-313). */
void orc_assemble_nonfinest(const double *KsPrev, const i32 *eum, i64 Mc, int nq, const double *P,
                            const i32 *lmap, int nProjNodes, double *Ks) {
    const int nd = 3 * nProjNodes;
#pragma omp parallel
    {
        double *tmpK = (double *)malloc(sizeof(double) * (size_t)nd * nd);
        double *B = (double *)malloc(sizeof(double) * 24 * (size_t)nd);
        const double **child = (const double **)calloc((size_t)nq, sizeof(double *));
#pragma omp for schedule(static)
        for (i64 i = 0; i < Mc; ++i) {
            for (int q = 0; q < nq; ++q) {
                i32 ch = eum[i + q * Mc];
                child[q] = ch ? KsPrev + 576 * (i64)(ch - 1) : NULL;
            }
            galerkin_one(child, nq, lmap, P, nd, tmpK, B, Ks + 576 * i);
        }
        free(tmpK);
        free(B);
        free((void *)child);
    }
}

/* Cone density filter (TopOpti_SetupDensityFilter_mex.cpp:23-50 and
 * TopOpti_PerformDensityFiltering_mex.cpp:75-102).  x == NULL computes the
 * weight sums Hs, otherwise the filtered field. */
void orc_density_filter(const double *x, double rmin, const i32 *eleMapForward, int resX, int resY,
                        int resZ, double *y) {
    const int r = (int)ceil(rmin) - 1;
    const i64 rxy = (i64)resX * resY;
#pragma omp parallel for collapse(3) schedule(static)
    for (int kk = 0; kk < resZ; ++kk)
        for (int ii = 0; ii < resX; ++ii)
            for (int jj = 0; jj < resY; ++jj) {
                i32 e1 = eleMapForward[kk * rxy + (i64)ii * resY + jj];
                if (!e1) continue;
                double acc = 0.0;
                for (int k2 = (kk - r > 0 ? kk - r : 0); k2 <= (kk + r < resZ - 1 ? kk + r : resZ - 1); ++k2)
                    for (int i2 = (ii - r > 0 ? ii - r : 0); i2 <= (ii + r < resX - 1 ? ii + r : resX - 1); ++i2)
                        for (int j2 = (jj - r > 0 ? jj - r : 0); j2 <= (jj + r < resY - 1 ? jj + r : resY - 1); ++j2) {
                            i32 e2 = eleMapForward[k2 * rxy + (i64)i2 * resY + j2];
                            if (!e2) continue;
                            double w = rmin - sqrt((double)((ii - i2) * (ii - i2) + (jj - j2) * (jj - j2) +
                                                            (kk - k2) * (kk - k2)));
                            if (w < 0.0) w = 0.0;
                            acc += x ? w * x[e2 - 1] : w;
                        }
                y[e1 - 1] = acc;
            }
}
