// Host side of the C ABI (include/sgld_gpu.h): grid hierarchy, element
// matrices, assembly and the PCG driver.  Every entry point mirrors one
// function of the reference's solve path (cited in the header).
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <limits>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/sgld_gpu.h"
#include "sgld_internal.cuh"

using namespace sgld;

thread_local int64_t sgld::g_launches = 0;

namespace {

// ---------------------------------------------------------------------------
// element matrices (FEA_VoxelBasedElementStiffnessMatrix.m:10-23 and helpers)
// ---------------------------------------------------------------------------
const double kGauss = 0.577350269189626;   // FEA_GaussianIntegral.m:10-15
const double kGs[8] = {-kGauss, kGauss, kGauss, -kGauss, -kGauss, kGauss, kGauss, -kGauss};
const double kGt[8] = {-kGauss, -kGauss, kGauss, kGauss, -kGauss, -kGauss, kGauss, kGauss};
const double kGp[8] = {-kGauss, -kGauss, -kGauss, -kGauss, kGauss, kGauss, kGauss, kGauss};
// natural coordinates of the 8 nodes (FEA_ShapeFunction.m:11-18)
const double kNs[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
const double kNt[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
const double kNp[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
// reference corner j -> offsets (dy, dx, dz) on the grid (FEA_VoxelBasedDiscretization.m:72-79)
const int kCdy[8] = {1, 1, 0, 0, 1, 1, 0, 0};
const int kCdx[8] = {0, 1, 1, 0, 0, 1, 1, 0};
const int kCdz[8] = {0, 0, 0, 0, 1, 1, 1, 1};

void hooke(double nu, double S[6][6]) {   // FEA_HookeLaw.m:4-13 (E = 1)
    memset(S, 0, sizeof(double) * 36);
    const double c1 = (1 + nu) * (1 - 2 * nu), c2 = 2 * (1 + nu);
    S[0][0] = S[1][1] = S[2][2] = (1 - nu) / c1;
    S[0][1] = S[0][2] = S[1][0] = S[1][2] = S[2][0] = S[2][1] = nu / c1;
    S[3][3] = S[4][4] = S[5][5] = 1.0 / c2;
}

// strain-displacement matrix at Gauss point g: 6 x 24 (FEA_ElementStrainMatrix.m)
void strain_at(int g, double h, double B[6][24]) {
    const double s = kGs[g], t = kGt[g], p = kGp[g];
    memset(B, 0, sizeof(double) * 144);
    for (int n = 0; n < 8; ++n) {
        const double ds = 0.125 * kNs[n] * (1 + kNt[n] * t) * (1 + kNp[n] * p) * (2.0 / h);
        const double dt = 0.125 * kNt[n] * (1 + kNs[n] * s) * (1 + kNp[n] * p) * (2.0 / h);
        const double dp = 0.125 * kNp[n] * (1 + kNs[n] * s) * (1 + kNt[n] * t) * (2.0 / h);
        B[0][3 * n] = ds;
        B[1][3 * n + 1] = dt;
        B[2][3 * n + 2] = dp;
        B[3][3 * n + 1] = dp;
        B[3][3 * n + 2] = dt;
        B[4][3 * n] = dp;
        B[4][3 * n + 2] = ds;
        B[5][3 * n] = dt;
        B[5][3 * n + 1] = ds;
    }
}

void element_stiffness(double nu, double h, double Ke[576]) {
    double S[6][6], B[6][24];
    hooke(nu, S);
    const double w = h * h * h / 8.0;
    memset(Ke, 0, sizeof(double) * 576);
    for (int g = 0; g < 8; ++g) {
        strain_at(g, h, B);
        double SB[6][24];
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 24; ++j) {
                double v = 0;
                for (int k = 0; k < 6; ++k) v += S[i][k] * B[k][j];
                SB[i][j] = v * w;
            }
        for (int r = 0; r < 24; ++r)
            for (int c = 0; c < 24; ++c) {
                double v = 0;
                for (int k = 0; k < 6; ++k) v += B[k][r] * SB[k][c];
                Ke[r + 24 * c] += v;
            }
    }
}

// stress matrix M (48 x 24, column-major): corner stresses = M u_e
// (FEA_StressAnalysis.m:43-45: inv(sFM) * D * B).
void stress_matrix(double nu, double h, double M[48 * 24]) {
    double N[8][8];   // N[g][n] shape function n at Gauss point g
    for (int g = 0; g < 8; ++g)
        for (int n = 0; n < 8; ++n)
            N[g][n] = 0.125 * (1 + kNs[n] * kGs[g]) * (1 + kNt[n] * kGt[g]) * (1 + kNp[n] * kGp[g]);
    // invert N (8x8) by Gauss-Jordan with partial pivoting
    double A[8][16];
    for (int i = 0; i < 8; ++i)
        for (int j = 0; j < 16; ++j) A[i][j] = j < 8 ? N[i][j] : (j - 8 == i ? 1.0 : 0.0);
    for (int c = 0; c < 8; ++c) {
        int piv = c;
        for (int r = c + 1; r < 8; ++r)
            if (fabs(A[r][c]) > fabs(A[piv][c])) piv = r;
        for (int j = 0; j < 16; ++j) std::swap(A[c][j], A[piv][j]);
        const double d = A[c][c];
        for (int j = 0; j < 16; ++j) A[c][j] /= d;
        for (int r = 0; r < 8; ++r)
            if (r != c) {
                const double f = A[r][c];
                for (int j = 0; j < 16; ++j) A[r][j] -= f * A[c][j];
            }
    }
    double S[6][6], B[6][24], SB[8][6][24];
    hooke(nu, S);
    for (int g = 0; g < 8; ++g) {
        strain_at(g, h, B);
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 24; ++j) {
                double v = 0;
                for (int k = 0; k < 6; ++k) v += S[i][k] * B[k][j];
                SB[g][i][j] = v;
            }
    }
    for (int n = 0; n < 8; ++n)
        for (int k = 0; k < 6; ++k)
            for (int j = 0; j < 24; ++j) {
                double v = 0;
                for (int g = 0; g < 8; ++g) v += A[n][8 + g] * SB[g][k][j];
                M[(6 * n + k) + 48 * j] = v;
            }
}

// Ke in the Hadamard basis: verify the isotropic block structure and extract
// the 45 values in the kernels' block order.
const int kBlk[11][3] = {{3, 7, 14}, {4, 6, -1}, {5, 12, -1}, {8, 13, -1}, {9, 20, -1}, {10, 17, -1},
                         {11, 16, 18}, {15, 19, -1}, {21, -1, -1}, {22, -1, -1}, {23, -1, -1}};

bool hadamard_blocks(const double *Ke, double Kh45[KH_NNZ], std::string &why) {
    const int kmap[8] = {0, 1, 3, 2, 4, 5, 7, 6};   // reference corner -> bit index (ks | kt<<1 | kp<<2)
    double Kb[24][24];
    for (int j = 0; j < 8; ++j)
        for (int c = 0; c < 3; ++c)
            for (int jj = 0; jj < 8; ++jj)
                for (int cc = 0; cc < 3; ++cc)
                    Kb[3 * kmap[j] + c][3 * kmap[jj] + cc] = Ke[(3 * j + c) + 24 * (3 * jj + cc)];
    double H[8][8];
    for (int m = 0; m < 8; ++m)
        for (int k = 0; k < 8; ++k) {
            double v = 1;
            for (int ax = 0; ax < 3; ++ax)
                if ((m >> ax) & 1) v *= (((k >> ax) & 1) ? 1.0 : -1.0);
            H[m][k] = v;
        }
    double T[24][24], Kh[24][24];
    for (int r = 0; r < 24; ++r)
        for (int c = 0; c < 24; ++c) {
            double v = 0;
            for (int k = 0; k < 8; ++k) v += H[r / 3][k] * Kb[3 * k + r % 3][c];
            T[r][c] = v;
        }
    double mx = 0;
    for (int r = 0; r < 24; ++r)
        for (int c = 0; c < 24; ++c) {
            double v = 0;
            for (int k = 0; k < 8; ++k) v += T[r][3 * k + c % 3] * H[c / 3][k];
            Kh[r][c] = v / 64.0;
            mx = std::max(mx, fabs(Kh[r][c]));
        }
    bool in[24][24] = {};
    int o = 0;
    for (auto &b : kBlk) {
        int n = 0;
        while (n < 3 && b[n] >= 0) ++n;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                in[b[i]][b[j]] = true;
                Kh45[o++] = Kh[b[i]][b[j]];
            }
    }
    for (int r = 0; r < 24; ++r)
        for (int c = 0; c < 24; ++c) {
            if (!in[r][c] && fabs(Kh[r][c]) > 1e-12 * mx) {
                why = "element matrix does not have the isotropic hexahedral structure";
                return false;
            }
            if (fabs(Kh[r][c] - Kh[c][r]) > 1e-12 * mx) {
                why = "element matrix is not symmetric";
                return false;
            }
        }
    return true;
}

// level-2 templates H_q = P_q' Ke P_q for span s (column-major, q = child index, y fastest)
void make_templates(const double *Ke, int s, std::vector<double> &H) {
    const int nq = s * s * s;
    H.assign((size_t)nq * 576, 0.0);
    for (int q = 0; q < nq; ++q) {
        const int oy = q % s, ox = (q / s) % s, oz = q / (s * s);
        double W[8][8];
        for (int j = 0; j < 8; ++j) {
            const double py = oy + kCdy[j], px = ox + kCdx[j], pz = oz + kCdz[j];
            const double sn = -1.0 + 2.0 * px / s, tn = 1.0 - 2.0 * py / s, pn = -1.0 + 2.0 * pz / s;
            for (int a = 0; a < 8; ++a) W[j][a] = 0.125 * (1 + kNs[a] * sn) * (1 + kNt[a] * tn) * (1 + kNp[a] * pn);
        }
        double KP[24][24];   // Ke P_q
        for (int r = 0; r < 24; ++r)
            for (int a = 0; a < 8; ++a)
                for (int d = 0; d < 3; ++d) {
                    double v = 0;
                    for (int k = 0; k < 8; ++k) v += Ke[r + 24 * (3 * k + d)] * W[k][a];
                    KP[r][3 * a + d] = v;
                }
        double *h = H.data() + 576 * (size_t)q;
        for (int b = 0; b < 8; ++b)
            for (int c = 0; c < 3; ++c)
                for (int col = 0; col < 24; ++col) {
                    double v = 0;
                    for (int j = 0; j < 8; ++j) v += W[j][b] * KP[3 * j + c][col];
                    h[(3 * b + c) + 24 * col] = v;
                }
    }
}

template <typename T>
cudaError_t dalloc(T **p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    return cudaMalloc((void **)p, n * sizeof(T));
}

int fail(sgld_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->c.err = msg;
    return code;
}


#define CK(x)                                                                                            \
    do {                                                                                                 \
        cudaError_t e_ = (x);                                                                            \
        if (e_ != cudaSuccess) return fail(ctx, e_ == cudaErrorMemoryAllocation ? SGLD_ERR_NOMEM : SGLD_ERR_CUDA, \
                                           std::string(#x) + ": " + cudaGetErrorString(e_));             \
    } while (0)
#define CKL()                                                                                            \
    do {                                                                                                 \
        cudaError_t e_ = cudaGetLastError();                                                             \
        if (e_ != cudaSuccess) return fail(ctx, SGLD_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e_)); \
    } while (0)

// The finest level's active runs (Level::runs): the y-runs of every brick of
// 32 (y) x 8 (x) x 8 (z) nodes that holds an active node, in address order.
// Left empty when more than 85 % of the bricks are active (a solid box),
// where the flat float4 kernels stream faster.
int build_active_runs(sgld_ctx *ctx) {
    Level &l0 = ctx->c.lv[0];
    const int NY = l0.ny + 1, NX = l0.nx + 1, NZ = l0.nz + 1;
    const int64_t nn = (int64_t)NY * NX * NZ;
    if ((double)l0.nnode_active > 0.85 * (double)nn) return SGLD_OK;   // nearly full: the flat kernels run
    // the maximal y-runs of active nodes in address order, merged where they touch or lie
    // at most kRunGap floats apart, cut into chunks of at most kRunChunk floats on 16-byte
    // boundaries (kernels_mixed.cu)
    constexpr int64_t kRunChunk = 2048, kRunGap = 48;
    std::vector<int64_t> runs;
    runs.reserve((size_t)NX * NZ * 2);
    int64_t sb = -1, se = -1;   // current span [sb, se) in floats
    auto flush = [&]() {
        for (int64_t p = sb; p < se;) {
            int64_t q = std::min(se, p + kRunChunk);
            if (q < se) q &= ~(int64_t)3;   // interior cuts on 16-byte boundaries
            runs.push_back(p | ((q - p) << 40));
            p = q;
        }
    };
    const uint8_t *f = l0.h_nflag.data();
    for (int64_t n = 0; n < nn;) {
        if (!(f[n] & NF_ACTIVE)) {
            ++n;
            continue;
        }
        int64_t m = n + 1;   // the run ends at the column's end at the latest
        const int64_t col_end = (n / NY + 1) * NY;
        while (m < col_end && (f[m] & NF_ACTIVE)) ++m;
        // a gap of a few inactive nodes is bridged (their words are zero in every vector of
        // the inner solve, and the updates keep zeros zero): longer runs, fewer partial groups
        if (se >= 0 && 3 * n - se <= kRunGap) {
            se = 3 * m;
        } else {
            if (sb >= 0) flush();
            sb = 3 * n;
            se = 3 * m;
        }
        n = m;
    }
    if (sb >= 0) flush();    l0.nruns = (int64_t)runs.size();
    CK(dalloc(&l0.runs, runs.size()));
    CK(cudaMemcpy(l0.runs, runs.data(), sizeof(int64_t) * runs.size(), cudaMemcpyHostToDevice));
    return SGLD_OK;
}

int setup_templates(sgld_ctx *ctx) {
    Ctx &c = ctx->c;
    std::vector<double> H2, H4;
    make_templates(c.Ke, 2, H2);
    make_templates(c.Ke, 4, H4);
    if (c.d_H) cudaFree(c.d_H);
    // FP64 span-2 and span-4 templates, then the same values as (hi, lo) float
    // pairs for the double-float assembly kernel
    const size_t nh = H2.size() + H4.size();
    std::vector<double> all(2 * nh);
    std::copy(H2.begin(), H2.end(), all.begin());
    std::copy(H4.begin(), H4.end(), all.begin() + H2.size());
    float *pairs = reinterpret_cast<float *>(all.data() + nh);
    for (size_t i = 0; i < nh; ++i) {
        const float hi = (float)all[i];
        pairs[2 * i] = hi;
        pairs[2 * i + 1] = (float)(all[i] - (double)hi);
    }
    CK(dalloc(&c.d_H, 2 * nh));
    CK(cudaMemcpy(c.d_H, all.data(), all.size() * sizeof(double), cudaMemcpyHostToDevice));
    return bind_ctx(ctx);   // uploads c.Kh unless the device already holds an equal matrix
}

const double *templates(const Ctx &c, int S) { return S == 2 ? c.d_H : c.d_H + 8 * 576; }

// A dyadic hierarchy with more than two levels never needs the element
// matrices of level 2 (MATLAB index): its diagonal comes from the span-2
// templates and level 3 from the span-4 templates.
bool skip_level2_ks(const Ctx &c) { return c.L > 2 && c.lv[1].span == 2; }

// device V-cycle on full-grid vectors (Solving_Vcycle.m:12-50); partial dot z.r
int vcycle_dev(sgld_ctx *ctx, const double *r, double *z, double *partial, int *nb) {
    Ctx &c = ctx->c;
    const int L = c.L;
    if (ensure_coarse_m64(c)) return fail(ctx, SGLD_ERR_CUDA, "FP64 coarse inverse: CUDA error");
    const double *rf = r;
    for (int l = 1; l < L; ++l) {
        launch_restrict<double>(c.lv[l - 1], c.lv[l], rf, c.lv[l].r, c.stream);
        rf = c.lv[l].r;
    }
    launch_coarse_apply_f64(c, c.lv[L - 1].r, c.lv[L - 1].x, c.stream);
    for (int l = L - 2; l >= 0; --l) {
        const double *rl = (l == 0) ? r : c.lv[l].r;
        double *xl = (l == 0) ? z : c.lv[l].x;
        launch_prolong_smooth<double>(c.lv[l], c.lv[l + 1], c.lv[l + 1].x, rl, c.lv[l].idiag, c.omega, xl, l == 0,
                                      l == 0 ? partial : nullptr, l == 0 ? nb : nullptr, c.stream);
    }
    CKL();
    return SGLD_OK;
}

// the same additive V-cycle in FP32 (mixed-precision preconditioner)
int vcycle_dev32(sgld_ctx *ctx, const float *r, float *z, double *partial, int *nb, cudaStream_t st = nullptr) {
    Ctx &c = ctx->c;
    if (!st) st = c.stream;
    const int L = c.L;
    const float *rf = r;
    for (int l = 1; l < L; ++l) {
        launch_restrict<float>(c.lv[l - 1], c.lv[l], rf, c.lv[l].r32, st);
        rf = c.lv[l].r32;
    }
    launch_coarse_apply_f32(c, c.lv[L - 1].r32, c.lv[L - 1].x32, st);
    for (int l = L - 2; l >= 0; --l) {
        const float *rl = (l == 0) ? r : c.lv[l].r32;
        float *xl = (l == 0) ? z : c.lv[l].x32;
        launch_prolong_smooth<float>(c.lv[l], c.lv[l + 1], c.lv[l + 1].x32, rl, c.lv[l].idiag32, (float)c.omega, xl,
                                     l == 0, l == 0 ? partial : nullptr, l == 0 ? nb : nullptr, st);
    }
    return SGLD_OK;
}

// Inner solve of the mixed-precision preconditioner: FP32 CG on K e = r32 from
// e = 0, preconditioned by the FP32 V-cycle, result in d_e32.  It is one CUDA
// graph built once per (context, kmax, eta): entry nodes (s = r, e = d = 0,
// r0 = s.s) followed by a while node whose body is one CG iteration
//   z = V s;  beta = z.s / rho;  d = z + beta d;  t = K d;
//   alpha = z.s / d.t;  e += alpha d;  s -= alpha t;  continue?
// The last kernel of the body decides on the device whether to iterate again
// (kmax iterations, or ||s|| <= max(eta, tol / (2 relres)) ||r|| first when
// eta > 0, relres being the outer solve's current relative residual), so the
// solve needs no host round trip.  d_isc[IS_TOTAL] counts the iterations run.
constexpr int IS_TOTAL = 8;

// Adds a conditional node after the current capture position of stream s
// (which must be capturing) with handle h (created by the caller on the graph
// s captures into) and returns its body graph; capture continues after it.
static int add_conditional(sgld_ctx *ctx, cudaStream_t s, cudaGraphConditionalHandle h,
                           cudaGraphConditionalNodeType type, cudaGraph_t *body) {
    cudaStreamCaptureStatus st;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    cudaGraph_t g = nullptr;
    CK(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &ndeps));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = type;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &cp));
    CK(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    *body = cp.conditional.phGraph_out[0];
    return SGLD_OK;
}

static cudaGraph_t capturing_graph(cudaStream_t s) {
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    if (cudaStreamGetCaptureInfo(s, &st, nullptr, &g, nullptr, nullptr, nullptr) != cudaSuccess) return nullptr;
    return g;
}

// Captures one inner solve: entry kernels on s (capturing), then a while node
// whose body (one CG iteration) is captured on stream sb.  *entry / *body
// receive the kernel launches of each part.
// Inner iteration caps: an inner solve with a tolerance (eta > 0) starts the
// outer solve with at most kmax iterations; after one that stops at its cap
// short of its tolerance the cap doubles, up to 16 kmax.  On a badly
// conditioned system the restarts of a short inner solve would otherwise
// multiply the outer iterations (and the inner ones with them).  A fixed
// iteration count (eta <= 0) keeps kmax.
static int inner_cap_limit(int kmax, double eta) { return eta > 0.0 ? 16 * kmax : kmax; }

static int capture_inner(sgld_ctx *ctx, cudaStream_t s, cudaStream_t sb, int kmax, double eta, int64_t *entry,
                         int64_t *body_n) {
    Ctx &c = ctx->c;
    const Level &l0 = c.lv[0];
    const int64_t nv = 3 * l0.nnode;
    cudaGraphConditionalHandle h;
    CK(cudaGraphConditionalHandleCreate(&h, capturing_graph(s), 1, cudaGraphCondAssignDefault));
    int64_t before = g_launches;
    const int nbi = launch_icg_init(c.d_r32, c.d_s32, c.d_e32, c.d_d32, nv, c.d_part2, s);
    launch_icg_scalar(0, c.d_isc, c.d_part2, nbi, s, kmax, inner_cap_limit(kmax, eta));
    launch_set_cond(h, 1u, s);   // re-arm: the loop may sit in another loop's body
    *entry = g_launches - before;
    cudaGraph_t body = nullptr;
    int rc = add_conditional(ctx, s, h, cudaGraphCondTypeWhile, &body);
    if (rc) return rc;
    before = g_launches;
    CK(cudaStreamBeginCaptureToGraph(sb, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    int nb = 0;
    vcycle_dev32(ctx, c.d_s32, c.d_z32, c.d_part2, &nb, sb);
    launch_icg_scalar(2, c.d_isc, c.d_part2, nb, sb, 0, 0);
    if (l0.runs)
        launch_icg_dupdate_runs(c.d_e32, c.d_d32, c.d_z32, l0.runs, l0.nruns, c.d_isc, sb);
    else
        launch_icg_dupdate(c.d_e32, c.d_d32, c.d_z32, nv, c.d_isc, sb);
    launch_kbyu_f32(l0, c.d_E32, c.d_d32, c.d_t32, c.d_part2, &nb, sb);
    launch_icg_scalar(1, c.d_isc, c.d_part2, nb, sb, 0, 0);
    nb = l0.runs ? launch_icg_update_runs(c.d_s32, c.d_t32, l0.runs, l0.nruns, c.d_isc, c.d_part2, sb)
                 : launch_icg_update(c.d_e32, c.d_s32, c.d_d32, c.d_t32, nv, c.d_isc, c.d_part2, sb);
    launch_icg_cond(h, c.d_isc, c.d_part2, nb, kmax, eta, c.d_scal, c.d_isc + IS_TOTAL, sb);
    CK(cudaStreamEndCapture(sb, &body));
    *body_n = g_launches - before;
    return SGLD_OK;
}

static int build_inner_graph(sgld_ctx *ctx, int kmax, double eta) {
    Ctx &c = ctx->c;
    cudaGraph_t g = nullptr;
    CK(cudaGraphCreate(&g, 0));
    const int64_t before = g_launches;
    CK(cudaStreamBeginCaptureToGraph(c.stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    int rc = capture_inner(ctx, c.stream, c.aux[0], kmax, eta, &c.inner_entry_launches, &c.inner_body_launches);
    cudaGraph_t g2 = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(c.stream, &g2);
    g_launches = before;
    if (rc) {
        cudaGraphDestroy(g);
        return rc;
    }
    CK(ec);
    const cudaError_t e = cudaGraphInstantiate(&c.inner_graph, g, 0);
    cudaGraphDestroy(g);
    CK(e);
    c.inner_graph_k = kmax;
    c.inner_graph_eta = eta;
    return SGLD_OK;
}

// The same inner solve with the loop on the host (one kernel sequence per
// iteration, a flag read back after each): selected by the environment
// variable SGLD_INNER_LOOP=host so that profilers, which do not list the
// kernels of a conditional graph body, see every launch.  Same kernels, same
// arithmetic, same stopping rule.
static int inner_run_host(sgld_ctx *ctx, int kmax, double eta) {
    Ctx &c = ctx->c;
    const Level &l0 = c.lv[0];
    const int64_t nv = 3 * l0.nnode;
    int *d_flag = c.d_iflag + 12;
    const int nbi = launch_icg_init(c.d_r32, c.d_s32, c.d_e32, c.d_d32, nv, c.d_part2, c.stream);
    launch_icg_scalar(0, c.d_isc, c.d_part2, nbi, c.stream, kmax, inner_cap_limit(kmax, eta));
    const int kl = inner_cap_limit(kmax, eta);
    for (int it = 0; it < kl; ++it) {
        int nb = 0;
        vcycle_dev32(ctx, c.d_s32, c.d_z32, c.d_part2, &nb);
        launch_icg_scalar(2, c.d_isc, c.d_part2, nb, c.stream, 0, 0);
        if (l0.runs)
            launch_icg_dupdate_runs(c.d_e32, c.d_d32, c.d_z32, l0.runs, l0.nruns, c.d_isc, c.stream);
        else
            launch_icg_dupdate(c.d_e32, c.d_d32, c.d_z32, nv, c.d_isc, c.stream);
        launch_kbyu_f32(l0, c.d_E32, c.d_d32, c.d_t32, c.d_part2, &nb, c.stream);
        launch_icg_scalar(1, c.d_isc, c.d_part2, nb, c.stream, 0, 0);
        nb = l0.runs ? launch_icg_update_runs(c.d_s32, c.d_t32, l0.runs, l0.nruns, c.d_isc, c.d_part2, c.stream)
                     : launch_icg_update(c.d_e32, c.d_s32, c.d_d32, c.d_t32, nv, c.d_isc, c.d_part2, c.stream);
        launch_icg_cond_flag(d_flag, c.d_isc, c.d_part2, nb, kmax, eta, c.d_scal, c.d_isc + IS_TOTAL, c.stream);
        int more = 0;
        CK(cudaMemcpyAsync(&more, d_flag, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        CK(cudaStreamSynchronize(c.stream));
        if (!more) break;
    }
    return SGLD_OK;
}

static bool inner_loop_on_host() {
    const char *v = getenv("SGLD_INNER_LOOP");
    return v && strcmp(v, "host") == 0;
}

// one inner solve (graph launch); launch accounting of the iterations is done
// by the caller from d_isc[IS_TOTAL]
int inner_run(sgld_ctx *ctx, int kmax, double eta) {
    Ctx &c = ctx->c;
    if (inner_loop_on_host()) return inner_run_host(ctx, kmax, eta);   // launches counted as made
    if (!c.inner_graph || c.inner_graph_k != kmax || c.inner_graph_eta != eta) {
        if (c.inner_graph) {
            cudaGraphExecDestroy(c.inner_graph);
            c.inner_graph = nullptr;
        }
        int rc = build_inner_graph(ctx, kmax, eta);
        if (rc) return rc;
    }
    CK(cudaGraphLaunch(c.inner_graph, c.stream));
    g_launches += c.inner_entry_launches;
    return SGLD_OK;
}

int check_ready(sgld_ctx *ctx) {
    if (!ctx) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    if (!ctx->c.have_fixed) return fail(ctx, SGLD_ERR_STATE, "fixed DOFs not set (sgld_set_fixed_dofs)");
    if (!ctx->c.have_E) return fail(ctx, SGLD_ERR_STATE, "element moduli not set (sgld_set_modulus)");
    return SGLD_OK;
}

int check_assembled(sgld_ctx *ctx) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (!ctx->c.assembled) return fail(ctx, SGLD_ERR_STATE, "stencil not assembled (sgld_assemble)");
    return SGLD_OK;
}

// host compact -> device full (zeroed first)
int upload_nodes(sgld_ctx *ctx, const double *h, double *d_full) {
    Ctx &c = ctx->c;
    const int64_t n = (int64_t)c.h_nodemap.size();
    CK(cudaMemsetAsync(d_full, 0, sizeof(double) * 3 * c.lv[0].nnode, c.stream));
    CK(cudaMemcpyAsync(c.d_tmp, h, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c.stream));
    launch_scatter_nodes(c.d_nodemap, n, c.d_tmp, d_full, c.stream);
    CKL();
    return SGLD_OK;
}

int download_nodes(sgld_ctx *ctx, const double *d_full, double *h) {
    Ctx &c = ctx->c;
    const int64_t n = (int64_t)c.h_nodemap.size();
    launch_gather_nodes(c.d_nodemap, n, d_full, c.d_tmp, c.stream);
    CKL();
    CK(cudaMemcpyAsync(h, c.d_tmp, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return SGLD_OK;
}

int pcg_dev(sgld_ctx *ctx, const sgld_solve_opts *o, sgld_solve_info *info);
int pcg_mixed_dev(sgld_ctx *ctx, const sgld_solve_opts *o, sgld_solve_info *info);
static int run_solve_graph(sgld_ctx *ctx, int nrhs, bool staged, const sgld_solve_opts *o, sgld_solve_info *infos);
static int ensure_block_buffers(sgld_ctx *ctx, int nrhs);

// A mixed solve counts as converged only on its true residual ||b - K x|| /
// ||b|| <= tol.  One that did not converge, met a non-finite residual or whose
// true residual stays above tol after its residual replacements is not
// trusted: the reference-form FP64 solve reruns from the same start and its
// answer is returned (info->fallback = 1).  Plain FP64 MGPCG stays the arbiter.
bool mixed_failed(const sgld_solve_info &i, double tol) {
    return !i.converged || !std::isfinite(i.true_relres) || !std::isfinite(i.relres) || i.true_relres > tol;
}

constexpr int kMaxReplacements = 3;

// Residual replacement: while the recurrence has met tol but the recomputed
// true residual is above it, restart the solve (same precision) from the
// current x, whose first residual is the recomputed b - K x.  The restarts'
// iterations and times are added to info.
int replace_residual(sgld_ctx *ctx, const sgld_solve_opts *o, sgld_solve_info *info, bool mixed) {
    for (int k = 0; k < kMaxReplacements; ++k) {
        if (!info->converged || !std::isfinite(info->relres) || !std::isfinite(info->true_relres) ||
            info->true_relres <= o->tol || info->iterations >= o->maxit)
            break;
        sgld_solve_opts o2 = *o;
        o2.use_x0 = 1;
        o2.history = nullptr;
        o2.maxit = o->maxit - info->iterations;
        sgld_solve_info r;
        memset(&r, 0, sizeof r);
        int rc = mixed ? pcg_mixed_dev(ctx, &o2, &r) : pcg_dev(ctx, &o2, &r);
        if (rc) return rc;
        info->iterations += r.iterations;
        info->inner_iterations += r.inner_iterations;
        info->seconds += r.seconds;
        info->kbyu_seconds += r.kbyu_seconds;
        info->kbyu_launches += r.kbyu_launches;
        info->precond_seconds += r.precond_seconds;
        info->relres = r.relres;
        info->true_relres = r.true_relres;
        info->converged = r.converged;
        ++info->replacements;
    }
    info->converged = info->converged && std::isfinite(info->true_relres) && info->true_relres <= o->tol;
    return SGLD_OK;
}

// test hook of sgld_inject_fault kind 2: x *= 1 + 1e-3, then the true residual
// is recomputed as the solve's own epilogue does
int apply_drift_fault(sgld_ctx *ctx, const sgld_solve_opts *o, sgld_solve_info *info) {
    Ctx &c = ctx->c;
    c.fault_drift = false;
    const Level &l0 = c.lv[0];
    const int64_t nv = 3 * l0.nnode;
    const int nbv = reduce_blocks(nv);
    launch_scale(c.d_x, 1.0 + 1e-3, nv, c.stream);
    if (o->precision == SGLD_PREC_MIXED_DF)
        launch_kbyu_df(l0, c.E, c.d_x, c.d_q, nullptr, nullptr, c.stream);
    else
        launch_kbyu_f64(l0, c.E, c.d_x, c.d_q, nullptr, nullptr, c.stream);
    launch_residual(c.d_tmp, c.d_b, c.d_q, nv, c.stream);
    launch_dot(c.d_tmp, c.d_tmp, nv, c.d_part, nbv, c.stream);
    launch_finalize_sum(c.d_part, nbv, c.d_scal + 17, c.stream);
    launch_dot(c.d_b, c.d_b, nv, c.d_part, nbv, c.stream);
    launch_finalize_sum(c.d_part, nbv, c.d_scal + 31, c.stream);
    CKL();
    double rr = 0.0, bb = 0.0;
    CK(cudaMemcpyAsync(&rr, c.d_scal + 17, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaMemcpyAsync(&bb, c.d_scal + 31, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    info->true_relres = bb > 0.0 ? sqrt(rr / bb) : 0.0;
    return SGLD_OK;
}

int solve_dev(sgld_ctx *ctx, const sgld_solve_opts *o, sgld_solve_info *info) {
    if (o->maxit < 1 || !(o->tol >= 0.0)) return fail(ctx, SGLD_ERR_ARG, "maxit must be >= 1 and tol >= 0");
    const bool mixed = o->precision == SGLD_PREC_MIXED || o->precision == SGLD_PREC_MIXED_DF;
    if (!mixed && o->precision != SGLD_PREC_FP64) return fail(ctx, SGLD_ERR_ARG, "unknown precision mode");
    sgld_solve_info local;
    if (!info) info = &local;
    memset(info, 0, sizeof *info);
    NvtxRange range(mixed ? "solve mixed" : "solve fp64");
    Ctx &c = ctx->c;
    const size_t nv = 3 * (size_t)c.lv[0].nnode;
    {   // a zero load has the solution 0 (the reference's PCG would divide by ||b|| = 0)
        const int nbv = reduce_blocks((int64_t)nv);
        launch_dot(c.d_b, c.d_b, (int64_t)nv, c.d_part, nbv, c.stream);
        launch_finalize_sum(c.d_part, nbv, c.d_scal + 31, c.stream);
        double bb = 0.0;
        CK(cudaMemcpyAsync(&bb, c.d_scal + 31, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        CK(cudaStreamSynchronize(c.stream));
        if (bb == 0.0) {
            CK(cudaMemsetAsync(c.d_x, 0, sizeof(double) * nv, c.stream));
            info->converged = 1;
            return SGLD_OK;
        }
    }
    if (!mixed) return pcg_dev(ctx, o, info);
    if (o->use_x0) {
        if (!c.d_x0) CK(dalloc(&c.d_x0, nv));
        CK(cudaMemcpyAsync(c.d_x0, c.d_x, sizeof(double) * nv, cudaMemcpyDeviceToDevice, c.stream));
    }
    int rc = pcg_mixed_dev(ctx, o, info);
    if (rc) return rc;
    if (c.fault_drift && info->converged && (rc = apply_drift_fault(ctx, o, info))) return rc;
    if ((rc = replace_residual(ctx, o, info, true))) return rc;
    if (!mixed_failed(*info, o->tol)) return SGLD_OK;
    const int replaced = info->replacements;
    if (o->use_x0)
        CK(cudaMemcpyAsync(c.d_x, c.d_x0, sizeof(double) * nv, cudaMemcpyDeviceToDevice, c.stream));
    else
        CK(cudaMemsetAsync(c.d_x, 0, sizeof(double) * nv, c.stream));
    sgld_solve_opts o64 = *o;
    o64.precision = SGLD_PREC_FP64;
    NvtxRange fb("fp64 fallback");
    memset(info, 0, sizeof *info);
    if ((rc = pcg_dev(ctx, &o64, info))) return rc;
    // the fallback answer is judged by the same rule: true residual <= tol
    if ((rc = replace_residual(ctx, &o64, info, false))) return rc;
    info->replacements += replaced;
    info->fallback = 1;
    return SGLD_OK;
}

}  // namespace

namespace sgld {
namespace {
std::mutex g_bind_mu;
bool g_kh_valid[kMaxDevices] = {};
bool g_kh_stale[kMaxDevices] = {};      // upload again even if the record matches (after a create)
double g_kh_held[kMaxDevices][KH_NNZ];   // the element matrix in each device's constants
}  // namespace

// the FP32 K*u's 45-value form even for a cubic element matrix (environment
// SGLD_KH_GENERAL=1, read once; for comparisons)
static bool kh_general_forced() {
    static const bool v = [] {
        const char *e = getenv("SGLD_KH_GENERAL");
        return e && e[0] == '1';
    }();
    return v;
}

int bind_ctx(sgld_ctx *ctx) {
    Ctx &c = ctx->c;
    int dev = -1;
    CK(cudaGetDevice(&dev));
    if (dev != c.device) CK(cudaSetDevice(c.device));
    if (!c.lv.empty()) c.lv[0].kh_cubic = !kh_general_forced() && kh_cubic(c.Kh);
    std::lock_guard<std::mutex> lock(g_bind_mu);
    const bool same = g_kh_valid[c.device] && memcmp(g_kh_held[c.device], c.Kh, sizeof c.Kh) == 0;
    if (same && !g_kh_stale[c.device]) return SGLD_OK;
    // another context's matrix is held: its queued kernels still read it.  (Rewriting
    // the same values under running kernels is harmless.)
    if (g_kh_valid[c.device] && !same) CK(cudaDeviceSynchronize());
    g_kh_valid[c.device] = false;
    upload_kh(c.Kh, c.stream);
    upload_kh_df(c.Kh, c.stream);
    CK(cudaStreamSynchronize(c.stream));
    memcpy(g_kh_held[c.device], c.Kh, sizeof c.Kh);
    g_kh_valid[c.device] = true;
    g_kh_stale[c.device] = false;
    return SGLD_OK;
}

void forget_device_tables(int dev) {
    {
        std::lock_guard<std::mutex> lock(g_bind_mu);
        g_kh_stale[dev] = true;
    }
    forget_asm_tables(dev);
    forget_noalloc_scratch(dev);
}

bool kh_bound(const Ctx &c) {
    std::lock_guard<std::mutex> lock(g_bind_mu);
    return g_kh_valid[c.device] && memcmp(g_kh_held[c.device], c.Kh, sizeof c.Kh) == 0;
}
}  // namespace sgld

// =============================================================================
extern "C" {

void sgld_default_options(sgld_options *o) {
    if (!o) return;
    o->num_levels = 0;
    o->non_dyadic = 1;
    o->poisson_ratio = 0.3;
    o->cell_size = 1.0;
    o->omega = 0.35;
    o->device = 0;
}

int sgld_reference_num_levels(int64_t num_voxels, int64_t crc) {
    // FEA_VoxelBasedDiscretization.m:168-177 (MATLAB round = half away from zero)
    auto mround = [](double x) { return (int64_t)floor(x + 0.5); };
    crc = std::min<int64_t>(crc, mround((double)mround(num_voxels / 8.0) / 8.0));
    if (crc <= 0) return -1;
    int L = 0;
    int64_t nv = num_voxels;
    while (nv >= crc) {
        ++L;
        nv = mround(nv / 8.0);
    }
    return L + 1;
}

const char *sgld_last_error(const sgld_ctx *ctx) { return ctx ? ctx->c.err.c_str() : "null context"; }

void *sgld_get_stream(const sgld_ctx *ctx) { return ctx ? (void *)ctx->c.stream : nullptr; }

int64_t sgld_kernel_launches(void) { return g_launches; }

int sgld_create(int resY, int resX, int resZ, const uint8_t *solid, const sgld_options *opts, sgld_ctx **out) {
    if (!out || !solid || resX <= 0 || resY <= 0 || resZ <= 0) return SGLD_ERR_ARG;
    *out = nullptr;
    sgld_options o;
    sgld_default_options(&o);
    if (opts) o = *opts;
    auto *ctx = new sgld_ctx;
    Ctx &c = ctx->c;
    c.nu = o.poisson_ratio;
    c.cell = o.cell_size;
    c.omega = o.omega;
    c.device = o.device;
    int L = o.num_levels;
    int nd = o.non_dyadic;
    if (nd == 1 && L >= 4)
        L -= 1;
    else
        nd = 0;
    if (L < 2) {
        int rc = fail(ctx, SGLD_ERR_ARG, "at least two multigrid levels are required");
        *out = ctx;
        return rc;
    }
    c.L = L;
    c.non_dyadic = nd;
    c.lv.resize(L);
    int ny = resY, nx = resX, nz = resZ;
    for (int l = 0; l < L; ++l) {
        const int s = (l == 0) ? 1 : ((l == 1 && nd) ? 4 : 2);
        if (l > 0) {
            if (ny % s || nx % s || nz % s) {
                int rc = fail(ctx, SGLD_ERR_ARG, "grid resolution is not divisible by the coarsening factors");
                *out = ctx;
                return rc;
            }
            ny /= s;
            nx /= s;
            nz /= s;
        }
        Level &lv = c.lv[l];
        lv.nx = nx;
        lv.ny = ny;
        lv.nz = nz;
        lv.span = s;
        lv.nel = (int64_t)nx * ny * nz;
        lv.nnode = (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    }
    *out = ctx;
    if (c.device < 0 || c.device >= kMaxDevices) return fail(ctx, SGLD_ERR_ARG, "device ordinal out of range");
    if (cudaSetDevice(c.device) != cudaSuccess) return fail(ctx, SGLD_ERR_CUDA, "cudaSetDevice failed");
    forget_device_tables(c.device);   // the device may have been reset since the last create
    CK(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    for (auto &a : c.aux) CK(cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking));
    // element / node activity per level (host)
    ctx->nodemaps.resize(L);
    ctx->elemaps.resize(L);
    for (int l = 0; l < L; ++l) {
        Level &lv = c.lv[l];
        lv.h_eact.assign(lv.nel, 0);
        if (l == 0) {
            for (int64_t e = 0; e < lv.nel; ++e) lv.h_eact[e] = solid[e] ? 1 : 0;
        } else {
            const Level &f = c.lv[l - 1];
            const int s = lv.span;
            for (int64_t fz = 0; fz < f.nz; ++fz)
                for (int64_t fx = 0; fx < f.nx; ++fx)
                    for (int64_t fy = 0; fy < f.ny; ++fy)
                        if (f.h_eact[fy + f.ny * (fx + f.nx * fz)])
                            lv.h_eact[(fy / s) + lv.ny * ((fx / s) + lv.nx * (fz / s))] = 1;
        }
        lv.h_nflag.assign(lv.nnode, 0);
        const int64_t NY = lv.ny + 1, NX = lv.nx + 1;
        for (int64_t ez = 0; ez < lv.nz; ++ez)
            for (int64_t ex = 0; ex < lv.nx; ++ex)
                for (int64_t ey = 0; ey < lv.ny; ++ey)
                    if (lv.h_eact[ey + lv.ny * (ex + lv.nx * ez)])
                        for (int j = 0; j < 8; ++j)
                            lv.h_nflag[(ey + kCdy[j]) + NY * ((ex + kCdx[j]) + NX * (ez + kCdz[j]))] = NF_ACTIVE;
        auto &nm = ctx->nodemaps[l];
        auto &em = ctx->elemaps[l];
        for (int64_t n = 0; n < lv.nnode; ++n)
            if (lv.h_nflag[n]) nm.push_back(n);
        for (int64_t e = 0; e < lv.nel; ++e)
            if (lv.h_eact[e]) em.push_back(e);
        lv.nel_active = (int64_t)em.size();
        lv.nnode_active = (int64_t)nm.size();
        CK(dalloc(&lv.eact, lv.nel));
        CK(dalloc(&lv.nflag, lv.nnode));
        CK(cudaMemcpy(lv.eact, lv.h_eact.data(), lv.nel, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(lv.nflag, lv.h_nflag.data(), lv.nnode, cudaMemcpyHostToDevice));
        if (l < L - 1) {
            CK(dalloc(&lv.diag, 3 * lv.nnode));
            CK(dalloc(&lv.idiag, 3 * lv.nnode));
            CK(dalloc(&lv.idiag32, 3 * lv.nnode));
        }
        if (l > 0) {
            if (!(l == 1 && skip_level2_ks(c))) CK(dalloc(&lv.Ks, 576 * (size_t)lv.nel));
            CK(dalloc(&lv.r, 3 * lv.nnode));
            CK(dalloc(&lv.x, 3 * lv.nnode));
            CK(dalloc(&lv.r32, 3 * lv.nnode));
            CK(dalloc(&lv.x32, 3 * lv.nnode));
            // the FP32 prolongation skips empty cells and the FP32 restriction inactive
            // nodes: both rely on zeros at inactive nodes
            CK(cudaMemset(lv.x32, 0, sizeof(float) * 3 * lv.nnode));
            CK(cudaMemset(lv.r32, 0, sizeof(float) * 3 * lv.nnode));
        }
    }
    if (c.lv[0].nel_active == 0) return fail(ctx, SGLD_ERR_ARG, "the voxel grid has no solid voxel");
    if (int rc = build_active_runs(ctx)) return rc;
    c.h_nodemap = ctx->nodemaps[0];
    c.h_elemap = ctx->elemaps[0];
    CK(dalloc(&c.d_nodemap, c.h_nodemap.size()));
    CK(dalloc(&c.d_elemap, c.h_elemap.size()));
    CK(cudaMemcpy(c.d_nodemap, c.h_nodemap.data(), c.h_nodemap.size() * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c.d_elemap, c.h_elemap.data(), c.h_elemap.size() * 8, cudaMemcpyHostToDevice));
    const Level &l0 = c.lv[0];
    const size_t nv = 3 * (size_t)l0.nnode;
    CK(dalloc(&c.E, l0.nel));
    CK(cudaMemset(c.E, 0, sizeof(double) * l0.nel));
    CK(dalloc(&c.d_E32, l0.nel));
    for (double **p : {&c.d_b, &c.d_x, &c.d_r, &c.d_z, &c.d_p, &c.d_q, &c.d_tmp}) CK(dalloc(p, nv));
    CK(dalloc(&c.d_r32, nv));
    CK(dalloc(&c.d_z32, nv));
    CK(cudaMemset(c.d_z32, 0, sizeof(float) * nv));   // see lv.x32
    for (float **p : {&c.d_e32, &c.d_s32, &c.d_d32, &c.d_t32}) CK(dalloc(p, nv));
    // the FP32 K*u (whose output is always d_t32) never writes inactive nodes
    CK(cudaMemset(c.d_t32, 0, sizeof(float) * nv));
    CK(dalloc(&c.d_isc, 16));
    init_kernel_attributes();
    init_kbyu_df_attributes();
    // partial-sum slots: the largest grid of any kernel that writes per-CTA partials
    // (prolongation: ceil(NY*NX/256) CTAs per node plane)
    c.npart = (int)std::max<int64_t>({(int64_t)152 * 8, (l0.nel + 255) / 256 + 1,
                                      (int64_t)(((l0.ny + 1) * (l0.nx + 1) + 255) / 256) * (l0.nz + 1),
                                      (int64_t)((l0.ny + 31) / 31 + 1) * ((l0.nx + 7) / 7 + 1) * ((l0.nz + 16) / 16 + 1)});
    CK(dalloc(&c.d_part, c.npart));
    CK(dalloc(&c.d_part2, c.npart));
    CK(dalloc(&c.d_scal, 64));
    CK(dalloc(&c.d_iflag, 64));
    CK(cudaMemset(c.d_iflag, 0, 64 * sizeof(int)));
    element_stiffness(c.nu, c.cell, c.Ke);
    std::string why;
    if (!hadamard_blocks(c.Ke, c.Kh, why)) return fail(ctx, SGLD_ERR_ARG, why);
    return setup_templates(ctx);
}

void sgld_destroy(sgld_ctx *ctx) {
    if (!ctx) return;
    Ctx &c = ctx->c;
    int dev = -1;   // the buffers and streams belong to the context's device
    if (c.device >= 0 && c.device < kMaxDevices && cudaGetDevice(&dev) == cudaSuccess && dev != c.device)
        cudaSetDevice(c.device);
    for (Level &l : c.lv) {
        for (void *p : {(void *)l.eact, (void *)l.nflag, (void *)l.diag, (void *)l.idiag, (void *)l.idiag32, (void *)l.Ks, (void *)l.r,
                        (void *)l.x, (void *)l.r32, (void *)l.x32, (void *)l.tiles16, (void *)l.tiles_f32,
                        (void *)l.runs, (void *)l.kerr})
            if (p) cudaFree(p);
    }
    for (void *p : {(void *)c.d_nodemap, (void *)c.d_elemap, (void *)c.E, (void *)c.d_E32, (void *)c.d_b,
                    (void *)c.d_x, (void *)c.d_r, (void *)c.d_z, (void *)c.d_p, (void *)c.d_q, (void *)c.d_tmp,
                    (void *)c.d_r32, (void *)c.d_z32, (void *)c.d_part, (void *)c.d_scal, (void *)c.d_iflag,
                    (void *)c.d_Ac, (void *)c.d_Ainv, (void *)c.d_Ainv32, (void *)c.d_cpart, (void *)c.d_cfree,
                    (void *)c.d_H, (void *)ctx->d_s6, (void *)ctx->d_vmn, (void *)ctx->d_vme, (void *)c.d_e32,
                    (void *)c.d_s32, (void *)c.d_d32, (void *)c.d_t32, (void *)c.d_isc, (void *)c.d_part2, (void *)c.d_LB,
                    (void *)c.d_cy})
        if (p) cudaFree(p);
    if (c.inner_graph) cudaGraphExecDestroy(c.inner_graph);
    if (c.factor_graph) cudaGraphExecDestroy(c.factor_graph);
    if (c.stream) cudaStreamDestroy(c.stream);
    for (auto &a : c.aux)
        if (a) cudaStreamDestroy(a);
    if (c.solve_graph) cudaGraphExecDestroy(c.solve_graph);
    learned_free(c.lws);
    for (void *p : {(void *)c.d_x0, (void *)c.d_blk, (void *)c.d_binfo, (void *)c.t_x, (void *)c.t_xp, (void *)c.t_hs,
                    (void *)c.t_ce, (void *)c.t_dcs, (void *)c.t_dvs, (void *)c.t_dc, (void *)c.t_dv, (void *)c.t_q,
                    (void *)c.t_tmp, (void *)c.t_st, (void *)c.t_pde, (void *)c.t_fw, (void *)c.t_kp})
        if (p) cudaFree(p);
    delete ctx;
}

int sgld_num_levels(const sgld_ctx *ctx) { return ctx ? ctx->c.L : -1; }

int sgld_inject_fault(sgld_ctx *ctx, int kind) {
    if (!ctx || kind < 0 || kind > 2) return SGLD_ERR_ARG;
    if (kind == 0) return SGLD_OK;
    Ctx &c = ctx->c;
    if (!c.assembled || c.h_elemap.empty()) return fail(ctx, SGLD_ERR_STATE, "inject after sgld_assemble");
    if (kind == 2) {
        c.fault_drift = true;
        return SGLD_OK;
    }
    const float nan = std::numeric_limits<float>::quiet_NaN();
    CK(cudaMemcpy(c.d_E32 + c.h_elemap[c.h_elemap.size() / 2], &nan, sizeof(float), cudaMemcpyHostToDevice));
    return SGLD_OK;
}

int sgld_kbyu_tile(const sgld_ctx *ctx, int *tile_x, int *z_chunk) {
    if (!ctx || ctx->c.L < 1) return SGLD_ERR_ARG;
    const Level &l0 = ctx->c.lv[0];
    if (tile_x) *tile_x = kbyu_f32_tx(l0);
    if (z_chunk) *z_chunk = kbyu_f32_cta_layers(l0);
    return SGLD_OK;
}

int sgld_level_info(const sgld_ctx *ctx, int level, int res[3], int *span, int64_t *ne, int64_t *nn) {
    if (!ctx || level < 1 || level > ctx->c.L) return SGLD_ERR_ARG;
    const Level &l = ctx->c.lv[level - 1];
    if (res) {
        res[0] = l.ny;
        res[1] = l.nx;
        res[2] = l.nz;
    }
    if (span) *span = l.span;
    if (ne) *ne = l.nel_active;
    if (nn) *nn = l.nnode_active;
    return SGLD_OK;
}

int sgld_node_map(const sgld_ctx *ctx, int level, int64_t *map) {
    if (!ctx || !map || level < 1 || level > ctx->c.L) return SGLD_ERR_ARG;
    const auto &m = ctx->nodemaps[level - 1];
    for (size_t i = 0; i < m.size(); ++i) map[i] = m[i] + 1;
    return SGLD_OK;
}

int sgld_element_map(const sgld_ctx *ctx, int level, int64_t *map) {
    if (!ctx || !map || level < 1 || level > ctx->c.L) return SGLD_ERR_ARG;
    const auto &m = ctx->elemaps[level - 1];
    for (size_t i = 0; i < m.size(); ++i) map[i] = m[i] + 1;
    return SGLD_OK;
}

int sgld_get_ke(const sgld_ctx *ctx, double *Ke) {
    if (!ctx || !Ke) return SGLD_ERR_ARG;
    memcpy(Ke, ctx->c.Ke, sizeof(double) * 576);
    return SGLD_OK;
}

int sgld_set_ke(sgld_ctx *ctx, const double *Ke) {
    if (!ctx || !Ke) return SGLD_ERR_ARG;
    double Kh[KH_NNZ];
    std::string why;
    if (!hadamard_blocks(Ke, Kh, why)) return fail(ctx, SGLD_ERR_ARG, why);
    memcpy(ctx->c.Ke, Ke, sizeof(double) * 576);
    memcpy(ctx->c.Kh, Kh, sizeof Kh);
    ctx->c.assembled = false;
    // the captured solve graphs hold the FP32 K*u form chosen for the old matrix (kh_cubic)
    Ctx &c = ctx->c;
    if (c.solve_graph) {
        cudaGraphExecDestroy(c.solve_graph);
        c.solve_graph = nullptr;
    }
    if (c.inner_graph) {
        cudaGraphExecDestroy(c.inner_graph);
        c.inner_graph = nullptr;
    }
    return setup_templates(ctx);
}

int sgld_set_fixed_dofs(sgld_ctx *ctx, const uint8_t *fixed) {
    if (!ctx || !fixed) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    Ctx &c = ctx->c;
    Level &l0 = c.lv[0];
    for (int64_t n = 0; n < l0.nnode; ++n) l0.h_nflag[n] &= NF_ACTIVE;
    for (size_t i = 0; i < c.h_nodemap.size(); ++i)
        for (int d = 0; d < 3; ++d)
            if (fixed[3 * i + d]) l0.h_nflag[c.h_nodemap[i]] |= (uint8_t)(NF_FIXX << d);
    CK(cudaMemcpy(l0.nflag, l0.h_nflag.data(), l0.nnode, cudaMemcpyHostToDevice));
    // coarse masks: restrict the fixed indicator level by level (FEA_SetupVoxelBased.m:13-26)
    launch_fixed_indicator(l0, c.d_tmp, c.stream);
    const double *v = c.d_tmp;
    for (int l = 1; l < c.L; ++l) {
        launch_restrict<double>(c.lv[l - 1], c.lv[l], v, c.lv[l].r, c.stream);
        launch_mark_fixed(c.lv[l], c.lv[l].r, c.stream);
        v = c.lv[l].r;
    }
    CKL();
    for (int l = 1; l < c.L; ++l)
        CK(cudaMemcpyAsync(c.lv[l].h_nflag.data(), c.lv[l].nflag, c.lv[l].nnode, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    // coarsest free DOFs in a bandwidth-reducing order: slowest axis = longest
    const Level &lc = c.lv[c.L - 1];
    const int64_t NY = lc.ny + 1, NX = lc.nx + 1, NZ = lc.nz + 1;
    int ax[3] = {0, 1, 2};                    // 0 = y, 1 = x, 2 = z
    const int64_t dimn[3] = {NY, NX, NZ};
    std::sort(ax, ax + 3, [&](int a, int b) { return dimn[a] < dimn[b]; });   // fastest first
    std::vector<std::pair<int64_t, int>> order;   // (key, dof)
    for (int64_t n = 0; n < lc.nnode; ++n) {
        const uint8_t f = lc.h_nflag[n];
        if (!(f & NF_ACTIVE)) continue;
        const int64_t co[3] = {n % NY, (n / NY) % NX, n / (NY * NX)};
        const int64_t key = co[ax[0]] + dimn[ax[0]] * (co[ax[1]] + dimn[ax[1]] * co[ax[2]]);
        for (int d = 0; d < 3; ++d)
            if (!(f & (NF_FIXX << d))) order.push_back({3 * key + d, (int)(3 * n + d)});
    }
    std::sort(order.begin(), order.end());
    const int ncf = (int)order.size();
    std::vector<int> rows(ncf), pos(3 * lc.nnode, -1);
    for (int i = 0; i < ncf; ++i) {
        rows[i] = order[i].second;
        pos[rows[i]] = i;
    }
    // half bandwidth over the element connectivity
    int band = 0;
    for (int64_t ez = 0; ez < lc.nz; ++ez)
        for (int64_t ex = 0; ex < lc.nx; ++ex)
            for (int64_t ey = 0; ey < lc.ny; ++ey) {
                if (!lc.h_eact[ey + lc.ny * (ex + lc.nx * ez)]) continue;
                int lo = ncf, hi = -1;
                for (int j = 0; j < 8; ++j) {
                    const int64_t m = (ey + kCdy[j]) + NY * ((ex + kCdx[j]) + NX * (ez + kCdz[j]));
                    for (int d = 0; d < 3; ++d) {
                        const int p = pos[3 * m + d];
                        if (p >= 0) {
                            lo = std::min(lo, p);
                            hi = std::max(hi, p);
                        }
                    }
                }
                if (hi >= lo) band = std::max(band, hi - lo);
            }
    ctx->h_rows = rows;
    if (ncf != c.ncf || band != c.cband || !c.d_cfree) {
        for (void *p : {(void *)c.d_Ac, (void *)c.d_Ainv, (void *)c.d_Ainv32, (void *)c.d_cpart, (void *)c.d_cfree,
                        (void *)c.d_LB, (void *)c.d_cy})
            if (p) cudaFree(p);
        c.d_Ac = c.d_Ainv = c.d_LB = c.d_cy = c.d_cpart = nullptr;
        c.d_Ainv32 = nullptr;
        c.d_cfree = nullptr;
        c.ncf = ncf;
        c.cband = band;
        CK(dalloc(&c.d_Ac, (size_t)ncf * ncf));
        CK(dalloc(&c.d_Ainv, (size_t)ncf * ncf));
        CK(dalloc(&c.d_Ainv32, (size_t)ncf * ncf));
        CK(dalloc(&c.d_cpart, (size_t)CSPLIT * ncf));
        // band + 1/diag + inverses of the 32 x 32 diagonal blocks, as float pairs
        CK(dalloc(&c.d_LB, (size_t)ncf * (band + 1) + ncf + (size_t)((ncf + 31) / 32) * 1024));
        CK(dalloc(&c.d_cy, 2 * (size_t)ncf));
        CK(dalloc(&c.d_cfree, (size_t)ncf + 3 * lc.nnode));
        if (c.solve_graph) {
            cudaGraphExecDestroy(c.solve_graph);
            c.solve_graph = nullptr;
        }
        if (c.inner_graph) {   // the captured graphs hold the old coarse buffers
            cudaGraphExecDestroy(c.inner_graph);
            c.inner_graph = nullptr;
        }
        if (c.factor_graph) {
            cudaGraphExecDestroy(c.factor_graph);
            c.factor_graph = nullptr;
        }
    }
    CK(cudaMemcpy(c.d_cfree, rows.data(), sizeof(int) * ncf, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c.d_cfree + ncf, pos.data(), sizeof(int) * 3 * lc.nnode, cudaMemcpyHostToDevice));
    c.have_fixed = true;
    c.assembled = false;
    return SGLD_OK;
}

int sgld_get_free_dofs(const sgld_ctx *ctx, int level, uint8_t *free_mask) {
    if (!ctx || !free_mask || level < 1 || level > ctx->c.L) return SGLD_ERR_ARG;
    const Level &l = ctx->c.lv[level - 1];
    const auto &m = ctx->nodemaps[level - 1];
    for (size_t i = 0; i < m.size(); ++i)
        for (int d = 0; d < 3; ++d) free_mask[3 * i + d] = (l.h_nflag[m[i]] & (NF_FIXX << d)) ? 0 : 1;
    return SGLD_OK;
}

int sgld_set_modulus_device(sgld_ctx *ctx, const double *d_E) {
    if (!ctx || !d_E) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    Ctx &c = ctx->c;
    CK(cudaMemsetAsync(c.E, 0, sizeof(double) * c.lv[0].nel, c.stream));
    launch_scatter_elems(c.d_elemap, (int64_t)c.h_elemap.size(), d_E, c.E, c.stream);
    CKL();
    CK(cudaStreamSynchronize(c.stream));
    c.have_E = true;
    c.assembled = false;
    return SGLD_OK;
}

int sgld_set_modulus(sgld_ctx *ctx, const double *E) {
    if (!ctx || !E) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    Ctx &c = ctx->c;
    CK(cudaMemcpyAsync(c.d_tmp, E, sizeof(double) * c.h_elemap.size(), cudaMemcpyHostToDevice, c.stream));
    return sgld_set_modulus_device(ctx, c.d_tmp);
}

// Autotuner of the FP32 K*u's tile: x width (8 or 16 elements) times z-chunk
// (node layers per CTA).  Times each candidate with CUDA events on the
// context's stream (3 launches after a warm-up) and keeps the fastest in
// lv[0].kx_tx / kx_zc.  Runs once per context, at the first assembly (never
// during a graph capture); SGLD_AUTOTUNE=0 keeps the default tile.  Width
// and chunk trade halo work (one extra element column / layer per CTA)
// against the number of CTAs in flight.
static int tune_kbyu_f32(sgld_ctx *ctx) {
    Ctx &c = ctx->c;
    Level &l0 = c.lv[0];
    if (c.kbyu_tuned) return SGLD_OK;
    c.kbyu_tuned = true;
    const char *v = getenv("SGLD_AUTOTUNE");
    if (v && strcmp(v, "0") == 0) {
        if (update_kbyu_tiles(l0, c.stream)) return fail(ctx, SGLD_ERR_CUDA, "K*u tile maps");
        return SGLD_OK;
    }
    const int NZ = l0.nz + 1;
    std::vector<int> cand;
    for (int zc : {4, 6, 8, 12, 16, 24})   // node layers per stream, two streams per CTA
        if (2 * zc <= NZ + 1) cand.push_back(zc);
    cand.push_back(0);   // the default rule
    CK(cudaMemsetAsync(c.d_r32, 0, sizeof(float) * 3 * (size_t)l0.nnode, c.stream));
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    float best = 1e30f;
    int best_zc = 0, best_tx = 0;
    for (int tx : {16, 8})
        for (int zc : cand) {
            l0.kx_tx = tx;
            l0.kx_zc = zc;
            if (update_kbyu_tiles(l0, c.stream)) return fail(ctx, SGLD_ERR_CUDA, "K*u tile maps");
            if (launch_kbyu_f32(l0, c.d_E32, c.d_r32, c.d_t32, nullptr, nullptr, c.stream))
                return fail(ctx, SGLD_ERR_CUDA, "FP32 K*u: the vector's tensor map could not be made");
            CK(cudaEventRecord(a, c.stream));
            for (int r = 0; r < 3; ++r) launch_kbyu_f32(l0, c.d_E32, c.d_r32, c.d_t32, nullptr, nullptr, c.stream);
            CK(cudaEventRecord(b, c.stream));
            CK(cudaEventSynchronize(b));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, a, b);
            if (ms < best) {
                best = ms;
                best_zc = zc;
                best_tx = tx;
            }
        }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    l0.kx_tx = best_tx;
    l0.kx_zc = best_zc;
    if (update_kbyu_tiles(l0, c.stream)) return fail(ctx, SGLD_ERR_CUDA, "K*u tile maps");
    CKL();
    return SGLD_OK;
}

int sgld_assemble(sgld_ctx *ctx) {
    NvtxRange range("sgld_assemble");
    int rc = check_ready(ctx);
    if (rc) return rc;
    Ctx &c = ctx->c;
    const int L = c.L;
    launch_diag_finest(c.lv[0], c.E, c.Ke, c.lv[0].diag, c.stream);
    const bool skip2 = skip_level2_ks(c);
    for (int l = 1; l < L; ++l) {
        if (l == 1 && skip2) {
            launch_diag_templates(c.lv[1], c.E, templates(c, 2), c.lv[1].diag, c.stream);
            continue;
        }
        if (l == 1)
            launch_asm_templates(c.lv[1], c.lv[1].span, c.E, templates(c, c.lv[1].span), c.lv[1].Ks, c.stream);
        else if (l == 2 && skip2)
            launch_asm_templates(c.lv[2], 4, c.E, templates(c, 4), c.lv[2].Ks, c.stream);
        else
            launch_asm_coarse(c.lv[l], c.lv[l - 1], c.lv[l].Ks, c.stream);
        if (l < L - 1) launch_diag_from_Ks(c.lv[l], c.lv[l].diag, c.stream);
    }
    CKL();
    launch_coarse_dense(c.lv[L - 1], c.ncf, c.d_cfree, c.d_Ac, c.stream);
    CKL();
    const int info = coarse_factor_invert(c);
    CKL();
    CK(cudaStreamSynchronize(c.stream));
    if (info == -2) return fail(ctx, SGLD_ERR_ARG, "coarsest-level band too wide; use more multigrid levels");
    if (info == -1) return fail(ctx, SGLD_ERR_CUDA, "coarsest-level factorization could not be captured or launched");
    if (info != 0)
        return fail(ctx, SGLD_ERR_NUMERIC,
                    "coarsest-level matrix is not positive definite (pivot " + std::to_string(info) + ")");
    for (int l = 0; l < L - 1; ++l) launch_inverse_diag(c.lv[l], c.stream);
    launch_cast_f32(c.E, c.d_E32, c.lv[0].nel, c.stream);
    CKL();
    CK(cudaStreamSynchronize(c.stream));
    c.assembled = true;
    if (!c.kbyu_tuned) {
        const int rct = tune_kbyu_f32(ctx);
        if (rct) return rct;
    }
    return SGLD_OK;
}

int sgld_get_diag(const sgld_ctx *cctx, int level, double *diag) {
    auto *ctx = const_cast<sgld_ctx *>(cctx);
    if (!ctx || !diag || level < 1 || level >= ctx->c.L) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    const Level &l = ctx->c.lv[level - 1];
    std::vector<double> full(3 * l.nnode);
    CK(cudaMemcpy(full.data(), l.diag, sizeof(double) * full.size(), cudaMemcpyDeviceToHost));
    const auto &m = ctx->nodemaps[level - 1];
    for (size_t i = 0; i < m.size(); ++i)
        for (int d = 0; d < 3; ++d) diag[3 * i + d] = full[3 * m[i] + d];
    return SGLD_OK;
}

int sgld_get_ks(const sgld_ctx *cctx, int level, double *Ks) {
    auto *ctx = const_cast<sgld_ctx *>(cctx);
    if (!ctx || !Ks || level < 2 || level > ctx->c.L) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    Ctx &c = ctx->c;
    if (!c.assembled) return fail(ctx, SGLD_ERR_STATE, "stencil not assembled (sgld_assemble)");
    Level &l = c.lv[level - 1];
    if (!l.Ks) {   // level 2 of a dyadic hierarchy: formed on request only
        CK(dalloc(&l.Ks, 576 * (size_t)l.nel));
        launch_asm_templates(l, 2, c.E, templates(c, 2), l.Ks, c.stream);
        CKL();
        CK(cudaStreamSynchronize(c.stream));
    }
    const auto &m = ctx->elemaps[level - 1];
    for (size_t i = 0; i < m.size(); ++i)
        CK(cudaMemcpy(Ks + 576 * i, l.Ks + 576 * m[i], sizeof(double) * 576, cudaMemcpyDeviceToHost));
    return SGLD_OK;
}

int sgld_kbyu_device(sgld_ctx *ctx, const double *d_u, double *d_y) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    Ctx &c = ctx->c;
    const int64_t n = (int64_t)c.h_nodemap.size();
    CK(cudaMemsetAsync(c.d_p, 0, sizeof(double) * 3 * c.lv[0].nnode, c.stream));
    launch_scatter_nodes(c.d_nodemap, n, d_u, c.d_p, c.stream);
    launch_kbyu_f64(c.lv[0], c.E, c.d_p, c.d_q, nullptr, nullptr, c.stream);
    launch_gather_nodes(c.d_nodemap, n, c.d_q, d_y, c.stream);
    CKL();
    CK(cudaStreamSynchronize(c.stream));
    return SGLD_OK;
}

int sgld_kbyu(sgld_ctx *ctx, const double *u, double *y) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (!u || !y) return fail(ctx, SGLD_ERR_ARG, "null vector");
    Ctx &c = ctx->c;
    if ((rc = upload_nodes(ctx, u, c.d_p))) return rc;
    launch_kbyu_f64(c.lv[0], c.E, c.d_p, c.d_q, nullptr, nullptr, c.stream);
    CKL();
    return download_nodes(ctx, c.d_q, y);
}

int sgld_kbyu_df(sgld_ctx *ctx, const double *u, double *y) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (!u || !y) return fail(ctx, SGLD_ERR_ARG, "null vector");
    Ctx &c = ctx->c;
    if ((rc = upload_nodes(ctx, u, c.d_p))) return rc;
    launch_kbyu_df(c.lv[0], c.E, c.d_p, c.d_q, nullptr, nullptr, c.stream);
    CKL();
    return download_nodes(ctx, c.d_q, y);
}

static int level_vec_to_dev(sgld_ctx *ctx, int l, const double *h, double *d_full) {
    Ctx &c = ctx->c;
    const Level &lv = c.lv[l];
    std::vector<double> full(3 * lv.nnode, 0.0);
    const auto &m = ctx->nodemaps[l];
    for (size_t i = 0; i < m.size(); ++i)
        for (int d = 0; d < 3; ++d) full[3 * m[i] + d] = h[3 * i + d];
    CK(cudaMemcpy(d_full, full.data(), sizeof(double) * full.size(), cudaMemcpyHostToDevice));
    return SGLD_OK;
}

static int level_vec_to_host(sgld_ctx *ctx, int l, const double *d_full, double *h) {
    Ctx &c = ctx->c;
    const Level &lv = c.lv[l];
    CK(cudaStreamSynchronize(c.stream));
    std::vector<double> full(3 * lv.nnode);
    CK(cudaMemcpy(full.data(), d_full, sizeof(double) * full.size(), cudaMemcpyDeviceToHost));
    const auto &m = ctx->nodemaps[l];
    for (size_t i = 0; i < m.size(); ++i)
        for (int d = 0; d < 3; ++d) h[3 * i + d] = full[3 * m[i] + d];
    return SGLD_OK;
}

int sgld_restrict(sgld_ctx *ctx, int ii, const double *rf, double *rc_out) {
    if (!ctx || !rf || !rc_out || ii < 2 || ii > ctx->c.L) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    Ctx &c = ctx->c;
    const int l = ii - 1;
    int rc;
    double *fin = (l - 1 == 0) ? c.d_r : c.lv[l - 1].x;
    if ((rc = level_vec_to_dev(ctx, l - 1, rf, fin))) return rc;
    launch_restrict<double>(c.lv[l - 1], c.lv[l], fin, c.lv[l].r, c.stream);
    CKL();
    return level_vec_to_host(ctx, l, c.lv[l].r, rc_out);
}

int sgld_restrict_prec(sgld_ctx *ctx, int ii, const double *rf, double *rc_out, int precision) {
    if (precision == SGLD_PREC_FP64) return sgld_restrict(ctx, ii, rf, rc_out);
    if (precision != SGLD_PREC_MIXED && precision != SGLD_PREC_MIXED_DF) {
        if (ctx) ctx->c.err = "unknown precision mode";
        return SGLD_ERR_ARG;
    }
    if (!ctx || !rf || !rc_out || ii < 2 || ii > ctx->c.L) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    Ctx &c = ctx->c;
    const int l = ii - 1;
    int rc;
    // the fine vector in FP64 (zeros at inactive nodes), narrowed into the FP32 vector the
    // V-cycle restricts from at that level
    double *fin = (l - 1 == 0) ? c.d_r : c.lv[l - 1].x;
    if ((rc = level_vec_to_dev(ctx, l - 1, rf, fin))) return rc;
    float *fin32 = (l - 1 == 0) ? c.d_r32 : c.lv[l - 1].r32;
    launch_narrow(fin, fin32, 3 * c.lv[l - 1].nnode, c.stream);
    launch_restrict<float>(c.lv[l - 1], c.lv[l], fin32, c.lv[l].r32, c.stream);
    launch_widen(c.lv[l].r32, c.lv[l].r, 3 * c.lv[l].nnode, c.stream);
    CKL();
    return level_vec_to_host(ctx, l, c.lv[l].r, rc_out);
}

int sgld_interpolate(sgld_ctx *ctx, int ii, const double *xc, double *xf) {
    if (!ctx || !xc || !xf || ii < 2 || ii > ctx->c.L) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    Ctx &c = ctx->c;
    const int l = ii - 1;
    int rc;
    if ((rc = level_vec_to_dev(ctx, l, xc, c.lv[l].x))) return rc;
    // P x with t = 0: zero residual, unit diagonal
    const Level &f = c.lv[l - 1];
    double *rzero = c.d_tmp, *ones = c.d_q, *out = c.d_z;
    CK(cudaMemsetAsync(rzero, 0, sizeof(double) * 3 * f.nnode, c.stream));
    std::vector<double> one(3 * f.nnode, 1.0);
    CK(cudaMemcpy(ones, one.data(), sizeof(double) * one.size(), cudaMemcpyHostToDevice));
    launch_prolong_smooth<double>(f, c.lv[l], c.lv[l].x, rzero, ones, 0.0, out, false, nullptr, nullptr, c.stream);
    CKL();
    return level_vec_to_host(ctx, l - 1, out, xf);
}

int sgld_vcycle(sgld_ctx *ctx, const double *r, double *z) {
    int rc = check_assembled(ctx);
    if (rc) return rc;
    if (!r || !z) return fail(ctx, SGLD_ERR_ARG, "null vector");
    Ctx &c = ctx->c;
    if ((rc = upload_nodes(ctx, r, c.d_r))) return rc;
    if ((rc = vcycle_dev(ctx, c.d_r, c.d_z, nullptr, nullptr))) return rc;
    return download_nodes(ctx, c.d_z, z);
}

int sgld_pcg_device(sgld_ctx *ctx, const double *d_b, double *d_x, const sgld_solve_opts *o, sgld_solve_info *info) {
    int rc = check_assembled(ctx);
    if (rc) return rc;
    if (!d_b || !d_x || !o) return fail(ctx, SGLD_ERR_ARG, "null argument");
    Ctx &c = ctx->c;
    const int64_t n = (int64_t)c.h_nodemap.size();
    const size_t nv = 3 * (size_t)c.lv[0].nnode;
    CK(cudaMemsetAsync(c.d_b, 0, sizeof(double) * nv, c.stream));
    CK(cudaMemsetAsync(c.d_x, 0, sizeof(double) * nv, c.stream));
    launch_scatter_nodes(c.d_nodemap, n, d_b, c.d_b, c.stream);
    if (o->use_x0) launch_scatter_nodes(c.d_nodemap, n, d_x, c.d_x, c.stream);
    CKL();
    if ((rc = solve_dev(ctx, o, info))) return rc;
    launch_gather_nodes(c.d_nodemap, n, c.d_x, d_x, c.stream);
    CKL();
    CK(cudaStreamSynchronize(c.stream));
    return SGLD_OK;
}

int sgld_pcg(sgld_ctx *ctx, const double *b, double *x, const sgld_solve_opts *o, sgld_solve_info *info) {
    int rc = check_assembled(ctx);
    if (rc) return rc;
    if (!b || !x || !o) return fail(ctx, SGLD_ERR_ARG, "null argument");
    Ctx &c = ctx->c;
    if ((rc = upload_nodes(ctx, b, c.d_b))) return rc;
    if (o->use_x0) {
        if ((rc = upload_nodes(ctx, x, c.d_x))) return rc;
    } else {
        CK(cudaMemsetAsync(c.d_x, 0, sizeof(double) * 3 * c.lv[0].nnode, c.stream));
    }
    if ((rc = solve_dev(ctx, o, info))) return rc;
    return download_nodes(ctx, c.d_x, x);
}

int sgld_solve_block(sgld_ctx *ctx, int nrhs, const double *F, double *U, const sgld_solve_opts *o,
                     sgld_solve_info *info) {
    int rc = check_assembled(ctx);
    if (rc) return rc;
    if (nrhs < 0 || (nrhs > 0 && (!F || !U || !o))) return fail(ctx, SGLD_ERR_ARG, "bad block arguments");
    const int64_t nd = 3 * (int64_t)ctx->c.h_nodemap.size();
    const bool mixed = o && (o->precision == SGLD_PREC_MIXED || o->precision == SGLD_PREC_MIXED_DF);
    if (nrhs > 0 && mixed && !o->history && !o->profile && !inner_loop_on_host()) {
        // all cases in one graph launch: F (and U0) staged in d_blk, U back from it
        if (o->maxit < 1 || !(o->tol >= 0.0)) return fail(ctx, SGLD_ERR_ARG, "maxit must be >= 1 and tol >= 0");
        Ctx &c = ctx->c;
        if ((rc = ensure_block_buffers(ctx, nrhs))) return rc;
        const size_t bytes = sizeof(double) * (size_t)nrhs * nd;
        CK(cudaMemcpyAsync(c.d_blk, F, bytes, cudaMemcpyHostToDevice, c.stream));
        if (o->use_x0) CK(cudaMemcpyAsync(c.d_blk + (size_t)nrhs * nd, U, bytes, cudaMemcpyHostToDevice, c.stream));
        std::vector<double> u0;   // starts of the cases, for a fallback
        if (o->use_x0) u0.assign(U, U + (size_t)nrhs * nd);
        std::vector<sgld_solve_info> local;
        if (!info) {
            local.resize((size_t)nrhs);
            info = local.data();
        }
        for (int j = 0; j < nrhs; ++j) memset(info + j, 0, sizeof *info);
        if ((rc = run_solve_graph(ctx, nrhs, true, o, info))) return rc;
        CK(cudaMemcpyAsync(U, c.d_blk + (size_t)nrhs * nd, bytes, cudaMemcpyDeviceToHost, c.stream));
        CK(cudaStreamSynchronize(c.stream));
        // cases whose recurrence met tol but whose true residual is above it
        // restart from their x (a single-load mixed solve, with its own residual
        // replacement and fallback); cases whose mixed solve failed: a zero load
        // has the solution 0, any other case reruns as the reference-form FP64
        // solve from the same start
        for (int j = 0; j < nrhs; ++j) {
            if (!mixed_failed(info[j], o->tol)) continue;
            if (info[j].converged && std::isfinite(info[j].relres) && std::isfinite(info[j].true_relres) &&
                info[j].iterations < o->maxit) {
                sgld_solve_opts o2 = *o;
                o2.use_x0 = 1;
                o2.maxit = o->maxit - info[j].iterations;
                sgld_solve_info r;
                if ((rc = sgld_pcg(ctx, F + (size_t)j * nd, U + (size_t)j * nd, &o2, &r))) return rc;
                if (!r.fallback) {
                    r.iterations += info[j].iterations;
                    r.inner_iterations += info[j].inner_iterations;
                }
                r.seconds += info[j].seconds;
                r.replacements += 1;
                info[j] = r;
                continue;
            }
            const double *Fj = F + (size_t)j * nd;
            if (std::all_of(Fj, Fj + nd, [](double v) { return v == 0.0; })) {
                std::fill(U + (size_t)j * nd, U + (size_t)(j + 1) * nd, 0.0);
                memset(info + j, 0, sizeof *info);
                info[j].converged = 1;
                continue;
            }
            sgld_solve_opts o64 = *o;
            o64.precision = SGLD_PREC_FP64;
            if (o->use_x0)
                std::copy(u0.begin() + (size_t)j * nd, u0.begin() + (size_t)(j + 1) * nd, U + (size_t)j * nd);
            else
                std::fill(U + (size_t)j * nd, U + (size_t)(j + 1) * nd, 0.0);
            if ((rc = sgld_pcg(ctx, F + (size_t)j * nd, U + (size_t)j * nd, &o64, info + j))) return rc;
            info[j].fallback = 1;
        }
        return SGLD_OK;
    }
    for (int j = 0; j < nrhs; ++j)
        if ((rc = sgld_pcg(ctx, F + j * nd, U + j * nd, o, info ? info + j : nullptr))) return rc;
    return SGLD_OK;
}

int sgld_compliance(sgld_ctx *ctx, const double *U, double *ce, double *cval) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (!U) return fail(ctx, SGLD_ERR_ARG, "null vector");
    Ctx &c = ctx->c;
    if ((rc = upload_nodes(ctx, U, c.d_z))) return rc;
    int nb = 0;
    launch_unit_compliance(c.lv[0], c.d_z, c.E, c.d_q, c.d_part, &nb, c.stream);
    launch_finalize_sum(c.d_part, nb, c.d_scal + 16, c.stream);
    CKL();
    if (cval) CK(cudaMemcpyAsync(cval, c.d_scal + 16, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    if (ce) {
        const int64_t ne = (int64_t)c.h_elemap.size();
        launch_gather_elems(c.d_elemap, ne, c.d_q, c.d_tmp, c.stream);
        CKL();
        CK(cudaMemcpyAsync(ce, c.d_tmp, sizeof(double) * ne, cudaMemcpyDeviceToHost, c.stream));
    }
    CK(cudaStreamSynchronize(c.stream));
    return SGLD_OK;
}

int sgld_stress(sgld_ctx *ctx, const double *U, double *nodal, double *vmn, double *vme) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (!U) return fail(ctx, SGLD_ERR_ARG, "null vector");
    Ctx &c = ctx->c;
    const Level &l0 = c.lv[0];
    if (!ctx->d_s6) {
        CK(dalloc(&ctx->d_s6, 6 * (size_t)l0.nnode));
        CK(dalloc(&ctx->d_vmn, (size_t)l0.nnode));
        CK(dalloc(&ctx->d_vme, (size_t)l0.nel));
    }
    if ((rc = upload_nodes(ctx, U, c.d_z))) return rc;
    double M[48 * 24];
    stress_matrix(c.nu, c.cell, M);
    launch_stress(l0, c.E, c.d_z, M, ctx->d_s6, ctx->d_vmn, c.stream);
    launch_elem_vm(l0, ctx->d_s6, ctx->d_vme, c.stream);
    CKL();
    CK(cudaStreamSynchronize(c.stream));
    const auto &nm = c.h_nodemap;
    if (nodal || vmn) {
        std::vector<double> s6(6 * l0.nnode), v(l0.nnode);
        CK(cudaMemcpy(s6.data(), ctx->d_s6, sizeof(double) * s6.size(), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(v.data(), ctx->d_vmn, sizeof(double) * v.size(), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < nm.size(); ++i) {
            if (nodal)
                for (int k = 0; k < 6; ++k) nodal[6 * i + k] = s6[6 * nm[i] + k];
            if (vmn) vmn[i] = v[nm[i]];
        }
    }
    if (vme) {
        const int64_t ne = (int64_t)c.h_elemap.size();
        launch_gather_elems(c.d_elemap, ne, ctx->d_vme, c.d_tmp, c.stream);
        CKL();
        CK(cudaMemcpyAsync(vme, c.d_tmp, sizeof(double) * ne, cudaMemcpyDeviceToHost, c.stream));
        CK(cudaStreamSynchronize(c.stream));
    }
    return SGLD_OK;
}

int sgld_principal_stress(sgld_ctx *ctx, const double *U, double *ps_node, double *dir_elem) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (!U) return fail(ctx, SGLD_ERR_ARG, "null vector");
    Ctx &c = ctx->c;
    const Level &l0 = c.lv[0];
    if (!ctx->d_s6) {
        CK(dalloc(&ctx->d_s6, 6 * (size_t)l0.nnode));
        CK(dalloc(&ctx->d_vmn, (size_t)l0.nnode));
        CK(dalloc(&ctx->d_vme, (size_t)l0.nel));
    }
    if ((rc = upload_nodes(ctx, U, c.d_z))) return rc;
    double M[48 * 24];
    stress_matrix(c.nu, c.cell, M);
    launch_stress(l0, c.E, c.d_z, M, ctx->d_s6, ctx->d_vmn, c.stream);
    // one output at a time through a temporary full-grid buffer (12 doubles
    // per node or 3 per element), gathered to the compact order on the host
    auto fetch = [&](int per, int64_t count, const std::vector<int64_t> &map, double *out, bool nodes) -> int {
        double *d_buf = nullptr;
        CK(dalloc(&d_buf, (size_t)per * count));
        if (nodes)
            launch_principal(l0, ctx->d_s6, d_buf, nullptr, c.stream);
        else
            launch_principal(l0, ctx->d_s6, nullptr, d_buf, c.stream);
        std::vector<double> h((size_t)per * count);
        const cudaError_t e1 = cudaGetLastError();
        const cudaError_t e2 = cudaMemcpyAsync(h.data(), d_buf, sizeof(double) * h.size(), cudaMemcpyDeviceToHost,
                                               c.stream);
        const cudaError_t e3 = cudaStreamSynchronize(c.stream);
        cudaFree(d_buf);
        CK(e1);
        CK(e2);
        CK(e3);
        for (size_t i = 0; i < map.size(); ++i)
            for (int k = 0; k < per; ++k) out[(size_t)per * i + k] = h[(size_t)per * map[i] + k];
        return SGLD_OK;
    };
    if (ps_node && (rc = fetch(12, l0.nnode, c.h_nodemap, ps_node, true))) return rc;
    if (dir_elem && (rc = fetch(3, l0.nel, c.h_elemap, dir_elem, false))) return rc;
    return SGLD_OK;
}

int sgld_kbyu_prec(sgld_ctx *ctx, const double *u, double *y, int precision) {
    if (precision == SGLD_PREC_FP64) return sgld_kbyu(ctx, u, y);
    if (precision == SGLD_PREC_MIXED_DF) return sgld_kbyu_df(ctx, u, y);
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (precision != SGLD_PREC_MIXED) return fail(ctx, SGLD_ERR_ARG, "unknown precision mode");
    if (!u || !y) return fail(ctx, SGLD_ERR_ARG, "null vector");
    Ctx &c = ctx->c;
    const Level &l0 = c.lv[0];
    const int64_t nv = 3 * l0.nnode;
    if ((rc = upload_nodes(ctx, u, c.d_p))) return rc;
    launch_cast_f32(c.E, c.d_E32, l0.nel, c.stream);
    launch_narrow(c.d_p, c.d_r32, nv, c.stream);
    launch_kbyu_f32(l0, c.d_E32, c.d_r32, c.d_t32, nullptr, nullptr, c.stream);
    launch_widen(c.d_t32, c.d_q, nv, c.stream);
    CKL();
    return download_nodes(ctx, c.d_q, y);
}

int sgld_vcycle_prec(sgld_ctx *ctx, const double *r, double *z, int precision) {
    if (precision == SGLD_PREC_FP64) return sgld_vcycle(ctx, r, z);
    int rc = check_assembled(ctx);
    if (rc) return rc;
    if (precision != SGLD_PREC_MIXED && precision != SGLD_PREC_MIXED_DF)
        return fail(ctx, SGLD_ERR_ARG, "unknown precision mode");
    if (!r || !z) return fail(ctx, SGLD_ERR_ARG, "null vector");
    Ctx &c = ctx->c;
    const int64_t nv = 3 * c.lv[0].nnode;
    if ((rc = upload_nodes(ctx, r, c.d_p))) return rc;
    launch_narrow(c.d_p, c.d_r32, nv, c.stream);
    if ((rc = vcycle_dev32(ctx, c.d_r32, c.d_z32, nullptr, nullptr))) return rc;
    launch_widen(c.d_z32, c.d_z, nv, c.stream);
    CKL();
    return download_nodes(ctx, c.d_z, z);
}

int sgld_build_hierarchy(sgld_ctx *ctx, int num_levels, int non_dyadic) {
    if (!ctx) return SGLD_ERR_ARG;
    if (int rc = bind_ctx(ctx)) return rc;
    Ctx &c = ctx->c;
    const Level &l0 = c.lv[0];
    sgld_options o;
    sgld_default_options(&o);
    o.num_levels = num_levels;
    o.non_dyadic = non_dyadic;
    o.poisson_ratio = c.nu;
    o.cell_size = c.cell;
    o.omega = c.omega;
    o.device = c.device;
    sgld_ctx *fresh = nullptr;
    int rc = sgld_create(l0.ny, l0.nx, l0.nz, l0.h_eact.data(), &o, &fresh);
    if (rc == SGLD_OK && memcmp(fresh->c.Ke, c.Ke, sizeof c.Ke) != 0) rc = sgld_set_ke(fresh, c.Ke);
    if (rc != SGLD_OK) {
        c.err = fresh ? fresh->c.err : std::string("sgld_build_hierarchy: create failed");
        sgld_destroy(fresh);
        return rc;
    }
    std::swap(*ctx, *fresh);   // the handle keeps its address; the old levels go with `fresh`
    sgld_destroy(fresh);
    return bind_ctx(ctx);
}

int sgld_solve(sgld_ctx *ctx, int nrhs, const double *F, double *U, double tol, int maxit, int precision, int *its,
               double *relres) {
    sgld_solve_opts o;
    memset(&o, 0, sizeof o);
    o.tol = tol;
    o.maxit = maxit;
    o.precision = precision;
    std::vector<sgld_solve_info> infos((size_t)std::max(nrhs, 1));
    const int rc = sgld_solve_block(ctx, nrhs, F, U, &o, infos.data());
    if (rc) return rc;
    for (int i = 0; i < nrhs; ++i) {
        if (its) its[i] = infos[i].iterations;
        if (relres) relres[i] = infos[i].relres;
    }
    return SGLD_OK;
}

int sgld_vonmises(sgld_ctx *ctx, const double *U, double *vm_elem, double *vm_node) {
    return sgld_stress(ctx, U, nullptr, vm_node, vm_elem);
}

}  // extern "C"

// =============================================================================
namespace {

// FP64 PCG on the full-grid vectors in ctx (Solving_PreconditionedConjugateGradientSolver.m:7-36)
int pcg_dev(sgld_ctx *ctx, const sgld_solve_opts *o, sgld_solve_info *info) {
    Ctx &c = ctx->c;
    const Level &l0 = c.lv[0];
    const int64_t nv = 3 * l0.nnode;
    const int nbv = reduce_blocks(nv);
    const double tol = o->tol;
    const int maxit = o->maxit;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, c.stream));
    int nb = 0;
    launch_pcg_scalar(5, c.d_scal, c.d_iflag, c.d_part, 1, tol, maxit, c.stream);
    launch_dot(c.d_b, c.d_b, nv, c.d_part, nbv, c.stream);
    launch_pcg_scalar(0, c.d_scal, c.d_iflag, c.d_part, nbv, tol, maxit, c.stream);
    if (o->use_x0) {
        launch_kbyu_f64(l0, c.E, c.d_x, c.d_q, nullptr, nullptr, c.stream);
        launch_residual(c.d_r, c.d_b, c.d_q, nv, c.stream);
    } else {
        CK(cudaMemcpyAsync(c.d_r, c.d_b, sizeof(double) * nv, cudaMemcpyDeviceToDevice, c.stream));
    }
    int rc = vcycle_dev(ctx, c.d_r, c.d_z, c.d_part, &nb);
    if (rc) return rc;
    launch_pcg_scalar(1, c.d_scal, c.d_iflag, c.d_part, nb, tol, maxit, c.stream);
    CK(cudaMemcpyAsync(c.d_p, c.d_z, sizeof(double) * nv, cudaMemcpyDeviceToDevice, c.stream));
    int h_flag[4] = {0, 0, 0, 0};
    int its = 0;
    const int poll = 1;
    const bool prof = o->profile != 0;
    cudaEvent_t pe[4] = {nullptr, nullptr, nullptr, nullptr};   // K*u start/end, precond start/end
    if (prof)
        for (auto &e : pe) CK(cudaEventCreate(&e));
    double kb_ms = 0.0, pc_ms = 0.0;
    int kb_n = 0;
    bool pc_pending = false;
    for (int k = 1; k <= maxit; ++k) {
        if (prof) CK(cudaEventRecord(pe[0], c.stream));
        launch_kbyu_f64(l0, c.E, c.d_p, c.d_q, c.d_part, &nb, c.stream);
        if (prof) CK(cudaEventRecord(pe[1], c.stream));
        launch_pcg_scalar(2, c.d_scal, c.d_iflag, c.d_part, nb, tol, maxit, c.stream);
        launch_pcg_update(c.d_x, c.d_r, c.d_p, c.d_q, nv, c.d_scal, c.d_iflag, c.d_part, nbv, c.stream);
        launch_pcg_scalar(3, c.d_scal, c.d_iflag, c.d_part, nbv, tol, maxit, c.stream);
        if (o->history || (k % poll) == 0 || k == maxit) {
            CK(cudaMemcpyAsync(h_flag, c.d_iflag, sizeof(int) * 4, cudaMemcpyDeviceToHost, c.stream));
            if (o->history) CK(cudaMemcpyAsync(o->history + (k - 1), c.d_scal + 3, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            CK(cudaStreamSynchronize(c.stream));
            if (prof) {
                float t = 0.f;
                cudaEventElapsedTime(&t, pe[0], pe[1]);
                kb_ms += t;
                ++kb_n;
                if (pc_pending) {
                    cudaEventElapsedTime(&t, pe[2], pe[3]);
                    pc_ms += t;
                    pc_pending = false;
                }
            }
            if (h_flag[2]) break;
        }
        if (prof) CK(cudaEventRecord(pe[2], c.stream));
        if ((rc = vcycle_dev(ctx, c.d_r, c.d_z, c.d_part, &nb))) return rc;
        if (prof) {
            CK(cudaEventRecord(pe[3], c.stream));
            pc_pending = true;
        }
        launch_pcg_scalar(4, c.d_scal, c.d_iflag, c.d_part, nb, tol, maxit, c.stream);
        launch_pcg_pupdate(c.d_p, c.d_z, nv, c.d_scal, c.d_iflag, c.stream);
        CKL();
    }
    CK(cudaEventRecord(e1, c.stream));
    if (prof) {
        CK(cudaStreamSynchronize(c.stream));
        if (pc_pending) {
            float t = 0.f;
            cudaEventElapsedTime(&t, pe[2], pe[3]);
            pc_ms += t;
        }
        for (auto &e : pe) cudaEventDestroy(e);
    }
    CK(cudaMemcpyAsync(h_flag, c.d_iflag, sizeof(int) * 4, cudaMemcpyDeviceToHost, c.stream));
    double sc[8];
    CK(cudaMemcpyAsync(sc, c.d_scal, sizeof(double) * 8, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    its = h_flag[0];
    // true residual in FP64
    launch_kbyu_f64(l0, c.E, c.d_x, c.d_q, nullptr, nullptr, c.stream);
    launch_residual(c.d_tmp, c.d_b, c.d_q, nv, c.stream);
    launch_dot(c.d_tmp, c.d_tmp, nv, c.d_part, nbv, c.stream);
    launch_finalize_sum(c.d_part, nbv, c.d_scal + 17, c.stream);
    CKL();
    double rr = 0;
    CK(cudaMemcpyAsync(&rr, c.d_scal + 17, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    if (info) {
        info->iterations = its;
        info->converged = h_flag[1];
        info->relres = sc[3];
        info->true_relres = sc[0] > 0 ? sqrt(rr) / sc[0] : 0.0;
        info->inner_iterations = 0;
        info->seconds = ms * 1e-3;
        info->kbyu_seconds = kb_ms * 1e-3;
        info->kbyu_launches = kb_n;
        info->precond_seconds = pc_ms * 1e-3;
    }
    return SGLD_OK;
}

// Mixed precision: FP64 flexible PCG whose preconditioner is k FP32 CG
// iterations with the FP32 additive V-cycle (graph-captured).  The FP64
// residual recurrence, dot products and stopping test stay in FP64, so the
// outer solve reaches the same tolerance on the true residual.  The outer K*p
// is the native FP64 operator (SGLD_PREC_MIXED) or the double-float one
// (SGLD_PREC_MIXED_DF, ~2^-48 relative, FP32 issue rate), and so are the
// warm-start residual and the true residual at exit.
int pcg_mixed_dev(sgld_ctx *ctx, const sgld_solve_opts *o, sgld_solve_info *info) {
    // the whole solve as one graph launch unless a per-iteration host record
    // (history, profile) or the host-driven inner loop is asked for
    if (!o->history && !o->profile && !inner_loop_on_host()) return run_solve_graph(ctx, 1, false, o, info);
    Ctx &c = ctx->c;
    const Level &l0 = c.lv[0];
    const int64_t nv = 3 * l0.nnode;
    const int nbv = reduce_blocks(nv);
    const double tol = o->tol;
    const int maxit = o->maxit;
    // inner solve: a fixed inner_its iterations when inner_tol == 0 and
    // inner_its > 0; otherwise stop at ||s|| <= max(inner_tol, tol / (2 relres))
    // ||r|| (inner_tol default 3e-4) or after inner_its (default 64) iterations
    const bool fixed_k = o->inner_its > 0 && !(o->inner_tol > 0.0);
    const int k = o->inner_its > 0 ? o->inner_its : 64;
    const double eta = fixed_k ? 0.0 : (o->inner_tol > 0.0 ? o->inner_tol : 3e-4);
    const bool dfk = o->precision == SGLD_PREC_MIXED_DF;
    CK(cudaMemsetAsync(c.d_isc + IS_TOTAL, 0, sizeof(double), c.stream));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, c.stream));
    int nb = 0, rc;
    launch_pcg_scalar(5, c.d_scal, c.d_iflag, c.d_part, 1, tol, maxit, c.stream);
    launch_dot(c.d_b, c.d_b, nv, c.d_part, nbv, c.stream);
    launch_pcg_scalar(0, c.d_scal, c.d_iflag, c.d_part, nbv, tol, maxit, c.stream);
    if (o->use_x0) {
        if (dfk)
            launch_kbyu_df(l0, c.E, c.d_x, c.d_q, nullptr, nullptr, c.stream);
        else
            launch_kbyu_f64(l0, c.E, c.d_x, c.d_q, nullptr, nullptr, c.stream);
        launch_residual(c.d_r, c.d_b, c.d_q, nv, c.stream);
    } else {
        CK(cudaMemcpyAsync(c.d_r, c.d_b, sizeof(double) * nv, cudaMemcpyDeviceToDevice, c.stream));
    }
    launch_narrow(c.d_r, c.d_r32, nv, c.stream);
    if ((rc = inner_run(ctx, k, eta))) return rc;
    launch_widen_dots(c.d_e32, c.d_d32, c.d_isc, c.d_z, c.d_r, c.d_r, nv, c.d_part, c.d_part2, nbv, c.stream);
    launch_flex_beta(c.d_scal, c.d_iflag, c.d_part, c.d_part2, nbv, 1, c.stream);
    CK(cudaMemcpyAsync(c.d_p, c.d_z, sizeof(double) * nv, cudaMemcpyDeviceToDevice, c.stream));
    int h_flag[4] = {0, 0, 0, 0};
    const bool prof = o->profile != 0;
    cudaEvent_t pe[4] = {nullptr, nullptr, nullptr, nullptr};
    if (prof)
        for (auto &e : pe) CK(cudaEventCreate(&e));
    double kb_ms = 0.0, pc_ms = 0.0;
    int kb_n = 0;
    bool pc_pending = false;
    for (int it = 1; it <= maxit; ++it) {
        if (prof) CK(cudaEventRecord(pe[0], c.stream));
        if (dfk)
            launch_kbyu_df(l0, c.E, c.d_p, c.d_q, c.d_part, &nb, c.stream);
        else
            launch_kbyu_f64(l0, c.E, c.d_p, c.d_q, c.d_part, &nb, c.stream);
        if (prof) CK(cudaEventRecord(pe[1], c.stream));
        launch_pcg_scalar(2, c.d_scal, c.d_iflag, c.d_part, nb, tol, maxit, c.stream);
        launch_pcg_update(c.d_x, c.d_r, c.d_p, c.d_q, nv, c.d_scal, c.d_iflag, c.d_part, nbv, c.stream);
        launch_pcg_scalar(3, c.d_scal, c.d_iflag, c.d_part, nbv, tol, maxit, c.stream);
        CK(cudaMemcpyAsync(h_flag, c.d_iflag, sizeof(int) * 4, cudaMemcpyDeviceToHost, c.stream));
        if (o->history) CK(cudaMemcpyAsync(o->history + (it - 1), c.d_scal + 3, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        CK(cudaStreamSynchronize(c.stream));
        if (prof) {
            float t = 0.f;
            cudaEventElapsedTime(&t, pe[0], pe[1]);
            kb_ms += t;
            ++kb_n;
            if (pc_pending) {
                cudaEventElapsedTime(&t, pe[2], pe[3]);
                pc_ms += t;
                pc_pending = false;
            }
        }
        if (h_flag[2]) break;
        if (prof) CK(cudaEventRecord(pe[2], c.stream));
        launch_narrow(c.d_r, c.d_r32, nv, c.stream);
        if ((rc = inner_run(ctx, k, eta))) return rc;
        launch_widen_dots(c.d_e32, c.d_d32, c.d_isc, c.d_z, c.d_r, c.d_q, nv, c.d_part, c.d_part2, nbv, c.stream);
        if (prof) {
            CK(cudaEventRecord(pe[3], c.stream));
            pc_pending = true;
        }
        launch_flex_beta(c.d_scal, c.d_iflag, c.d_part, c.d_part2, nbv, 0, c.stream);
        launch_pcg_pupdate(c.d_p, c.d_z, nv, c.d_scal, c.d_iflag, c.stream);
        CKL();
    }
    CK(cudaEventRecord(e1, c.stream));
    double sc[8], inner_total = 0.0;
    CK(cudaMemcpyAsync(h_flag, c.d_iflag, sizeof(int) * 4, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaMemcpyAsync(sc, c.d_scal, sizeof(double) * 8, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaMemcpyAsync(&inner_total, c.d_isc + IS_TOTAL, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    if (!inner_loop_on_host()) g_launches += (int64_t)inner_total * c.inner_body_launches;
    if (prof) {
        if (pc_pending) {
            float t = 0.f;
            cudaEventElapsedTime(&t, pe[2], pe[3]);
            pc_ms += t;
        }
        for (auto &e : pe) cudaEventDestroy(e);
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (dfk)
        launch_kbyu_df(l0, c.E, c.d_x, c.d_q, nullptr, nullptr, c.stream);
    else
        launch_kbyu_f64(l0, c.E, c.d_x, c.d_q, nullptr, nullptr, c.stream);
    launch_residual(c.d_tmp, c.d_b, c.d_q, nv, c.stream);
    launch_dot(c.d_tmp, c.d_tmp, nv, c.d_part, nbv, c.stream);
    launch_finalize_sum(c.d_part, nbv, c.d_scal + 17, c.stream);
    CKL();
    double rr = 0;
    CK(cudaMemcpyAsync(&rr, c.d_scal + 17, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    if (info) {
        info->iterations = h_flag[0];
        info->converged = h_flag[1];
        info->relres = sc[3];
        info->true_relres = sc[0] > 0 ? sqrt(rr) / sc[0] : 0.0;
        info->inner_iterations = (int)inner_total;
        info->seconds = ms * 1e-3;
        info->kbyu_seconds = kb_ms * 1e-3;
        info->kbyu_launches = kb_n;
        info->precond_seconds = pc_ms * 1e-3;
    }
    return SGLD_OK;
}

// ---------------------------------------------------------------------------
// The mixed-precision solve of one or several load cases as ONE CUDA graph:
// per case a prologue, the outer flexible-PCG loop as a conditional while
// node, and an epilogue.  The outer body is
//   q = K p; lambda; x, r update; residual test; set the loop conditions;
//   if not stopped (conditional if node): r32 = r; inner FP32 CG (its own
//     while node, nested); z = e + alpha d; flexible beta; p = z + beta p,
// so a whole block of cases runs from one launch with no host round trip.
// Staged cases take F (and U0) from d_blk (compact DOFs, case after case) and
// return U there; an unstaged single case uses d_b / d_x as they are.
// Per-case results land in d_binfo (8 doubles each): the outer flags (4 ints),
// relative residual, ||b||, true residual^2, inner iterations.
static int build_solve_graph(sgld_ctx *ctx, int nrhs, bool staged, bool use_x0, int kmax, double eta, double tol,
                             int maxit, bool dfk) {
    Ctx &c = ctx->c;
    const Level &l0 = c.lv[0];
    const int64_t nv = 3 * l0.nnode, ncomp = (int64_t)c.h_nodemap.size(), nd = 3 * ncomp;
    const int nbv = reduce_blocks(nv);
    auto kbyu_outer = [&](const double *u, double *y, double *part, int *nb, cudaStream_t st) {
        if (dfk)
            launch_kbyu_df(l0, c.E, u, y, part, nb, st);
        else
            launch_kbyu_f64(l0, c.E, u, y, part, nb, st);
    };
    cudaGraph_t g = nullptr;
    CK(cudaGraphCreate(&g, 0));
    const int64_t start = g_launches;
    cudaStream_t s = c.stream;
    CK(cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    int rc = SGLD_OK;
    int64_t fixed = 0, outer = 0, ifb = 0, inner = 0, e_in = 0;
    for (int j = 0; j < nrhs && rc == SGLD_OK; ++j) {
        int64_t t0 = g_launches;
        cudaMemsetAsync(c.d_isc + IS_TOTAL, 0, sizeof(double), s);
        if (staged) {
            cudaMemsetAsync(c.d_b, 0, sizeof(double) * nv, s);
            launch_scatter_nodes(c.d_nodemap, ncomp, c.d_blk + j * nd, c.d_b, s);
            cudaMemsetAsync(c.d_x, 0, sizeof(double) * nv, s);
            if (use_x0) launch_scatter_nodes(c.d_nodemap, ncomp, c.d_blk + (nrhs + j) * nd, c.d_x, s);
        }
        launch_pcg_scalar(5, c.d_scal, c.d_iflag, c.d_part, 1, tol, maxit, s);
        launch_dot(c.d_b, c.d_b, nv, c.d_part, nbv, s);
        launch_pcg_scalar(0, c.d_scal, c.d_iflag, c.d_part, nbv, tol, maxit, s);
        if (use_x0) {
            kbyu_outer(c.d_x, c.d_q, nullptr, nullptr, s);
            launch_residual(c.d_r, c.d_b, c.d_q, nv, s);
        } else {
            cudaMemcpyAsync(c.d_r, c.d_b, sizeof(double) * nv, cudaMemcpyDeviceToDevice, s);
        }
        launch_narrow(c.d_r, c.d_r32, nv, s);
        const int64_t t1 = g_launches;
        if ((rc = capture_inner(ctx, s, c.aux[0], kmax, eta, &e_in, &inner))) break;
        const int64_t t2 = g_launches;
        launch_widen_dots(c.d_e32, c.d_d32, c.d_isc, c.d_z, c.d_r, c.d_r, nv, c.d_part, c.d_part2, nbv, s);
        launch_flex_beta(c.d_scal, c.d_iflag, c.d_part, c.d_part2, nbv, 1, s);
        cudaMemcpyAsync(c.d_p, c.d_z, sizeof(double) * nv, cudaMemcpyDeviceToDevice, s);
        const int64_t t3 = g_launches;
        // outer loop
        cudaGraphConditionalHandle hw;
        if (cudaGraphConditionalHandleCreate(&hw, capturing_graph(s), 1, cudaGraphCondAssignDefault) != cudaSuccess) {
            rc = fail(ctx, SGLD_ERR_CUDA, "conditional handle");
            break;
        }
        cudaGraph_t wbody = nullptr;
        if ((rc = add_conditional(ctx, s, hw, cudaGraphCondTypeWhile, &wbody))) break;
        cudaStream_t sw = c.aux[0], si = c.aux[1];
        CK(cudaStreamBeginCaptureToGraph(sw, wbody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        const int64_t t4 = g_launches;
        int nb = 0;
        kbyu_outer(c.d_p, c.d_q, c.d_part, &nb, sw);
        launch_pcg_scalar(2, c.d_scal, c.d_iflag, c.d_part, nb, tol, maxit, sw);
        launch_pcg_update(c.d_x, c.d_r, c.d_p, c.d_q, nv, c.d_scal, c.d_iflag, c.d_part, nbv, sw);
        launch_pcg_scalar(3, c.d_scal, c.d_iflag, c.d_part, nbv, tol, maxit, sw);
        cudaGraphConditionalHandle hi;
        CK(cudaGraphConditionalHandleCreate(&hi, capturing_graph(sw), 0, cudaGraphCondAssignDefault));
        launch_outer_cond(hw, hi, c.d_iflag, sw);
        const int64_t t5 = g_launches;
        cudaGraph_t ibody = nullptr;
        if ((rc = add_conditional(ctx, sw, hi, cudaGraphCondTypeIf, &ibody))) break;
        CK(cudaStreamBeginCaptureToGraph(si, ibody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        launch_narrow(c.d_r, c.d_r32, nv, si);
        const int64_t t6 = g_launches;
        int64_t e2 = 0, b2 = 0;
        if ((rc = capture_inner(ctx, si, c.aux[2], kmax, eta, &e2, &b2))) break;
        const int64_t t7 = g_launches;
        launch_widen_dots(c.d_e32, c.d_d32, c.d_isc, c.d_z, c.d_r, c.d_q, nv, c.d_part, c.d_part2, nbv, si);
        launch_flex_beta(c.d_scal, c.d_iflag, c.d_part, c.d_part2, nbv, 0, si);
        launch_pcg_pupdate(c.d_p, c.d_z, nv, c.d_scal, c.d_iflag, si);
        const int64_t t8 = g_launches;
        CK(cudaStreamEndCapture(si, &ibody));
        CK(cudaStreamEndCapture(sw, &wbody));
        // epilogue: true residual, results, U
        const int64_t t9 = g_launches;
        kbyu_outer(c.d_x, c.d_q, nullptr, nullptr, s);
        launch_residual(c.d_tmp, c.d_b, c.d_q, nv, s);
        launch_dot(c.d_tmp, c.d_tmp, nv, c.d_part, nbv, s);
        double *info = c.d_binfo + 8 * j;
        launch_finalize_sum(c.d_part, nbv, info + 4, s);
        cudaMemcpyAsync(info, c.d_iflag, 4 * sizeof(int), cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(info + 2, c.d_scal + 3, sizeof(double), cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(info + 3, c.d_scal + 0, sizeof(double), cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(info + 5, c.d_isc + IS_TOTAL, sizeof(double), cudaMemcpyDeviceToDevice, s);
        if (staged) launch_gather_nodes(c.d_nodemap, ncomp, c.d_x, c.d_blk + (nrhs + j) * nd, s);
        const int64_t t10 = g_launches;
        fixed = (t1 - t0) + e_in + (t3 - t2) + (t10 - t9);
        outer = t5 - t4;
        ifb = (t6 - t5) + e2 + (t8 - t7);
    }
    cudaGraph_t gend = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(s, &gend);
    g_launches = start;
    if (rc == SGLD_OK && ec != cudaSuccess) rc = fail(ctx, SGLD_ERR_CUDA, std::string("solve graph capture: ") + cudaGetErrorString(ec));
    if (rc == SGLD_OK) {
        const cudaError_t ei = cudaGraphInstantiate(&c.solve_graph, g, 0);
        if (ei != cudaSuccess) rc = fail(ctx, SGLD_ERR_CUDA, std::string("solve graph instantiate: ") + cudaGetErrorString(ei));
    }
    cudaGraphDestroy(g);
    c.sg_fixed = fixed;
    c.sg_outer = outer;
    c.sg_if = ifb;
    c.sg_inner = inner;
    return rc;
}

static int ensure_block_buffers(sgld_ctx *ctx, int nrhs) {
    Ctx &c = ctx->c;
    if (nrhs <= c.blk_cap) return SGLD_OK;
    if (c.d_blk) cudaFree(c.d_blk);
    if (c.d_binfo) cudaFree(c.d_binfo);
    c.d_blk = nullptr;
    c.d_binfo = nullptr;
    c.blk_cap = 0;
    if (c.solve_graph) {   // the graph refers to the old buffers
        cudaGraphExecDestroy(c.solve_graph);
        c.solve_graph = nullptr;
    }
    const size_t nd = 3 * c.h_nodemap.size();
    CK(dalloc(&c.d_blk, 2 * (size_t)nrhs * nd));
    CK(dalloc(&c.d_binfo, 8 * (size_t)nrhs));
    c.blk_cap = nrhs;
    return SGLD_OK;
}

// runs the solve graph for nrhs cases (building it when the key changed)
static int run_solve_graph(sgld_ctx *ctx, int nrhs, bool staged, const sgld_solve_opts *o, sgld_solve_info *infos) {
    Ctx &c = ctx->c;
    const bool fixed_k = o->inner_its > 0 && !(o->inner_tol > 0.0);
    const int kmax = o->inner_its > 0 ? o->inner_its : 64;
    const double eta = fixed_k ? 0.0 : (o->inner_tol > 0.0 ? o->inner_tol : 3e-4);
    const bool dfk = o->precision == SGLD_PREC_MIXED_DF;
    int rc = ensure_block_buffers(ctx, std::max(nrhs, 1));
    if (rc) return rc;
    const std::vector<double> key = {(double)nrhs, staged ? 1.0 : 0.0, o->use_x0 ? 1.0 : 0.0, (double)kmax, eta,
                                     o->tol, (double)o->maxit, dfk ? 1.0 : 0.0};
    if (!c.solve_graph || key != c.solve_key) {
        if (c.solve_graph) {
            cudaGraphExecDestroy(c.solve_graph);
            c.solve_graph = nullptr;
        }
        if ((rc = build_solve_graph(ctx, nrhs, staged, o->use_x0 != 0, kmax, eta, o->tol, o->maxit, dfk))) return rc;
        c.solve_key = key;
    }
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, c.stream));
    CK(cudaGraphLaunch(c.solve_graph, c.stream));
    CK(cudaEventRecord(e1, c.stream));
    std::vector<double> res(8 * (size_t)nrhs);
    CK(cudaMemcpyAsync(res.data(), c.d_binfo, sizeof(double) * res.size(), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (int j = 0; j < nrhs; ++j) {
        const double *r = res.data() + 8 * j;
        int fl[4];
        memcpy(fl, r, sizeof fl);
        const int its = fl[0];
        g_launches += c.sg_fixed + (int64_t)its * c.sg_outer + (int64_t)std::max(its - 1, 0) * c.sg_if +
                      (int64_t)r[5] * c.sg_inner;
        if (infos) {
            sgld_solve_info &in = infos[j];
            memset(&in, 0, sizeof in);
            in.iterations = its;
            in.converged = fl[1];
            in.relres = r[2];
            in.true_relres = r[3] > 0 ? sqrt(r[4]) / r[3] : 0.0;
            in.inner_iterations = (int)r[5];
            in.seconds = ms * 1e-3 / nrhs;
        }
    }
    return SGLD_OK;
}

}  // namespace

// PCG on the context's own full-grid vectors (b in d_b, x in d_x), used by the
// SIMP driver (sgld_topopt_api.cu)
int sgld::vcycle_f64(sgld_ctx *ctx, const double *r, double *z, double *partial, int *nb) {
    return vcycle_dev(ctx, r, z, partial, nb);
}

int sgld::vcycle_f32(sgld_ctx *ctx, const float *r, float *z, double *partial, int *nb) {
    return vcycle_dev32(ctx, r, z, partial, nb);
}

int sgld::solve_on_device(sgld_ctx *ctx, const sgld_solve_opts *o, sgld_solve_info *info) {
    int rc = check_assembled(ctx);
    if (rc) return rc;
    return solve_dev(ctx, o, info);
}

extern "C" int sgld_time_op(sgld_ctx *ctx, int op, int reps, double *ms_per_op) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (!ms_per_op || reps < 1 || op < 0 || op > 5) return fail(ctx, SGLD_ERR_ARG, "bad op / reps");
    if ((op == 2 || op == 3) && !ctx->c.assembled) return fail(ctx, SGLD_ERR_STATE, "stencil not assembled");
    Ctx &c = ctx->c;
    const Level &l0 = c.lv[0];
    const int64_t nv = 3 * l0.nnode;
    if (op == 1 || op == 3) {
        launch_cast_f32(c.E, c.d_E32, l0.nel, c.stream);
        launch_narrow(c.d_p, c.d_r32, nv, c.stream);
    }
    auto once = [&]() -> int {
        switch (op) {
            case 0: launch_kbyu_f64(l0, c.E, c.d_p, c.d_q, nullptr, nullptr, c.stream); break;
            case 1: launch_kbyu_f32(l0, c.d_E32, c.d_r32, c.d_t32, nullptr, nullptr, c.stream); break;
            case 2: return vcycle_dev(ctx, c.d_p, c.d_z, nullptr, nullptr);
            case 3: return vcycle_dev32(ctx, c.d_r32, c.d_z32, nullptr, nullptr);
            case 4: return sgld_assemble(ctx);
            case 5: launch_kbyu_df(l0, c.E, c.d_p, c.d_q, nullptr, nullptr, c.stream); break;
        }
        return SGLD_OK;
    };
    if ((rc = once())) return rc;   // warm-up
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaEventRecord(a, c.stream));
    for (int i = 0; i < reps; ++i)
        if ((rc = once())) return rc;
    CK(cudaEventRecord(b, c.stream));
    CK(cudaEventSynchronize(b));
    CKL();
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms_per_op = ms / reps;
    return SGLD_OK;
}
