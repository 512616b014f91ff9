// sgld_harness -- standalone command-line driver of the GB300 solver (C ABI only).
//
// Builds a solid cuboid cantilever ("Cuboid - Cantilever 3",
// FEA_BuiltInBoundaryConditions4CuboidDesignDomain.m:34-44: every node at x = 0
// fixed, a total unit -z load spread over the nodes of the x = max, z = 0 edge),
// sets a modulus field (uniform, or a seeded SIMP-graded field), assembles,
// solves with MGPCG and prints one JSON line with iterations, residuals,
// timings and the compliance.
//
//   sgld_harness [--size NX NY NZ] [--levels L] [--nondyadic 0|1] [--omega W]
//                [--tol T] [--maxit N] [--precision fp64|mixed|mixed_df] [--graded SEED] [--repeat R]
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <vector>

#include "sgld_gpu.h"

static void die(sgld_ctx *c, const char *where) {
    fprintf(stderr, "sgld_harness: %s failed: %s\n", where, c ? sgld_last_error(c) : "");
    exit(1);
}

// seeded density in [1e-3, 1]: uniform noise smoothed by three box passes
static std::vector<double> graded_modulus(int nx, int ny, int nz, unsigned seed) {
    const size_t n = (size_t)nx * ny * nz;
    std::vector<double> a(n), b(n);
    uint64_t s = 0x9E3779B97F4A7C15ull ^ seed;
    for (size_t i = 0; i < n; ++i) {
        s ^= s << 13;
        s ^= s >> 7;
        s ^= s << 17;
        a[i] = (double)(s >> 11) * (1.0 / 9007199254740992.0);
    }
    const int dims[3] = {ny, nx, nz};
    const size_t strides[3] = {1, (size_t)ny, (size_t)ny * nx};
    for (int pass = 0; pass < 3; ++pass)
        for (int ax = 0; ax < 3; ++ax) {
            for (size_t i = 0; i < n; ++i) {
                const int c = (int)((i / strides[ax]) % dims[ax]);
                double v = a[i], w = 1.0;
                if (c > 0) v += a[i - strides[ax]], w += 1.0;
                if (c + 1 < dims[ax]) v += a[i + strides[ax]], w += 1.0;
                b[i] = v / w;
            }
            a.swap(b);
        }
    double lo = 1e300, hi = -1e300;
    for (double v : a) lo = v < lo ? v : lo, hi = v > hi ? v : hi;
    for (double &v : a) {
        const double rho = 1e-3 + (v - lo) / (hi - lo) * (1.0 - 1e-3);
        v = 1e-9 + rho * rho * rho * (1.0 - 1e-9);   // TopOpti_MaterialInterpolationSIMP.m:5
    }
    return a;
}

int main(int argc, char **argv) {
    int nx = 64, ny = 32, nz = 32, levels = 4, nondyadic = 1, maxit = 500, graded = -1, repeat = 1;
    double omega = 0.6, tol = 1e-6;
    int precision = SGLD_PREC_FP64;
    for (int i = 1; i < argc; ++i) {
        if (!strcmp(argv[i], "--size") && i + 3 < argc) {
            nx = atoi(argv[++i]);
            ny = atoi(argv[++i]);
            nz = atoi(argv[++i]);
        } else if (!strcmp(argv[i], "--levels") && i + 1 < argc) {
            levels = atoi(argv[++i]);
        } else if (!strcmp(argv[i], "--nondyadic") && i + 1 < argc) {
            nondyadic = atoi(argv[++i]);
        } else if (!strcmp(argv[i], "--omega") && i + 1 < argc) {
            omega = atof(argv[++i]);
        } else if (!strcmp(argv[i], "--tol") && i + 1 < argc) {
            tol = atof(argv[++i]);
        } else if (!strcmp(argv[i], "--maxit") && i + 1 < argc) {
            maxit = atoi(argv[++i]);
        } else if (!strcmp(argv[i], "--precision") && i + 1 < argc) {
            const char *p = argv[++i];
            if (!strcmp(p, "fp64")) {
                precision = SGLD_PREC_FP64;
            } else if (!strcmp(p, "mixed")) {
                precision = SGLD_PREC_MIXED;
            } else if (!strcmp(p, "mixed_df")) {
                precision = SGLD_PREC_MIXED_DF;
            } else {
                fprintf(stderr, "sgld_harness: unknown precision %s (fp64, mixed or mixed_df)\n", p);
                return 2;
            }
        } else if (!strcmp(argv[i], "--graded") && i + 1 < argc) {
            graded = atoi(argv[++i]);
        } else if (!strcmp(argv[i], "--repeat") && i + 1 < argc) {
            repeat = atoi(argv[++i]);
        } else {
            fprintf(stderr, "usage: %s [--size NX NY NZ] [--levels L] [--nondyadic 0|1] [--omega W] [--tol T] "
                            "[--maxit N] [--precision fp64|mixed|mixed_df] [--graded SEED] [--repeat R]\n", argv[0]);
            return 2;
        }
    }
    std::vector<uint8_t> solid((size_t)nx * ny * nz, 1);
    sgld_options o;
    sgld_default_options(&o);
    o.num_levels = levels;
    o.non_dyadic = nondyadic;
    o.omega = omega;
    sgld_ctx *ctx = nullptr;
    if (sgld_create(ny, nx, nz, solid.data(), &o, &ctx) != SGLD_OK) die(ctx, "sgld_create");
    int res[3], span;
    int64_t ne = 0, nn = 0;
    if (sgld_level_info(ctx, 1, res, &span, &ne, &nn) != SGLD_OK) die(ctx, "sgld_level_info");
    std::vector<int64_t> nodes(nn);
    if (sgld_node_map(ctx, 1, nodes.data()) != SGLD_OK) die(ctx, "sgld_node_map");
    // boundary conditions: solid cuboid -> every node is active, compact = full order
    std::vector<uint8_t> fixed(3 * nn, 0);
    std::vector<double> F(3 * nn, 0.0);
    const int64_t NY = ny + 1, NX = nx + 1;
    int nload = 0;
    for (int64_t i = 0; i < nn; ++i) {
        const int64_t g = nodes[i] - 1, iy = g % NY, ix = (g / NY) % NX, iz = g / (NY * NX);
        (void)iy;
        if (ix == 0) fixed[3 * i] = fixed[3 * i + 1] = fixed[3 * i + 2] = 1;
        if (ix == nx && iz == 0) ++nload;
    }
    for (int64_t i = 0; i < nn; ++i) {
        const int64_t g = nodes[i] - 1, ix = (g / NY) % NX, iz = g / (NY * NX);
        if (ix == nx && iz == 0) F[3 * i + 2] = -1.0 / nload;
    }
    if (sgld_set_fixed_dofs(ctx, fixed.data()) != SGLD_OK) die(ctx, "sgld_set_fixed_dofs");
    std::vector<double> E = graded >= 0 ? graded_modulus(nx, ny, nz, (unsigned)graded) : std::vector<double>(ne, 1.0);
    std::vector<double> U(3 * nn, 0.0), ce(ne);
    sgld_solve_opts so;
    memset(&so, 0, sizeof so);
    so.tol = tol;
    so.maxit = maxit;
    so.precision = precision;
    sgld_solve_info info;
    double best = 1e300, c = 0.0;
    for (int r = 0; r < repeat; ++r) {
        const auto t0 = std::chrono::steady_clock::now();
        if (sgld_set_modulus(ctx, E.data()) != SGLD_OK) die(ctx, "sgld_set_modulus");
        if (sgld_assemble(ctx) != SGLD_OK) die(ctx, "sgld_assemble");
        if (sgld_pcg(ctx, F.data(), U.data(), &so, &info) != SGLD_OK) die(ctx, "sgld_pcg");
        const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        best = dt < best ? dt : best;
    }
    if (sgld_compliance(ctx, U.data(), ce.data(), &c) != SGLD_OK) die(ctx, "sgld_compliance");
    printf("{\"grid\": [%d, %d, %d], \"dofs\": %lld, \"levels\": %d, \"precision\": \"%s\", \"iterations\": %d, "
           "\"converged\": %d, \"relres\": %.6e, \"true_relres\": %.6e, \"solve_s\": %.6f, \"wall_s\": %.6f, "
           "\"compliance\": %.12e}\n",
           nx, ny, nz, (long long)(3 * nn), sgld_num_levels(ctx),
           precision == SGLD_PREC_MIXED ? "mixed" : precision == SGLD_PREC_MIXED_DF ? "mixed_df" : "fp64",
           info.iterations, info.converged, info.relres, info.true_relres, info.seconds, best, c);
    sgld_destroy(ctx);
    return info.converged ? 0 : 3;
}
