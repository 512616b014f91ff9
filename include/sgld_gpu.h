/*
 * sgld_gpu.h -- C ABI of the GB300 matrix-free voxel-elasticity MGPCG solver.
 *
 * This is the drop-in boundary for SGLDBench's solve path.  Every entry point
 * replaces one MATLAB function (or MEX kernel) of the reference; the citation
 * next to each declaration is that function's file:line in SGLDBench.  All
 * vectors cross the ABI in the reference's own layout:
 *
 *   - DOF vectors: numDOFs = 3 * numNodes doubles, node-major interleaved
 *     [ux uy uz] per node, nodes in the reference's compact order (the active
 *     nodes of the (resY+1) x (resX+1) x (resZ+1) node grid in column-major
 *     order, y fastest -- FEA_VoxelBasedDiscretization.m:71,218-222);
 *   - element vectors: numElements doubles in the reference's compact element
 *     order (eleMapBack, FEA_VoxelBasedDiscretization.m:200);
 *   - the voxel grid: resY x resX x resZ bytes, column-major, nonzero = solid
 *     (the padded voxelizedVolume_ of FEA_VoxelBasedDiscretization.m:163-186).
 *
 * Host buffers belong to the caller and are only read or written during the
 * call.  Functions with the _device suffix take device pointers (same compact
 * layout) and do not copy through the host.  Device memory belongs to the
 * context.  A context is not thread-safe; use one per host thread.
 *
 * Every entry point that touches the GPU first makes the context's device
 * (sgld_options.device) current, and leaves it current.  The element matrix
 * lives in constant memory, one copy per device shared by the contexts on it:
 * when a call reaches a context whose matrix (Poisson ratio, cell size,
 * sgld_set_ke) differs from the one held, the library waits for the device to
 * go idle and uploads the context's own.  Contexts of different materials on
 * one device may therefore be called in turn, but not from concurrent threads;
 * contexts of equal matrices may.
 *
 * Every function returns SGLD_OK (0) or an error code; sgld_last_error()
 * gives the message.  No exceptions cross the ABI.
 */
#ifndef SGLD_GPU_H
#define SGLD_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SGLD_OK 0
#define SGLD_ERR_ARG 1       /* invalid argument or size                     */
#define SGLD_ERR_CUDA 2      /* CUDA runtime failure                         */
#define SGLD_ERR_STATE 3     /* call out of order (e.g. solve before assemble) */
#define SGLD_ERR_NUMERIC 4   /* coarsest matrix not positive definite        */
#define SGLD_ERR_NOMEM 5     /* device allocation failed                     */

#define SGLD_PREC_FP64 0     /* reference form: FP64 PCG, FP64 additive V-cycle            */
#define SGLD_PREC_MIXED 1    /* FP64 flexible PCG outer, preconditioner = FP32 inner PCG with
                                the FP32 V-cycle; same tolerance on the FP64 true residual  */
#define SGLD_PREC_MIXED_DF 2 /* as SGLD_PREC_MIXED, with every outer K*u (K*p, warm-start
                                and exit residuals) in double-float arithmetic (FP32
                                pairs, ~2^-48 relative); FP64 vectors and dot products    */

typedef struct sgld_ctx sgld_ctx;

typedef struct sgld_options {
    int num_levels;        /* numLevels_ as produced by FEA_VoxelBasedDiscretization.m:169-177 */
    int non_dyadic;        /* nonDyadic_ (Data_GlobalVariables.m:15): first coarsening 4:1 if
                              set and num_levels >= 4 (Solving_BuildingMeshHierarchy.m:12-23) */
    double poisson_ratio;  /* poissonRatio_ (Data_GlobalVariables.m:20) */
    double cell_size;      /* cellSize_ (Data_GlobalVariables.m:22) */
    double omega;          /* weightFactorJacobi_ (Data_GlobalVariables.m:12) */
    int device;            /* CUDA device ordinal */
} sgld_options;

typedef struct sgld_solve_opts {
    double tol;            /* relative residual ||r||/||b|| to stop at (tol_) */
    int maxit;             /* iteration cap (maxIT_) */
    int use_x0;            /* 1: x holds the initial guess (Solving_CG_GMGS.m:7 warm start) */
    int precision;         /* SGLD_PREC_* */
    int inner_its;         /* SGLD_PREC_MIXED(_DF): initial cap on the FP32 inner CG iterations per
                              outer step (0 = 64); the cap doubles after an inner solve that stops
                              at it short of its tolerance, up to 16 inner_its.  With inner_tol
                              == 0 and inner_its > 0: exactly inner_its iterations, no doubling */
    double *history;       /* optional host buffer [maxit]: relative residual per iteration */
    int profile;           /* 1: time the K*u and preconditioner launches with CUDA events
                              (the SpMV / PtV split of QuickAccess/zTmp_Benchmarking_SpMV.m:63-111) */
    double inner_tol;      /* SGLD_PREC_MIXED(_DF): the inner CG of an outer step stops once its
                              FP32 residual is below max(inner_tol, tol / (2 relres)) times
                              the outer residual, relres = the outer relative residual so
                              far (inner_tol 0 = 3e-4 when inner_its == 0); decided on the
                              device */
} sgld_solve_opts;

typedef struct sgld_solve_info {
    int iterations;        /* outer iterations, as the reference's `its` */
    int converged;         /* SGLD_PREC_FP64: 1 if relres < tol, the reference's own stopping test
                              (Solving_PreconditionedConjugateGradientSolver.m:22).  Mixed modes:
                              1 only if true_relres <= tol as well */
    double relres;         /* recursive residual norm / ||b|| at exit */
    double true_relres;    /* ||b - K x|| / ||b|| recomputed at exit (FP64 vectors; K x by the
                              precision mode's outer operator) */
    int inner_iterations;  /* SGLD_PREC_MIXED(_DF): total FP32 inner CG iterations run */
    double seconds;        /* device time of the solve (CUDA events) */
    double kbyu_seconds;   /* profile: summed device time of the outer K*u launches */
    int kbyu_launches;     /* profile: number of those launches */
    double precond_seconds;/* profile: summed device time of the preconditioner applications */
    int fallback;          /* SGLD_PREC_MIXED(_DF): 1 if the mixed solve failed (not converged,
                              a non-finite residual, or a true residual still above tol after
                              its residual replacements) and the answer comes from the
                              reference-form FP64 solve rerun from the same start; the other
                              fields then describe that FP64 solve */
    int replacements;      /* SGLD_PREC_MIXED(_DF): residual replacements made.  When the
                              recurrence met tol but the recomputed true residual is above tol,
                              the outer PCG restarts from x with r = b - K x (at most 3 times);
                              their iterations are included in `iterations` and `seconds` */
} sgld_solve_info;

/* Test hook (no counterpart in the reference): corrupts, on the host side of
 * the next solve, data of a mixed solve so that its failure handling runs.
 * kind 1: the FP32 copy of the moduli gets a NaN (until the next
 * sgld_assemble), so the mixed solve fails and its FP64 fallback runs.
 * kind 2: the next single-load mixed solve's iterate is scaled by (1 + 1e-3)
 * after its recurrence has met tol, as a drifted recurrence would leave it, so
 * its true residual is above tol and residual replacement runs.  kind 0:
 * no-op.  Faults no GPU. */
int sgld_inject_fault(sgld_ctx *ctx, int kind);

/* The CUDA stream every call of this context runs on (a cudaStream_t).  No
 * counterpart in the reference, whose solve runs on the host: it lets a caller
 * order its own device work after the library's. */
void *sgld_get_stream(const sgld_ctx *ctx);

/* Number of CUDA kernels this library has launched from the calling thread
 * (a host-side counter, one per kernel, graph nodes included; no counterpart
 * in the reference, used for accounting). */
int64_t sgld_kernel_launches(void);

/* Times `reps` back-to-back applications of one internal operator on the
 * context's own (already set up) device buffers with CUDA events and returns
 * the mean milliseconds per application.  No counterpart in the reference:
 * it is the kernel-level measurement hook used for rooflines and profiling.
 *   op 0: FP64 K*u   op 1: FP32 K*u   op 2: FP64 V-cycle   op 3: FP32 V-cycle
 *   op 4: assembly (Galerkin levels + coarsest factorization)
 *   op 5: double-float K*u (the outer operator of SGLD_PREC_MIXED_DF) */
int sgld_time_op(sgld_ctx *ctx, int op, int reps, double *ms_per_op);

/* The tile of the FP32 K*u on the finest level: x width in elements (8 or 16)
 * and node layers per CTA, as chosen by the autotuner at the first
 * sgld_assemble (or the defaults before it / with SGLD_AUTOTUNE=0).  No
 * counterpart in the reference; reported beside measurements. */
int sgld_kbyu_tile(const sgld_ctx *ctx, int *tile_x, int *z_chunk);

/* Allocation-free K*u with its dot product (no counterpart in the reference).
 *
 * For callers that must not allocate device memory when they apply the
 * operator: a real-time loop whose device memory budget is fixed at start-up,
 * or a plugin in a process whose device memory belongs to another framework's
 * caching allocator.  Enqueues,
 * on `stream` (a cudaStream_t; NULL = the legacy default stream),
 *     d_y = K d_u (fixed DOFs of d_y set to 0)   and   *d_dot = d_u . d_y,
 * for the context's current moduli.  d_u and d_y are device arrays in the
 * full-grid layout: 3 * (resY+1) * (resX+1) * (resZ+1) doubles, node-major,
 * nodes in column-major grid order, zeros at inactive nodes; d_dot is one
 * device double.  The call allocates nothing: its scratch is a static device
 * array of SGLD_NOALLOC_MAX_CTAS doubles (256 KiB) that every GPU loading this
 * library holds until the process exits.  The first call on a device looks up
 * that array's address (once per device, the context's device must be
 * current).  Every call shares the array, so calls that overlap on the GPU
 * (other streams, other contexts on the same device) race; serialise them.
 * The call uploads no constants: if the device holds another context's
 * element matrix, it returns SGLD_ERR_STATE, and any other call on this
 * context binds the matrix again.  Grids needing more than
 * SGLD_NOALLOC_MAX_CTAS CTAs (on the order of 1e8 nodes; each CTA covers a
 * 31 x 7 x 16 node block) are rejected with SGLD_ERR_ARG. */
#define SGLD_NOALLOC_MAX_CTAS 32768
int sgld_kbyu_dot_noalloc(sgld_ctx *ctx, const double *d_u, double *d_y, double *d_dot, void *stream);

/* Fills opts with the reference defaults (Data_GlobalVariables.m:10-23). */
void sgld_default_options(sgld_options *opts);

/* Number of levels FEA_VoxelBasedDiscretization.m:163-177 derives for a voxel
 * count and coarsestResolutionControl_ (before the nonDyadic adjustment). */
int sgld_reference_num_levels(int64_t num_voxels, int64_t coarsest_resolution_control);

/* Builds the grid hierarchy for a padded voxel grid.  Replaces
 * FEA_VoxelBasedDiscretization.m:188-226 (element/node numbering) and
 * Solving_BuildingMeshHierarchy.m:9-165 (coarse levels). */
int sgld_create(int resY, int resX, int resZ, const uint8_t *solid, const sgld_options *opts, sgld_ctx **out);
void sgld_destroy(sgld_ctx *ctx);
/* Solving_BuildingMeshHierarchy.m:1-175 as a call of its own: rebuilds the
 * context's coarse levels for num_levels / non_dyadic (the numLevels_ and
 * nonDyadic_ globals it reads) from the context's own voxel grid, keeping
 * its material, omega and any Ke set by sgld_set_ke.  As after sgld_create,
 * fixed DOFs, moduli and passive elements must then be set again.  On error
 * the context is unchanged. */
int sgld_build_hierarchy(sgld_ctx *ctx, int num_levels, int non_dyadic);
const char *sgld_last_error(const sgld_ctx *ctx);

/* Sizes of level `level` (1 = finest, as meshHierarchy_(level)): resY/resX/resZ,
 * spanWidth, numElements and numNodes as FEA_VoxelBasedDiscretization.m:56-82
 * (level 1) and Solving_BuildingMeshHierarchy.m:24-34,104-122 set them; the
 * level count is numLevels_ (Solving_BuildingMeshHierarchy.m:13). */
int sgld_level_info(const sgld_ctx *ctx, int level, int res_yxz[3], int *span, int64_t *num_elements,
                    int64_t *num_nodes);
int sgld_num_levels(const sgld_ctx *ctx);
/* 1-based full-grid indices of the compact nodes / elements of a level
 * (nodMapBack / eleMapBack of that level, in that level's own grid:
 * FEA_VoxelBasedDiscretization.m:63,81, Solving_BuildingMeshHierarchy.m:104,122). */
int sgld_node_map(const sgld_ctx *ctx, int level, int64_t *map);
int sgld_element_map(const sgld_ctx *ctx, int level, int64_t *map);

/* Element stiffness matrix Ke (24 x 24, column-major).  sgld_create computes it
 * as FEA_VoxelBasedElementStiffnessMatrix.m:10-23 does; set_ke replaces it
 * (it must have the isotropic hexahedral structure). */
int sgld_get_ke(const sgld_ctx *ctx, double *Ke);
int sgld_set_ke(sgld_ctx *ctx, const double *Ke);

/* Fixed-DOF mask (numDOFs bytes, nonzero = fixed): meshHierarchy_(1).fixedDOFs of
 * FEA_ApplyBoundaryCondition.m:37-41; also derives the coarse masks as
 * FEA_SetupVoxelBased.m:13-26 does. */
int sgld_set_fixed_dofs(sgld_ctx *ctx, const uint8_t *fixed);
/* Coarse-level free-DOF mask of `level` (numDOFs of that level): meshHierarchy_(level).freeDOFs
 * of FEA_SetupVoxelBased.m:13-19 as a mask. */
int sgld_get_free_dofs(const sgld_ctx *ctx, int level, uint8_t *free_mask);

/* Element moduli (numElements): meshHierarchy_(1).eleModulus
 * (TopOpti_MaterialInterpolationSIMP.m:5). */
int sgld_set_modulus(sgld_ctx *ctx, const double *E);
int sgld_set_modulus_device(sgld_ctx *ctx, const double *d_E);

/* Solving_AssembleFEAstencil.m:7-135: Galerkin coarse element matrices, Jacobi
 * diagonals, coarsest-level factorization. */
int sgld_assemble(sgld_ctx *ctx);
/* Jacobi diagonal diagK of `level` (1..L-1), compact numDOFs (Solving_AssembleFEAstencil.m:24-96). */
int sgld_get_diag(const sgld_ctx *ctx, int level, double *diag);
/* Galerkin element matrices Ks of coarse `level` (2..L), 24 x 24 x numElements
 * (Solving_AssembleFEAstencil.m:33-58). */
int sgld_get_ks(const sgld_ctx *ctx, int level, double *Ks);

/* Solving_KbyU_MatrixFree.m:1-41 (Solving_KbyU_MatrixFree_mex.cpp:6-138): y = K u,
 * y(fixedDOFs) = 0. */
int sgld_kbyu(sgld_ctx *ctx, const double *u, double *y);
int sgld_kbyu_device(sgld_ctx *ctx, const double *d_u, double *d_y);
/* The same product in double-float arithmetic (the outer K*p of
 * SGLD_PREC_MIXED_DF); no counterpart in the reference, exposed so that its
 * accuracy against the FP64 operator can be checked. */
int sgld_kbyu_df(sgld_ctx *ctx, const double *u, double *y);

/* Solving_RestrictResidual.m:1-23 / Solving_InterpolationDeviation.m:1-23 for
 * MATLAB level index ii (2..L): coarse = R fine, fine = P coarse (compact DOFs). */
int sgld_restrict(sgld_ctx *ctx, int ii, const double *r_fine, double *r_coarse);
int sgld_interpolate(sgld_ctx *ctx, int ii, const double *x_coarse, double *x_fine);

/* Solving_Vcycle.m:1-52: z = M^-1 r (additive multilevel Jacobi + coarsest solve). */
int sgld_vcycle(sgld_ctx *ctx, const double *r, double *z);

/* K*u and the V-cycle at a chosen precision (SGLD_PREC_*), the operators the
 * solve modes use: FP64 (the reference form; = sgld_kbyu / sgld_vcycle);
 * SGLD_PREC_MIXED: K*u in FP32 on FP32 copies of u and the moduli, the FP32
 * V-cycle; SGLD_PREC_MIXED_DF: K*u in double-float (= sgld_kbyu_df), the FP32
 * V-cycle.  Inputs and outputs stay FP64 compact vectors. */
int sgld_kbyu_prec(sgld_ctx *ctx, const double *u, double *y, int precision);
int sgld_vcycle_prec(sgld_ctx *ctx, const double *r, double *z, int precision);
/* The restriction the FP32 V-cycle applies (SGLD_PREC_MIXED / _MIXED_DF: FP32
 * copy of r_fine, FP32 sums) or sgld_restrict (SGLD_PREC_FP64); level index ii
 * as sgld_restrict. */
int sgld_restrict_prec(sgld_ctx *ctx, int ii, const double *r_fine, double *r_coarse, int precision);

/* Solving_PreconditionedConjugateGradientSolver.m:1-37 with AtX = KbyU and
 * PtV = Vcycle (as Solving_CG_GMGS.m:7 binds them).  x: in = initial guess when
 * opts->use_x0, out = solution. */
int sgld_pcg(sgld_ctx *ctx, const double *b, double *x, const sgld_solve_opts *opts, sgld_solve_info *info);

/* Block right-hand side: the same solve for nrhs load cases sharing one
 * assembly (the reference solves its load cases one after another through
 * Solving_CG_GMGS.m:7).  F and U hold nrhs compact DOF vectors back to back
 * (case j at offset j * numDOFs); U holds the initial guesses when
 * opts->use_x0.  info, if not NULL, receives nrhs entries.  In the mixed
 * precision modes the whole block is one CUDA-graph launch (per case: the
 * outer flexible PCG and the inner FP32 CG as device-side while loops, so no
 * host round trip between iterations or cases); info[j].seconds is the
 * block's device time / nrhs.  In FP64 the cases are solved one after
 * another. */
int sgld_solve_block(sgld_ctx *ctx, int nrhs, const double *F, double *U, const sgld_solve_opts *opts,
                     sgld_solve_info *info);
/* Solving_CG_GMGS.m:1-9 for nrhs load cases with plain arguments: sgld_solve_block
 * from U = 0 with tol, maxit and precision; its[j] and relres[j] (either may be
 * NULL) receive case j's iteration count and relative residual, as the
 * reference's `its` and the final ||r||/||b||. */
int sgld_solve(sgld_ctx *ctx, int nrhs, const double *F, double *U, double tol, int maxit, int precision, int *its,
               double *relres);
int sgld_pcg_device(sgld_ctx *ctx, const double *d_b, double *d_x, const sgld_solve_opts *opts,
                    sgld_solve_info *info);

/* TopOpti_ComputeUnitCompliance.m:1-21 (TopOpti_CmptUnitCompliance_mex.cpp:6-107):
 * ce = u_e' Ke u_e per element; c = sum(E .* ce) (FEA_ComputeComplianceVoxel.m:20-22).
 * ce may be NULL. */
int sgld_compliance(sgld_ctx *ctx, const double *U, double *ce, double *c);

/* Cone density filter (TopOpti_PerformDensityFiltering_mex.cpp:8-52; with x ==
 * NULL the weight sums Hs of TopOpti_SetupDensityFilter_mex.cpp:9-51):
 * y_e = sum over solid e2 in the (2 ceil(rmin) - 1)^3 box of max(0, rmin - |e - e2|) x_e2.
 * Compact element vectors (numElements). */
int sgld_density_filter(sgld_ctx *ctx, double rmin, const double *x, double *y);

/* PDE (Helmholtz) density filter of an element field x (numElements):
 * TopOpti_PDEFiltering_matrixFree.m:1-36 with the element matrix of
 * TopOpti_BuildPDEfilter_matrixFree.m:9-20 for rHatMin = rhat -- the field is
 * spread to the nodes, K_pde t = src is solved by the reference's PCG with a
 * Jacobi preconditioner to relative residual tol (at most maxit iterations),
 * and t is averaged back to the elements into y.  *iterations (may be NULL)
 * receives the PCG iteration count. */
int sgld_pde_filter(sgld_ctx *ctx, double rhat, const double *x, double *y, double tol, int maxit, int *iterations);

/* MMA_mex.cpp:6-54 (Svanberg's MMA as in MMAseq.cpp; a fresh solver per call,
 * as the MEX gateway makes it): one update of n design variables under m
 * constraints, same arguments and outputs as the gateway (dfdx holds m*n
 * values, variable-major).  The subproblem's dual interior-point iteration
 * runs over device passes.  Only m = 1 (the reference's volume constraint)
 * is supported; other m return SGLD_ERR_ARG.  xold1_out = xval and
 * xold2_out = xold1, as MMAseq::Update sets them. */
int sgld_mma_update(sgld_ctx *ctx, int m, int n, const double *xval, const double *xmin, const double *xmax,
                    const double *xold1, const double *xold2, const double *df0dx, const double *fval,
                    const double *dfdx, double *xnew, double *xold1_out, double *xold2_out);

/* SIMP loop with a global volume constraint (TopOpti_GlobalVolumeConstraint_Tmp.m:26-120,
 * ft = 2): per iteration E = SIMP(xPhys), assembly, warm-started MGPCG, unit
 * compliance, sensitivities, filtered sensitivities, OC bisection on the
 * linearised volume constraint, filtered densities.  Defaults (0 fields) follow
 * Data_GlobalVariables.m / the reference. */
typedef struct sgld_topopt_opts {
    double volfrac;        /* V_ */
    double rmin;           /* rMin_ */
    double move;           /* move_ (0 = 0.1) */
    int n_loop;            /* nLoop_ */
    double min_change;     /* minChange_ (0 = 1e-4) */
    double max_sharpness;  /* maxSharpness_ (0 = 0.05) */
    double penalty;        /* SIMPpenalty_ (0 = 3) */
    double E0, Emin;       /* modulus_, modulusMin_ (0 = 1, 1e-6) */
    sgld_solve_opts solve; /* tol_, maxIT_, precision of every MGPCG solve (warm-started) */
    int optimizer;         /* SGLD_OPT_OC (0, the loop's bisection) or SGLD_OPT_MMA (1: the
                              MMA update of TopOpti_GlobalVolumeConstraint.m:139-156, one
                              volume constraint, passive elements excluded from the variables) */
    /* Learned warm start (no counterpart in the reference, which warm-starts
     * every solve from the previous displacement U, Solving_CG_GMGS.m:7).
     * With learned = 1 a U-Net (sgld_net_*) on the node grid of level
     * net_level is trained online on this loop's own solves: input the
     * restricted initial residual, the previous displacement change d, a
     * log-modulus field and the active-node mask; target the direction of the
     * displacement change the solve is about to find.  Its output v,
     * prolongated to the finest grid, and d span the correction: the start is
     * U + a d + b v with (a, b) minimising the energy error (a 2x2 Galerkin
     * system), kept only if it lowers the residual in the norm of the FP64
     * V-cycle M (r'Mr, which tracks the error's energy).  learned = 2 uses d
     * alone (the same method without the network, for comparison).  The
     * converged answer is the plain solve's: only iteration counts change. */
    int learned;           /* 0 off, 1 network + previous change, 2 previous change only */
    int net_level;         /* MATLAB level index of the network's grid (0 = 3, clamped to [1, levels]) */
    int net_train_steps;   /* Adam steps after each solve (0 = 4) */
    float net_lr;          /* Adam learning rate (0 = 1e-3) */
    /* Checkpoint / resume (no counterpart in the reference's global loop, which
     * cannot resume).  A loop stopped after k iterations and restarted with
     * x0 = its design x (x_out), xphys0 = its xPhys, U0 = its displacement
     * and loop0 = k runs the same iterations k+1.. as an uninterrupted loop,
     * bit for bit (the OC and MMA updates keep no state between iterations;
     * a learned warm start, if on, starts a fresh network). */
    const double *xphys0;  /* NULL: xPhys starts as x (TopOpti_CallTopOpti.m); else numElements */
    const double *U0;      /* NULL: U = 0; else numDOFs, the warm start of the first solve */
    int loop0;             /* iterations already run: numbering continues, n_loop is the total */
    double *x_out;         /* NULL or numElements: the final design variables x */
} sgld_topopt_opts;

#define SGLD_OPT_OC 0
#define SGLD_OPT_MMA 1

/* Passive elements (passiveElements_, IO_ImportTopVoxels.m:76-80): n compact
 * 0-based element indices kept solid by the SIMP loop (x = xPhys = 1,
 * TopOpti_GlobalVolumeConstraint.m:162,179).  n = 0 clears the set. */
int sgld_set_passive(sgld_ctx *ctx, int64_t n, const int64_t *elements);

typedef struct sgld_topopt_iter {
    int loop, cg_iterations;
    double compliance, volume, sharpness, change, constraint;   /* cHist_, volHist_, sharpHist_, change, consHist_ */
    double t_assemble, t_solve, t_opt, t_filter;                 /* tHist_ columns (device seconds) */
    /* learned warm start (zero when it is off or has no model yet) */
    int net_used;          /* the network proposed a guess this iteration */
    int net_accepted;      /* ... and it lowered the initial residual, so the solve started from it */
    double net_r0_ratio;   /* sqrt(r1'M r1 / r0'M r0), r1 = F - K u_start, r0 = F - K U (the step taken) */
    double ext_r0_ratio;   /* the same for the previous change d alone (without the network) */
    double net_loss;       /* training loss of the last Adam step after the solve */
    double t_net;          /* device seconds of the network's guess and training */
    int inner_iterations;  /* inner FP32 CG iterations of the solve (mixed precision; 0 for FP64) */
} sgld_topopt_iter;

/* x0: initial design (NULL = volfrac everywhere, TopOpti_CallTopOpti.m:34);
 * xphys: final filtered design (numElements); hist: n_loop - loop0 records;
 * *n_iter: iterations run by this call.  Leaves the last displacement in the
 * context (sgld_topopt_displacement reads it). */
int sgld_topopt(sgld_ctx *ctx, const sgld_topopt_opts *opts, const double *F, const double *x0, double *xphys,
                sgld_topopt_iter *hist, int *n_iter);

/* The displacement the last SIMP loop ended with (numDOFs), e.g. for a checkpoint: the
 * global U_ that the next Solving_CG_GMGS.m:7 would warm-start from. */
int sgld_topopt_displacement(sgld_ctx *ctx, double *U);

/* The projected SIMP loops with MMA, compliance normalised by the solid
 * domain's, density filter (rmin) and Heaviside projection (beta, eta) of the
 * design, one MMA update per iteration (passive elements excluded and kept
 * solid), beta doubling up to beta_max, and the sensitivity penalty raised by
 * penalty_increment every penalty_interval iterations (capped at 3):
 *   SGLD_CONS_LOCAL:  TopOpti_LocalVolumeConstraint.m:33-269 (porous infill):
 *       the p-norm of the PDE-filtered (radius rhat) local volume fraction is
 *       held below alpha (Initialize4GradedPorosity with alphaMax_ = alphaMin_);
 *       x starts at alpha (TopOpti_CallTopOpti.m:41-45); beta doubles every
 *       beta_interval iterations;
 *   SGLD_CONS_VOLUME: TopOpti_GlobalVolumeConstraint.m:50-228 with
 *       optimizer_ = 'MMA': sum(xPhys) <= volfrac numElements; x starts at
 *       volfrac (TopOpti_CallTopOpti.m:34-38); beta doubles every
 *       beta_interval iterations or once change <= 1e-3.
 * hist records use constraint = fval of the MMA constraint. */
#define SGLD_CONS_LOCAL 0
#define SGLD_CONS_VOLUME 1

typedef struct sgld_topopt_projected_opts {
    int constraint;           /* SGLD_CONS_LOCAL or SGLD_CONS_VOLUME */
    double volfrac;           /* V_ (SGLD_CONS_VOLUME) */
    double rmin;              /* rMin_ */
    double rhat;              /* rHatMin_ (0 = 8) */
    double alpha;             /* alphaMin_ (0 = 0.5) */
    double pnorm;             /* p_ (0 = 16) */
    double move;              /* move_ (0 = 0.1) */
    int n_loop;               /* nLoop_ */
    double min_change;        /* minChange_ (0 = 1e-4) */
    double max_sharpness;     /* maxSharpness_ (0 = 0.05) */
    double simp_penalty;      /* SIMPpenalty_ of the modulus (0 = 3) */
    double penalty;           /* penalty_ of the sensitivity, continued (0 = 3) */
    double penalty_increment; /* penaltyIncrement_ */
    int penalty_interval;     /* penaltyUpdateIterations_ (0 = no continuation) */
    double beta, eta;         /* beta_ (0 = 1), eta_ (0 = 0.5) */
    double beta_max;          /* pMax_ (0 = 128) */
    int beta_interval;        /* iterations between beta doublings (0 = 40) */
    double E0, Emin;          /* modulus_, modulusMin_ (0 = 1, 1e-6) */
    sgld_solve_opts solve;    /* tol_, maxIT_, precision of the MGPCG solves; tol_ and maxIT_ also
                                 drive the PDE filter's PCG (TopOpti_PDEFiltering_matrixFree.m:23) */
} sgld_topopt_projected_opts;

int sgld_topopt_projected(sgld_ctx *ctx, const sgld_topopt_projected_opts *opts, const double *F, double *xphys,
                          sgld_topopt_iter *hist, int *n_iter);

/* FEA_StressAnalysis.m:17-60 and FEA_ComputePerElementVonMisesStress.m:10-19:
 * nodal Cartesian stress (numNodes x 6, row-major [xx yy zz yz zx xy]), nodal
 * von Mises and per-element von Mises with the reference's final .^(1/2).
 * Any output may be NULL. */
int sgld_stress(sgld_ctx *ctx, const double *U, double *nodal_stress, double *vm_node, double *vm_elem);
/* The von Mises part of sgld_stress alone (FEA_ComputePerElementVonMisesStress.m:10-19,
 * FEA_ComputeVonMisesStress.m:1-7): per element (numElements) and per node
 * (numNodes); either may be NULL. */
int sgld_vonmises(sgld_ctx *ctx, const double *U, double *vm_elem, double *vm_node);

/* Principal stresses of the nodal Cartesian stress field of U
 * (FEA_ComputePrincipalStress.m:1-8 per node): ps_node is numNodes x 12,
 * row-major [l1 v1(3) l2 v2(3) l3 v3(3)] with l1 <= l2 <= l3 and each unit
 * eigenvector signed so that its entry of largest magnitude is positive.
 * dir_elem (numElements x 3, row-major): per element, the principal direction
 * of largest |l| of the centroid stress
 * (Common_ExtractDominantDirectionsFromPrincipalStressDirections.m:9-38).
 * Either output may be NULL. */
int sgld_principal_stress(sgld_ctx *ctx, const double *U, double *ps_node, double *dir_elem);

/* ---- the learned warm start's network on its own ------------------------------
 * No counterpart in the reference.  A 3D convolutional U-Net on a node grid
 * (ny, nx, nz), tensors channels-last [v][c] with v = y + ny (x + nx z):
 *   encoder level l: relu(conv3) twice, then 2x average pooling (ceil);
 *   decoder level l: relu(conv3) on level l+1 to w_l channels, nearest 2x
 *   upsampling plus the encoder's level-l output, relu(conv3);
 *   head: linear 1x1x1 convolution to out_channels (FP32 output).
 * Activations and weights are BF16 on the device, every product accumulates
 * in FP32, the master weights and Adam moments are FP32.  Parameters, per
 * convolution W[taps][cin][cout] then b[cout], convolutions in the order
 * a_0, b_0, .., a_{L-1}, b_{L-1}, u_{L-2}, m_{L-2}, .., u_0, m_0, head.
 * levels in [1, 4]; widths NULL = {16, 32, 48, 64}; channel counts are
 * multiples of 4 up to 64 (in_channels too).  The network lives on the device
 * current at sgld_net_create, with its own CUDA stream there; every later call
 * makes that device current again. */
typedef struct sgld_net sgld_net;

int sgld_net_create(int ny, int nx, int nz, int in_channels, int out_channels, int levels, const int *widths,
                    unsigned long long seed, sgld_net **out);
void sgld_net_destroy(sgld_net *net);
const char *sgld_net_last_error(const sgld_net *net);
int64_t sgld_net_num_params(const sgld_net *net);
int sgld_net_get_params(sgld_net *net, float *params);
/* also resets the Adam moments and step count (no reference counterpart, as for
 * every sgld_net_* call) */
int sgld_net_set_params(sgld_net *net, const float *params);
/* x [V][in_channels] (rounded to BF16 on upload) -> y [V][out_channels]; no reference
 * counterpart */
int sgld_net_forward(sgld_net *net, const float *x, float *y);
/* loss = sum_v mask_v |y_v - target_v|^2 / (out_channels sum_v mask_v) (mask NULL = 1)
 * and its gradient with respect to every parameter (grad may be NULL); no reference
 * counterpart */
int sgld_net_grad(sgld_net *net, const float *x, const float *target, const float *mask, double *loss,
                  float *grad);
/* sgld_net_grad followed by one Adam step (beta 0.9, 0.999, eps 1e-8); loss before the
 * step; no reference counterpart */
int sgld_net_train_step(sgld_net *net, const float *x, const float *target, const float *mask, float lr,
                        double *loss);

/* ---- learned start for a sequence of load cases on one model -----------------
 * No counterpart in the reference, which solves every new load case from
 * U_ = 0 (Solving_CG_GMGS.m:7; GUIs/Mtd_StructuralRobustnessExploration.m:119
 * re-solves per rotated load).  The object learns from the solves it is given
 * for training: a K-orthonormal basis of their solutions (FP64, compact DOF
 * order, at most max_basis <= 32 vectors) and, with net_level >= 0, a U-Net on a
 * coarse level trained on (residual left by the basis start -> correction the
 * solve found) pairs.  A new case starts from the energy-optimal combination of
 * the basis, plus the network's correction when that lowers r'Mr (M = the FP64
 * V-cycle).  The solve then runs to its tolerance on the true residual like any
 * other, so the start changes iteration counts, never the converged answer.
 * net_level: MATLAB level index of the network's grid, 0 = the finest level of
 * at most 110K nodes, -1 = no network.  train_steps: Adam steps per training
 * case.  Memory: max_basis * numDOFs * 8 bytes plus four full-grid FP64 vectors.
 * Destroy it before its context. */
typedef struct sgld_cases sgld_cases;

typedef struct sgld_cases_stats {
    int diagnostics;     /* in: 1 = also measure the starts' sqrt(r'Mr) ratios (two FP64 V-cycles) */
    int basis;           /* basis vectors the start was formed from */
    int net_used;        /* the network's correction was evaluated ... */
    int net_accepted;    /* ... and kept (it lowered r'Mr) */
    double net_ratio;    /* sqrt(r'Mr) with the kept correction / without it */
    double basis_ratio;  /* diagnostics: sqrt(r'Mr) of the basis start / of the zero start */
    double start_ratio;  /* diagnostics: the same for the start used */
    double net_loss_before;  /* train: loss on this case's sample before its Adam steps */
    double net_loss;     /* train: loss on this case's sample after them */
    double t_start;      /* device seconds forming the start (CUDA events) */
    double t_solve;      /* device seconds of the solve */
    double t_train;      /* device seconds adding the case to the basis and training */
} sgld_cases_stats;

int sgld_cases_create(sgld_ctx *ctx, int max_basis, int net_level, int train_steps, sgld_cases **out);
void sgld_cases_destroy(sgld_cases *cases);
int sgld_cases_basis_size(const sgld_cases *cases);
/* Solves one load case (F, U: compact host vectors as sgld_pcg) with the
 * context's assembled stencil and opts (use_x0 is ignored).  mode 0: zero start;
 * 1: the basis start; 2: the basis start and the network's correction.  train:
 * afterwards add the solution to the basis and train the network on the case. */
int sgld_cases_solve(sgld_cases *cases, const double *F, double *U, const sgld_solve_opts *opts, int mode,
                     int train, sgld_solve_info *info, sgld_cases_stats *stats);
/* the same with compact device vectors */
int sgld_cases_solve_device(sgld_cases *cases, const double *d_F, double *d_U, const sgld_solve_opts *opts,
                            int mode, int train, sgld_solve_info *info, sgld_cases_stats *stats);

#ifdef __cplusplus
}
#endif
#endif /* SGLD_GPU_H */
