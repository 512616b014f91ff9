// Internal declarations shared by the CUDA translation units of the GB300
// MGPCG voxel-elasticity solver.  Nothing here crosses the C ABI.
//
// Device data layout (every level, every vector):
//   * structured full grid: elements (ny, nx, nz), nodes (ny+1, nx+1, nz+1),
//     linear index y + NY*(x + NX*z) with y fastest -- the reference's own
//     column-major node numbering (src/FEA_VoxelBasedDiscretization.m:71),
//     so the reference's compact numbering is this order with the inactive
//     nodes removed;
//   * nodal vectors node-major interleaved: v[3*node + c], c = x, y, z;
//   * inactive nodes hold exact zeros, inactive elements have modulus 0.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace sgld {

// NVTX range for the phases of a call (assembly, solves, SIMP iterations);
// free unless a profiler is attached
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// node flag bits
enum : uint8_t { NF_ACTIVE = 1, NF_FIXX = 2, NF_FIXY = 4, NF_FIXZ = 8 };

// The isotropic hexahedral element matrix in the 8-corner Hadamard basis has
// 45 nonzeros in 11 symmetric blocks (index = 3*mode + component, mode bits:
// bit0 = x/s, bit1 = y/t, bit2 = z/p).  KH_BLOCKS lists the blocks; the values
// sit in constant memory in the same order (row-major within each block).
constexpr int KH_NNZ = 45;

struct Level {
    int nx = 0, ny = 0, nz = 0;   // elements
    int span = 1;                 // coarsening factor from the next finer level
    int kx_zc = 0;                // node layers per z stream of the FP32 K*u, two streams per CTA
                                  // (0 = default rule; set by the tuner)
    int kx_tx = 0;                // x width of the FP32 K*u tile, 8 or 16 (0 = 8; set by the tuner)
    bool kh_cubic = false;        // finest level: the bound element matrix has the hexahedron's
                                  // cubic symmetry (kh_cubic), so the FP32 K*u takes its 8-value form
    int64_t nel = 0, nnode = 0;   // full-grid counts
    int64_t nel_active = 0, nnode_active = 0;
    uint8_t *eact = nullptr;      // [nel] element non-empty
    // active-tile maps of the finest level's K*u launches (one byte per CTA:
    // 0 = no active element in the CTA's element box, so every node it owns
    // is inactive and its result is zero): the 32 x 8 x 16-layer grid of the
    // FP64 and double-float kernels, and the FP32 kernel's grid for the tile
    // (tiles_f32_tx, tiles_f32_zc) it was made for
    uint8_t *tiles16 = nullptr, *tiles_f32 = nullptr;
    // finest level: the words of the active nodes as chunks of contiguous
    // floats (runs of active nodes along y, gaps of a few nodes bridged), each
    // first DOF | floats << 40, in address order; empty when nearly every node
    // is active (then the flat kernels run)
    int64_t *runs = nullptr;
    int64_t nruns = 0;
    int tiles_f32_tx = 0, tiles_f32_zc = 0;
    // finest level: set to 1 by an FP32 K*u CTA that gave up waiting for its
    // staged node rows (the CTA writes NaN to the nodes it owns)
    int *kerr = nullptr;
    int64_t tiles_f32_cap = 0;
    uint8_t *nflag = nullptr;     // [nnode] NF_* bits
    double *diag = nullptr;       // [3*nnode] Jacobi diagonal (levels 1..L-1)
    double *idiag = nullptr;      // [3*nnode] 1 / diag on active nodes, 0 elsewhere
    float *idiag32 = nullptr;
    double *Ks = nullptr;         // [576*nel] Galerkin element matrices (coarse levels)
    double *r = nullptr, *x = nullptr;      // [3*nnode] V-cycle work (coarse levels)
    float *r32 = nullptr, *x32 = nullptr;
    std::vector<uint8_t> h_eact, h_nflag;
};

struct Ctx {
    int L = 0;
    int non_dyadic = 0;
    std::vector<Level> lv;
    double nu = 0.3, cell = 1.0;
    double omega = 0.35;
    double Ke[576];       // column-major 24x24, reference DOF order
    double Kh[KH_NNZ];
    // finest-level compact <-> full maps (host + device)
    std::vector<int64_t> h_nodemap, h_elemap;   // compact -> full (0-based)
    int64_t *d_nodemap = nullptr, *d_elemap = nullptr;
    double *E = nullptr;            // [nel] modulus on the full grid (0 = void)
    bool have_fixed = false, have_E = false, assembled = false;
    // coarsest direct solve
    int ncf = 0;                    // free DOFs on the coarsest level
    int cband = 0;                  // half bandwidth of the permuted coarse matrix
    int *d_cfree = nullptr;         // [ncf] full-grid DOF index (3*node + c), permuted order
    double *d_Ac = nullptr;         // [ncf*ncf] dense matrix / Cholesky factor
    double *d_Ainv = nullptr;       // [ncf*ncf] inverse (symmetric)
    float *d_Ainv32 = nullptr;
    double *d_LB = nullptr;         // [ncf*(cband+1) + ncf + ceil(ncf/32)*1024] doubles holding the
                                    // Cholesky band, 1/diag and the diagonal-block inverses as
                                    // float pairs (hi, lo arrays)
    double *d_cy = nullptr;         // [2*ncf] intermediate of the coarse apply
    // SIMP loop fields on the finest element grid (allocated on first use)
    double *t_x = nullptr, *t_xp = nullptr, *t_hs = nullptr, *t_ce = nullptr, *t_dcs = nullptr, *t_dvs = nullptr,
           *t_dc = nullptr, *t_dv = nullptr, *t_q = nullptr, *t_tmp = nullptr, *t_st = nullptr;
    double t_rmin = -1.0;
    double *t_pde = nullptr;   // [7 nnode] PDE-filter PCG work (finest nodes, one value each)
    double *t_fw = nullptr;    // [7^3] density-filter weights of the last radius
    double *t_kp = nullptr;    // [64] PDE-filter element matrix of the last radius
    cudaGraphExec_t factor_graph = nullptr;   // captured factorization of the coarsest matrix
    int64_t factor_graph_launches = 0;
    int trinv_ring = 0;
    int trinv_g = 16;               // columns per CTA of the L^-1 sweeps (narrower for wide bands)
    size_t trinv_smem = 0;
    bool m64_valid = false;         // d_Ainv holds L^-1 of the current factorization (made on first use)
    double *d_cpart = nullptr;      // [CSPLIT*ncf] GEMV partials
    // templates for the level-2 Galerkin assembly
    double *d_H = nullptr;          // [2 (8 + 64) * 576] templates for span 2, span 4, then both as
                                    // (hi, lo) float pairs
    // PCG vectors (full grid, FP64)
    double *d_b = nullptr, *d_x = nullptr, *d_r = nullptr, *d_z = nullptr, *d_p = nullptr, *d_q = nullptr;
    double *d_tmp = nullptr;
    double *d_part = nullptr;       // reduction partials
    double *d_scal = nullptr;       // device scalars
    int *d_iflag = nullptr;         // device int scalars (iteration, done)
    int npart = 0;
    // mixed-precision work
    float *d_r32 = nullptr, *d_z32 = nullptr, *d_E32 = nullptr;
    float *d_e32 = nullptr, *d_s32 = nullptr, *d_d32 = nullptr, *d_t32 = nullptr;
    double *d_part2 = nullptr;      // second partial-sum buffer
    double *d_isc = nullptr;        // inner CG scalars
    cudaStream_t aux[3] = {nullptr, nullptr, nullptr};   // capture streams of conditional bodies
    // whole mixed-precision solves of a block of load cases as one graph
    // (outer and inner loops as device-side while nodes), cached by its key
    cudaGraphExec_t solve_graph = nullptr;
    std::vector<double> solve_key;
    int64_t sg_fixed = 0, sg_outer = 0, sg_if = 0, sg_inner = 0;   // launches per part
    double *d_blk = nullptr;   // [2 nrhs numDOFs] compact F and U of the block
    double *d_binfo = nullptr; // [8 nrhs] per-case results
    int blk_cap = 0;
    bool kbyu_tuned = false;   // the FP32 K*u z-chunk was tuned (tune_kbyu_f32)
    std::vector<int64_t> h_passive;   // passive elements (full-grid indices, sorted) of the SIMP loop
    cudaGraphExec_t inner_graph = nullptr;   // inner FP32 CG: entry nodes + while node
    int inner_graph_k = 0;
    double inner_graph_eta = -1.0;
    int64_t inner_entry_launches = 0, inner_body_launches = 0;
    struct LearnedWS *lws = nullptr;   // learned warm start of the SIMP loop (sgld_learned.cu)
    double *d_x0 = nullptr;            // [3*nnode] start of a mixed solve, kept for its FP64 fallback
    bool fault_drift = false;          // test hook (sgld_inject_fault kind 2): perturb the next mixed
                                       // solve's iterate before its true residual is checked
    cudaStream_t stream = nullptr;
    std::string err;
    int device = 0;
};

}  // namespace sgld

// The opaque handle of the C ABI.
struct sgld_ctx {
    sgld::Ctx c;
    // lazily allocated stress buffers
    double *d_s6 = nullptr, *d_vmn = nullptr, *d_vme = nullptr;
    std::vector<std::vector<int64_t>> nodemaps, elemaps;   // per level, 0-based full indices
    std::vector<int> h_rows;                               // coarsest free DOFs (full DOF index)
};

namespace sgld {

constexpr int CSPLIT = 16;   // column chunks of the coarse GEMV

// learned warm start of the SIMP loop (sgld_learned.cu)
void learned_free(LearnedWS *w);
int learned_setup(sgld_ctx *ctx, LearnedWS **pw, int net_level, bool need_net);
int learned_before_solve(sgld_ctx *ctx, LearnedWS *w, int mode, double E0, int *used, int *accepted,
                         double *ratio, double *ext_ratio);
int learned_after_solve(sgld_ctx *ctx, LearnedWS *w, int mode, int steps, float lr, double *loss);

// number of kernels this library has launched from the calling thread
// (host-side counter, one per launch; per thread, so that the launches counted
// while a thread captures a graph are exactly that graph's)
extern thread_local int64_t g_launches;

// ---- launchers (kernels_*.cu) ------------------------------------------------
void upload_kh(const double *Kh, cudaStream_t s);
// true when the 45 Hadamard-basis values take the 8 distinct values that the cubic
// symmetry of an isotropic hexahedral element gives them (to 1e-12 of the largest)
bool kh_cubic(const double *Kh);
void launch_kbyu_f64(const Level &l0, const double *E, const double *u, double *y, double *partial_dot,
                     int *nblocks_out, cudaStream_t s);
// (re)makes l0's active-tile maps for its current FP32 tile; 0 or a CUDA error
int update_kbyu_tiles(Level &l0, cudaStream_t s);
// 0, or a CUDA error code when the launch could not be set up (the input's tensor map).
// y is written at active nodes only: its inactive nodes must already hold zeros
// (every caller passes the context's d_t32, zeroed when allocated)
int launch_kbyu_f32(const Level &l0, const float *E, const float *u, float *y, double *partial_dot,
                    int *nblocks_out, cudaStream_t s);
void init_kernel_attributes();
int kbyu_f32_zc(const Level &l0);   // node layers per CTA the FP32 K*u uses on this level
int kbyu_f32_tx(const Level &l0);   // x width (elements) of the FP32 K*u tile on this level
int kbyu_f32_cta_layers(const Level &l0);   // node layers one CTA of the FP32 K*u covers
// double-float K*u (kernels_df.cu)
void upload_kh_df(const double *Kh, cudaStream_t s);
void init_kbyu_df_attributes();
void launch_kbyu_df(const Level &l0, const double *E, const double *u, double *y, double *partial_dot,
                    int *nblocks_out, cudaStream_t s);
// mixed-precision solve (kernels_mixed.cu)
// op 0 also sets the inner iteration cap (kbase at an outer solve's first inner solve,
// doubled up to klimit after a capped inner solve that missed its tolerance)
void launch_icg_scalar(int op, double *sc, const double *part, int nb, cudaStream_t s, int kbase, int klimit);
int launch_icg_update(float *e, float *s, const float *d, const float *t, int64_t n, const double *sc,
                      double *part, cudaStream_t st);
void launch_icg_cond(cudaGraphConditionalHandle h, double *sc, const double *part, int nb, int kmax,
                     double eta_min, const double *outer, double *total, cudaStream_t s);
int launch_icg_init(const float *r, float *s, float *e, float *d, int64_t n, double *part, cudaStream_t st);
void launch_outer_cond(cudaGraphConditionalHandle hw, cudaGraphConditionalHandle hi, const int *iflag,
                       cudaStream_t s);
void launch_set_cond(cudaGraphConditionalHandle h, unsigned v, cudaStream_t s);
void launch_icg_cond_flag(int *flag, double *sc, const double *part, int nb, int kmax, double eta_min,
                          const double *outer, double *total, cudaStream_t s);
void launch_icg_dupdate(float *e, float *d, const float *w, int64_t n, const double *sc, cudaStream_t st);
// the same updates over the finest level's active runs (Level::runs)
int launch_icg_update_runs(float *s, const float *t, const int64_t *runs, int64_t nruns, const double *sc,
                           double *part, cudaStream_t st);
void launch_icg_dupdate_runs(float *e, float *d, const float *w, const int64_t *runs, int64_t nruns,
                             const double *sc, cudaStream_t st);
void launch_widen_dots(const float *e, const float *d, const double *sc, double *z, const double *r,
                       const double *q, int64_t n, double *p1,
                       double *p2, int nb, cudaStream_t st);
void launch_flex_beta(double *scal, const int *iflag, const double *p1, const double *p2, int nb, int first,
                      cudaStream_t st);
void launch_narrow(const double *a, float *b, int64_t n, cudaStream_t st);
void launch_widen(const float *a, double *b, int64_t n, cudaStream_t st);
}  // namespace sgld
struct sgld_solve_opts;
struct sgld_solve_info;
namespace sgld {
// Devices a process can bind contexts on (ordinals 0 .. kMaxDevices-1).
constexpr int kMaxDevices = 64;
// Every entry point that touches the device binds its context first
// (sgld_api.cu): the context's device becomes current, and the element
// matrix's Hadamard blocks in __constant__ memory (one copy per device, shared
// by all contexts on it) become this context's.  A context whose matrix differs
// from the one held waits for the device to go idle before the upload, so
// contexts of different materials may alternate from one thread; contexts of
// equal matrices never re-upload and may run concurrently.
int bind_ctx(sgld_ctx *ctx);
// true if the constants on the current device hold c's element matrix
bool kh_bound(const Ctx &c);
// sgld_create calls this for its device: a device reset (cudaDeviceReset, or
// MATLAB's reset(gpuDevice)) clears every __constant__ table and module
// address, while the host-side records of what each device holds survive it.
// Creation therefore uploads the element matrix again and makes the assembly
// tables and the allocation-free scratch address be set up anew on first use.
void forget_device_tables(int dev);
void forget_asm_tables(int dev);       // kernels_asm.cu
void forget_noalloc_scratch(int dev);  // noalloc.cu
// PCG on the context's own full-grid vectors d_b / d_x (sgld_api.cu)
int solve_on_device(sgld_ctx *ctx, const sgld_solve_opts *o, sgld_solve_info *info);
// FP64 additive V-cycle z = M r on full-grid vectors; with partial, the CTA
// partials of z.r (nb of them) for launch_finalize_sum
int vcycle_f64(sgld_ctx *ctx, const double *r, double *z, double *partial, int *nb);
// the FP32 V-cycle on FP32 full-grid vectors (z: the context's d_z32, whose inactive nodes hold 0)
int vcycle_f32(sgld_ctx *ctx, const float *r, float *z, double *partial, int *nb);
// SIMP loop (kernels_topopt.cu)
void upload_filter_weights(double rmin, int *radius, double *d_w, cudaStream_t s);
void launch_density_filter(const Level &l0, const double *x, int r, const double *fw, double *y, cudaStream_t s);
void launch_topo_modulus(const Level &l0, const double *xp, double p, double E0, double Emin, double *E,
                         double *pv, double *ps, int nb, cudaStream_t s);
void launch_topo_sens(const Level &l0, const double *xp, const double *ce, const double *Hs, double p, double E0,
                      double Emin, double *dcs, double *dvs, int nb, cudaStream_t s);
void launch_topo_q(const Level &l0, const double *x, const double *dc, const double *dv, double *q, int nb,
                   cudaStream_t s);
void launch_oc_step(const Level &l0, const double *x, const double *q, const double *dv, double move,
                    const double *st, double *part, int nb, cudaStream_t s);
void launch_oc_scalar(int op, double *st, const double *part, int nb, double nact, double volfrac, cudaStream_t s);
void launch_oc_apply(const Level &l0, double *x, const double *q, double move, const double *st, double *part,
                     int nb, cudaStream_t s);
void launch_max_partials(const double *part, int nb, double *out, cudaStream_t s);
void launch_div(const Level &l0, const double *a, const double *b, double *y, int nb, cudaStream_t s);
void launch_fill_active(const Level &l0, double *y, double v, int nb, cudaStream_t s);
// local-volume loop (kernels_topopt.cu)
void launch_heaviside(const Level &l0, const double *xt, double beta, double eta, double *xp, double *dx, int nb,
                      cudaStream_t s);
void launch_local_sens(const Level &l0, const double *xp, const double *ce, const double *dx, const double *Hs,
                       double p, double E0, double Emin, double inv_csolid, double *dcs, int nb, cudaStream_t s);
// S = sum (xh/vmax)^p into *S (device), g = dfdx of the p-norm local volume
void launch_pnorm(const Level &l0, const double *xh, double p, double alpha, double *part, double *S, double N,
                  double *g, int nb, cudaStream_t s);
void launch_mul_div(const Level &l0, const double *a, const double *b, const double *c, double *y, int nb,
                    cudaStream_t s);
int launch_mma_gather(const int64_t *var, int64_t nvar, const double *x, const double *dc, const double *dv,
                      double move, double scale, double *xv, double *xmin, double *xmax, double *df0, double *dg,
                      cudaStream_t s);
void launch_mma_scatter(const int64_t *var, int64_t nvar, const double *xn, const double *xv, double *x,
                        double *part, int nb, cudaStream_t s);
void launch_set_passive_x(const Level &l0, double *x, int nb, cudaStream_t s);
void launch_mark_passive(const Level &l0, const int64_t *full, int64_t np, int nb, cudaStream_t s);
void launch_unit_compliance(const Level &l0, const double *u, const double *E, double *ce_full,
                            double *partial, int *nblocks_out, cudaStream_t s);
void launch_stress(const Level &l0, const double *E, const double *u, const double *M48x24,
                   double *nodal6, double *vm_node, cudaStream_t s);
void launch_elem_vm(const Level &l0, const double *nodal6, double *vm_elem_full, cudaStream_t s);
void launch_principal(const Level &l0, const double *s6, double *ps_node, double *dir_elem, cudaStream_t s);
// PDE density filter (kernels_pde.cu)
void upload_kpde(const double *K, double *d_kp, cudaStream_t s);
void launch_pde_e2n(const Level &l0, const double *xe, double *yn, cudaStream_t s);
int launch_pde_kbyu(const Level &l0, const double *Kp, const double *u, double *y, double *partial, cudaStream_t s);
void launch_pde_diag(const Level &l0, const double *Kp, double *dinv, cudaStream_t s);
void launch_pde_jacobi(const double *r, const double *dinv, int64_t n, double *z, double *partial, int nb,
                       cudaStream_t s);
void launch_pde_n2e(const Level &l0, const double *t, double *xe, cudaStream_t s);
// MMA update (kernels_mma.cu)
int mma_blocks(int64_t n);
void launch_mma_eval(const double *xv, const double *xmin, const double *xmax, const double *df0, const double *dg,
                     int64_t n, double lam, double *xout, double *part1, double *part2, double *sums2,
                     cudaStream_t s);

template <typename T>
void launch_restrict(const Level &fine, const Level &coarse, const T *rf, T *rc, cudaStream_t s);
template <typename T>
void launch_prolong_smooth(const Level &fine, const Level &coarse, const T *xc, const T *rf, const T *diag,
                           T omega, T *xf, bool final_level, double *partial_dot, int *nblocks_out,
                           cudaStream_t s);
void launch_diag_finest(const Level &l0, const double *E, const double *Ke, double *diag, cudaStream_t s);
void launch_diag_from_Ks(const Level &l, double *diag, cudaStream_t s);
void launch_inverse_diag(const Level &l, cudaStream_t s);   // l.idiag, l.idiag32 from l.diag
void launch_scatter_nodes(const int64_t *map, int64_t n, const double *compact, double *full, cudaStream_t s);
void launch_gather_nodes(const int64_t *map, int64_t n, const double *full, double *compact, cudaStream_t s);
void launch_scatter_elems(const int64_t *map, int64_t n, const double *compact, double *full, cudaStream_t s);
void launch_gather_elems(const int64_t *map, int64_t n, const double *full, double *compact, cudaStream_t s);
void launch_fixed_indicator(const Level &l, double *v, cudaStream_t s);
void launch_mark_fixed(Level &l, const double *restricted, cudaStream_t s);

void launch_asm_templates(const Level &coarse, int S, const double *E, const double *H, double *Ks, cudaStream_t s);
void launch_diag_templates(const Level &coarse, const double *E, const double *H2, double *diag, cudaStream_t s);
void launch_asm_coarse(const Level &coarse, const Level &fine, double *Ks, cudaStream_t s);
void launch_coarse_dense(const Level &lc, int ncf, const int *cfree_pos_of_dof, double *A, cudaStream_t s);
int coarse_factor_invert(Ctx &c);
int ensure_coarse_m64(Ctx &c);   // FP64 L^-1 for the FP64 V-cycle (0 or -1 on a CUDA error)  // returns 0 or error
void launch_coarse_apply_f64(const Ctx &c, const double *rc, double *xc, cudaStream_t s);
void launch_coarse_apply_f32(const Ctx &c, const float *rc, float *xc, cudaStream_t s);

// vector ops (FP64 PCG)
int reduce_blocks(int64_t n);
void launch_dot(const double *a, const double *b, int64_t n, double *partial, int nb, cudaStream_t s);
void launch_finalize_sum(const double *partial, int nb, double *out, cudaStream_t s);
void launch_pcg_update(double *x, double *r, const double *p, const double *q, int64_t n, const double *scal,
                       int *iflag, double *partial, int nb, cudaStream_t s);
void launch_pcg_pupdate(double *p, const double *z, int64_t n, const double *scal, const int *iflag,
                        cudaStream_t s);
void launch_residual(double *r, const double *b, const double *Ax, int64_t n, cudaStream_t s);
void launch_scale(double *x, double a, int64_t n, cudaStream_t s);
void launch_pcg_scalar(int op, double *scal, int *iflag, const double *partial, int nb, double tol, int maxit,
                       cudaStream_t s);
void launch_mask_fixed(const Level &l0, double *v, cudaStream_t s);
void launch_cast_f32(const double *a, float *b, int64_t n, cudaStream_t s);
void launch_cast_f64(const float *a, double *b, int64_t n, cudaStream_t s);

}  // namespace sgld
