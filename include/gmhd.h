/*
 * gmhd.h — C ABI of the GB300-native MUSCL-Hancock + constrained-transport MHD stage.
 *
 * Drop-in for the hot path of godunov_mhd_ct: the GodunovImplemBase implementation interface
 * (scheme/GodunovImplemBase.h:45-90) plus the two device calls the solver makes around it,
 * ComputeDtMHDFunctor::apply (scheme/ComputeDtMHDFunctor.cpp:44-82) and
 * FillOutsideCellFunctor::apply (border_conditions/FillOutside.cpp:47-93).
 *
 * Conventions
 *  - Every entry point returns an int status (GMHD_OK == 0, negative on error) and never aborts;
 *    the reference aborts through Kokkos::abort / KOKKOS_ASSERT instead.
 *  - Array arguments of the step / CFL / fill calls are DEVICE pointers, FP64, in this layout
 *    (one leaf block after another, blocks in the order of the mesh tables):
 *      U : [n_blocks][5][bz][by][bx]       (rho, E, rho u, rho v, rho w)
 *      B : [n_blocks][Bx | By | Bz]        Bx: [bz][by][bx+1], By: [bz][by+1][bx],
 *                                          Bz: [bz+1][by][bx] in 3D, [by][bx] cell-centred in 2D
 *    (DataArrayBlock / FaceDataArrayBlock hold the same per-block data; their in-block order is
 *    kalypsso-core's and cannot be checked here.) gmhd_layout_check() verifies a caller's
 *    strides against this layout.
 *  - Host-buffer variants (suffix _host) take HOST pointers and do the copies themselves.
 *  - Streams are cudaStream_t passed as void*; NULL is the legacy default stream.
 */
#ifndef GMHD_H_
#define GMHD_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum gmhd_status
{
  GMHD_OK = 0,
  GMHD_ERR_ARGUMENT = -1,    /* null pointer, bad size, unsupported option */
  GMHD_ERR_MESH = -2,        /* mesh not set, inconsistent tables, level jump */
  GMHD_ERR_CUDA = -3,        /* a CUDA call failed; see gmhd_last_cuda_error() */
  GMHD_ERR_ALIAS = -4,       /* output aliases an input */
  GMHD_ERR_HEALTH = -5,      /* the step produced a non-physical state (see gmhd_last_status) */
  GMHD_ERR_TOO_LARGE = -6,   /* request exceeds a fixed capacity */
};

enum gmhd_riemann
{ /* numeric values of RiemannSolverType (models/riemann_solver_types.h:26-37) */
  GMHD_RIEMANN_LLF = 2,
  GMHD_RIEMANN_HLL = 3,
  GMHD_RIEMANN_HLLC = 4,
  GMHD_RIEMANN_HLLD = 5
};

enum gmhd_precision
{
  GMHD_PRECISION_FP64 = 0,  /* reference arithmetic in FP64 (the drop-in) */
  GMHD_PRECISION_MIXED = 1  /* FP32 reconstruction/Riemann/EMF, FP64 accumulation and CT curl */
};

enum gmhd_bc
{ /* numeric values of BC_MHD (border_conditions/FillOutside.h:55-61) */
  GMHD_BC_NONE = 0,
  GMHD_BC_PERIODIC = 1,
  GMHD_BC_ZERO_GRADIENT = 2,
  GMHD_BC_WALL = 3
};

enum gmhd_prolongation
{ /* [amr] cell_centered_prolongation_type: hydro ghosts taken from a coarser neighbour
   * (scheme/ConvertToPrimitivesVariablesFunctor.cpp:699-718) */
  GMHD_PROLONG_SIMPLE_COPY = 0,
  GMHD_PROLONG_LINEAR_MINMOD = 1 /* EXTRAPOLATE_LINEAR_MINMOD */
};

enum gmhd_time_integrator
{ /* [amr] time_integrator (SolverGodunovMHD.cpp:488-647) */
  GMHD_TIME_HANCOCK = 0, /* MUSCL-Hancock: one stage with the half-step predictor */
  GMHD_TIME_RK2_SSP = 1  /* two stages without the predictor, U = 1/2 U + 1/2 U2 (gmhd_advance) */
};

/* Regrid refinement criterion ([amr] refine_criterion, epsilon_refine, epsilon_coarsen, epsilon_lohner,
 * level_min, level_max, variable_used_to_compute_refine_criterion; SolverGodunovMHD.cpp:1092-1186). */
enum gmhd_refine_criterion
{
  GMHD_REFINE_SIMPLE_GRADIENT = 0,
  GMHD_REFINE_LOHNER_UNSPLIT = 1
};

typedef struct gmhd_refine_params
{
  int32_t criterion; /* enum gmhd_refine_criterion */
  int32_t level_min, level_max;
  int32_t use_rho, use_pressure; /* quantities the indicator is taken on (max over them) */
  double  eps_refine, eps_coarsen, eps_lohner;
} gmhd_refine_params;

/* Health flags reported by gmhd_last_status. */
enum gmhd_health_flags
{
  GMHD_HEALTH_MISSING_NEIGHBOR = 1u,
  GMHD_HEALTH_LEVEL_JUMP = 2u,
  GMHD_HEALTH_BAD_DENSITY = 4u,
  GMHD_HEALTH_NONFINITE = 8u,
  GMHD_HEALTH_LOW_BETA_FP64 = 16u /* informational */
};

/* Settings read on the hot path: [hydro] gamma0, cfl, slope_type, smallr, smallc, riemann
 * (models/HydroSettings.cpp:18-31) and [mesh] scaling_factor. smallp = smallc^2/gamma0 is derived
 * as in the reference. */
typedef struct gmhd_params
{
  double  gamma0;
  double  cfl;
  double  slope_type;
  double  smallr;
  double  smallc;
  double  scaling_factor;
  int32_t riemann;   /* enum gmhd_riemann */
  int32_t precision; /* enum gmhd_precision */
  int32_t prolongation; /* [amr] cell_centered_prolongation_type: enum gmhd_prolongation */
  int32_t time_integrator; /* [amr] time_integrator: enum gmhd_time_integrator */
  /* Uniform gravity ([gravity] enabled, uniform_gx/gy/gz): the half-step velocity kick of the Hancock
   * predictor (scheme/ComputeUpdatedPrimitiveVariablesFunctor.cpp:372-377, 505-511), the momentum and
   * energy source after the update (scheme/AddGravitySourceTerm.cpp:47-99) and the CFL with gravity
   * (scheme/ComputeDtMHDFunctor.cpp:155-249). gravity[2] is ignored in 2D. */
  int32_t gravity_enabled;
  double  gravity[3];
  /* Viscosity ([viscosity] enabled, mu): viscous face fluxes applied after the hydro fluxes
   * (scheme/ComputeViscousFluxesAndStoreFunctor.cpp:168-344, scheme/GodunovImplemV0.cpp:179-192),
   * the CFL bound 4 mu / (rho dx^2) (scheme/ComputeDtMHDFunctor.cpp:144-148) and, with
   * viscous_predictor, the Hancock predictor term (ComputeUpdatedPrimitiveVariablesFunctor.cpp:174-280). */
  int32_t viscosity_enabled;
  double  viscosity_mu;
  int32_t viscous_predictor;
} gmhd_params;

/* Leaf-block mesh (HOST pointers; copied by gmhd_set_mesh). Blocks [0, n_owned) are updated;
 * blocks [n_owned, n_blocks) are outside blocks filled by gmhd_fill_outside.
 * neighbor[b*27 + (oz+1)*9 + (oy+1)*3 + (ox+1)] is the block across face/edge/corner (ox,oy,oz)
 * of block b, or -1. cell size of block b = scaling_factor / (bx * 2^level[b]).
 *
 * Coarse/fine meshes (2:1 balanced across faces, edges and corners, as p4est's full balance;
 * the reference's AMR, scheme/ConvertToPrimitivesVariablesFunctor.cpp:699-718,
 * scheme/ReadFluxesAndConservativeUpdateFunctor.cpp:141-172,
 * scheme/CorrectEmfAtBlockBorderFunctor.cpp:94-360): the block-sized region next to b in
 * direction (ox,oy,oz) at b's level is either a leaf at that level (neighbor = it), part of a leaf
 * one level coarser (neighbor = that leaf; coord gives the position inside it), or split into
 * leaves one level finer (neighbor = -1 and fine_neighbor[(b*27 + slot)*8 + cx + 2cy + 4cz] = the
 * children, -1 where absent). Outside blocks are at the level of the block they serve, with a
 * same-level inside block across the border. Bx, by, bz must be even. */
typedef struct gmhd_mesh
{
  int32_t         dim;   /* 2 or 3 */
  int32_t         bx, by, bz; /* bz == 1 in 2D */
  int32_t         n_blocks;
  int32_t         n_owned;
  const int32_t * level;     /* [n_blocks] */
  const int32_t * neighbor;  /* [n_blocks * 27] */
  const int32_t * problem;   /* [n_blocks] independent-problem id, or NULL for a single problem */
  int32_t         n_problems;
  const int32_t * outside_src;    /* [n_blocks - n_owned] inside block across the outside normal */
  const int32_t * outside_normal; /* [3 * (n_blocks - n_owned)] per axis: +1 below the domain,
                                     -1 above it, 0 inside its range (points into the domain) */
  int32_t         bc[6];          /* enum gmhd_bc for XMIN, XMAX, YMIN, YMAX, ZMIN, ZMAX */
  const int32_t * coord;          /* [3 * n_blocks] block coordinates at the block's level, or NULL
                                     (needed when a neighbour is coarser; orchard-key position) */
  const int32_t * fine_neighbor;  /* [27 * 8 * n_blocks] children of refined neighbour regions, or
                                     NULL on meshes without finer neighbours */
  /* The same children as a list, read when fine_neighbor is NULL: entry i is
   * fine_neighbor[fine_at[i]] = fine_id[i], every other entry -1 (gmhd_forest_fine gives this list;
   * it avoids building and uploading the mostly empty table). n_fine = 0: no list. */
  int64_t         n_fine;
  const int64_t * fine_at;
  const int32_t * fine_id;
} gmhd_mesh;

typedef struct gmhd_ctx gmhd_ctx;

/* --- lifetime ------------------------------------------------------------------------------- */

/* Constructor of the implementation (GodunovImplemV0 ctor, scheme/GodunovImplemV0.h:46-104,
 * selected by create_godunov_implem, SolverGodunovMHD.h:326-340). Binds the current device.
 * Returns NULL on invalid parameters. */
gmhd_ctx * gmhd_create(const gmhd_params * params);
void       gmhd_destroy(gmhd_ctx * ctx);

/* resize_auxiliary_data (scheme/GodunovImplemBase.h:78-79): (re)loads the mesh tables after a
 * regrid or repartition. */
int gmhd_set_mesh(gmhd_ctx * ctx, const gmhd_mesh * mesh);

/* total_mem_size_in_bytes (scheme/GodunovImplemBase.h:82-83): device memory held by ctx. */
uint64_t gmhd_mem_bytes(const gmhd_ctx * ctx);

/* --- the stage ------------------------------------------------------------------------------ */

/* do_time_step (scheme/GodunovImplemBase.h:85-90, scheme/GodunovImplemV0.cpp:101-207).
 * Writes U2 = U + conservative update and B2 = B + CT update for the owned blocks. Unlike the
 * reference, U2/B2 need not equal U/B on entry (they are overwritten); they must not alias U/B.
 * Ghost/outside blocks of U and B must be filled (SolverGodunovMHD.cpp:497-498). U and B must be
 * 16-byte aligned (device allocations are); otherwise GMHD_ERR_ARGUMENT. */
int gmhd_step(gmhd_ctx * ctx, const double * U, double * U2, const double * B, double * B2, double dt,
              void * stream);

/* ComputeDtMHDFunctor::apply (scheme/ComputeDtMHDFunctor.cpp:44-82): invDt = max over owned
 * cells of sum_d (c_f,d + |v_d|)/dx, returned on the host (synchronises the stream). With
 * several problems, inv_dt receives n_problems values. */
int gmhd_inv_dt(gmhd_ctx * ctx, const double * U, const double * B, double * inv_dt, void * stream);

/* FillOutsideCellFunctor::apply (border_conditions/FillOutside.cpp:47-93): fills the outside
 * blocks of U and B from the adjacent inside blocks (ZERO_GRADIENT / WALL). No-op when periodic. */
int gmhd_fill_outside(gmhd_ctx * ctx, double * U, double * B, void * stream);

/* Solver loop (SolverGodunovMHD::next_iteration_impl, SolverGodunovMHD.cpp:407-484, without AMR,
 * IO and monitoring): nsteps of { dt = cfl / invDt (capped so no problem passes t_end);
 * fill outside; do_time_step; U <- U2, B <- B2 } with the CFL reduction fused into each step and
 * dt kept on the device. U/B hold the final state on return and U2/B2 are scratch of the same
 * size. t (per problem, in/out) and t_end may be NULL (no cap). dt_log (host, nsteps * n_problems)
 * may be NULL. The step sequence is captured once as a CUDA graph and replayed when use_graph. */
int gmhd_advance(gmhd_ctx * ctx, double * U, double * U2, double * B, double * B2, int32_t nsteps,
                 double * t, const double * t_end, double * dt_log, int32_t use_graph, void * stream);

/* Capacity of gmhd_inv_dt_noalloc: independent problems per call. */
#define GMHD_NOALLOC_MAX_PROBLEMS 1024

/* No counterpart in the reference. gmhd_inv_dt without any device allocation, for callers that
 * cannot call cudaMalloc (code running under CUDA-graph stream capture, frameworks that own all
 * device memory). No context is needed: the caller passes the state U, B (device, the layout
 * above, n_blocks blocks all at refinement level `level`), optional per-block problem ids
 * (device, NULL for one problem) and a device output inv_dt[n_problems]; the call is asynchronous
 * on `stream`. The reduction uses a fixed array of GMHD_NOALLOC_MAX_PROBLEMS slots in the library
 * (8 KB per GPU, held until the process exits); larger n_problems returns GMHD_ERR_TOO_LARGE.
 * The first call on each device looks that array up (cudaGetSymbolAddress); make that first call
 * before any stream capture. `stream` must belong to the current device (the array used is the
 * current device's); a stream of another device returns GMHD_ERR_ARGUMENT. Problem ids are read on
 * the device and never used as indices unchecked: a block whose id is outside [0, n_problems) is
 * skipped and every inv_dt[p] of that call is NaN. The call clears a CUDA error left by earlier work
 * (cudaGetLastError) before launching, so GMHD_ERR_CUDA reports only its own launches. Calls share
 * the array and clear their slots first; calls that overlap on the GPU race on it. Results equal
 * gmhd_inv_dt's. */
int gmhd_inv_dt_noalloc(const gmhd_params * params, int32_t dim, int32_t bx, int32_t by, int32_t bz,
                        int32_t n_blocks, int32_t level, const int32_t * problem, int32_t n_problems,
                        const double * U, const double * B, double * inv_dt, void * stream);

/* Tile autotuner (no counterpart in the reference): runs the step (U -> U2, B -> B2, time step dt; U2
 * and B2 are scratch here) with every shared-memory tile configuration compiled for this context's
 * precision and block size (x extents 8 and 4 in 3D, 16, 8 and 4 in 2D, where they divide the block),
 * two warm-up and five timed launches each on `stream`, and keeps the fastest for the context's
 * later steps, across gmhd_set_mesh calls with the same block size (the coarse/fine tile lists are
 * rebuilt for it). FP64 results do not depend on the tile; mixed-precision ones may differ in the last
 * FP32 bits (each tile is a separately compiled kernel). Writes the chosen x extent and its time per
 * step in ms (either pointer may be NULL). Synchronises the device. */
int gmhd_autotune(gmhd_ctx * ctx, const double * U, double * U2, const double * B, double * B2, double dt,
                  int32_t * tile_out, double * ms_out, void * stream);
/* Sets the tile request by hand: an x extent from the list above (one that does not divide the block
 * falls back to the largest that does), or 0 for that default. Synchronises the device. */
int gmhd_set_tile(gmhd_ctx * ctx, int32_t tile);

/* --- host-buffer variants ------------------------------------------------------------------- */

/* gmhd_step on HOST arrays: copies U, B to the device, runs the step, copies U2, B2 back, and returns
 * when U2, B2 hold the result. On conforming meshes without outside blocks (16 or more blocks) the work
 * is split into up to 8 chunks of blocks (slabs along the last axis when the mesh carries block
 * coordinates): a tile steps as soon as the blocks it reads have been copied in, and a chunk's results are
 * copied out while the next tiles step, so the copies in both directions overlap the step. The
 * results equal gmhd_step's bit for bit. Host buffers should be page-locked for the copies to run at
 * full speed and overlap. */
int gmhd_step_host(gmhd_ctx * ctx, const double * U, double * U2, const double * B, double * B2, double dt,
                   void * stream);

/* Refinement flags of the owned blocks (-1 coarsen, 0 keep, +1 refine) of the state U, B on the mesh
 * set in ctx (compute_refine_flags, SolverGodunovMHD.cpp:1092-1186; the indicator of kalypsso-core's
 * ComputeRefineFlags restated: per cell and axis, neighbours clamped to the block, SIMPLE_GRADIENT
 * max(|q+ - q|, |q - q-|) / |q| or LOHNER_UNSPLIT |dp - dm| / (|dp| + |dm| + eps (|q+| + 2|q| + |q-|)),
 * block error = max; +1 when error > eps_refine and level < level_max, -1 when error < eps_coarsen and
 * level > level_min). flags: HOST array of n_owned bytes. Synchronises `stream`. */
int gmhd_refine_flags(gmhd_ctx * ctx, const double * U, const double * B, const gmhd_refine_params * params,
                      int8_t * flags, void * stream);

/* Remap of the conservative state and face B to an adapted mesh (map_userdata_after_adapt,
 * SolverGodunovMHD.cpp:1189-1262; kalypsso-core's UserDataRemapper restated). remap: HOST array of
 * 15 ints per new owned block: kind (0 kept, 1 refined child, 2 coarsened parent), sources (kind 0:
 * old block; 1: old parent, child index x fastest; 2: the 2^d old children, x fastest), then the old
 * blocks of the same level kept across the faces -x, +x, -y, +y, -z, +z (-1 otherwise). Kept blocks are
 * copied; coarsened ones take the mean of their children (faces shared with a kept block copy it);
 * refined ones copy the parent cell and prolong face B divergence-free (faces shared with a kept block
 * copy it and the faces inside each parent cell absorb the difference). Writes the owned blocks of
 * U_new, B_new (device); synchronises `stream`. */
int gmhd_remap(int32_t dim, int32_t bx, int32_t by, int32_t bz, int32_t n_old_blocks, int32_t n_new_owned,
               const int32_t * remap, const double * U_old, const double * B_old, double * U_new, double * B_new,
               void * stream);

/* --- host-side leaf forest (p4est's adapt + balance and the mesh tables; SolverGodunovMHD.cpp:263-319) --- */

typedef struct gmhd_forest gmhd_forest;

/* Leaves keys[n] = (level, x, y, z) (position at the level over bricks[0..2] root trees). With flags
 * (one per leaf, -1 coarsen / 0 keep / +1 refine) the leaves are adapted first: flagged leaves below
 * level_max are refined, complete families flagged above level_min are coarsened; then the set is
 * 2:1 balanced across faces, edges and corners (refinement wins; a coarsening that balance would undo is
 * dropped) and the tables of gmhd_mesh are built (p4est order, outside blocks for non-periodic axes).
 * Without flags the keys are balanced and tabulated as given. Returns NULL on invalid input, on an
 * outside block without a same-level inside block, or on exhaustion. */
gmhd_forest * gmhd_forest_build(int32_t dim, const int32_t * bricks, const int32_t * periodic, int32_t bx, int32_t by,
                                 int32_t bz, int32_t level_min, int32_t level_max, int32_t n_leaves,
                                 const int32_t * keys, const int8_t * flags);
/* Block counts of the tabulated leaf set; *has_fine (may be NULL) is 1 when some neighbour region is
 * split into finer leaves (a coarse/fine mesh: fine_neighbor is needed), else 0. */
int gmhd_forest_sizes(const gmhd_forest * forest, int32_t * n_owned, int32_t * n_blocks, int32_t * has_fine);
/* Copies the tables (HOST arrays sized by gmhd_forest_sizes; any may be NULL): level[n_blocks],
 * coord[3 n_blocks], neighbor[27 n_blocks], fine_neighbor[27 * 8 n_blocks], outside_src[n_blocks - n_owned],
 * outside_normal[3 (n_blocks - n_owned)], remap[15 n_owned] (the rows gmhd_remap takes). */
int  gmhd_forest_tables(const gmhd_forest * forest, int32_t * level, int32_t * coord, int32_t * neighbor,
                        int32_t * fine_neighbor, int32_t * outside_src, int32_t * outside_normal, int32_t * remap);
/* The children table of the leaf set as a list (the entries of fine_neighbor that are not -1):
 * *n_fine receives their count; at[*n_fine] (int64 indices into the [27 * 8 n_blocks] table) and
 * id[*n_fine] are filled when not NULL (sized by a first call with NULL). */
int  gmhd_forest_fine(const gmhd_forest * forest, int64_t * n_fine, int64_t * at, int32_t * id);
void gmhd_forest_destroy(gmhd_forest * forest);

/* Stream-ordered gmhd_step_host (no counterpart in the reference; it exists for callers that keep the
 * state in host memory): copies U, B in, runs the step and copies the owned blocks of U2, B2 out, then
 * returns without waiting; the results are in U2/B2 once `stream` has completed the work enqueued
 * before this call returns (synchronise `stream`). Consecutive calls overlap: the host->device copy of
 * one call, the step of the previous call and the device->host copy of the one before run at the same
 * time (two device input sets and two output sets, released independently, and three streams owned by
 * ctx). U and B are read as they are in host
 * memory when the call is made (the copy-in does not wait for work on `stream`: synchronise `stream`
 * first when they are the results of an earlier call). Until the call completes, U and B must stay
 * unchanged and U2, B2 must not be read. Host buffers should be page-locked for the copies to overlap. */
int gmhd_step_host_async(gmhd_ctx * ctx, const double * U, double * U2, const double * B, double * B2, double dt,
                         void * stream);

/* --- diagnostics ---------------------------------------------------------------------------- */

/* Health flags accumulated since the last call (clears them). Synchronises the context stream. */
int gmhd_last_status(gmhd_ctx * ctx, uint32_t * flags);

/* Last CUDA error code seen by ctx (0 if none). */
int gmhd_last_cuda_error(const gmhd_ctx * ctx);

const char * gmhd_error_string(int status);

/* Checks a caller layout: strides (in doubles) of U between variables and blocks, and of B
 * between blocks, against the layout above. Returns GMHD_OK or GMHD_ERR_ARGUMENT. */
int gmhd_layout_check(const gmhd_mesh * mesh, int64_t u_var_stride, int64_t u_block_stride,
                      int64_t b_block_stride);

#ifdef __cplusplus
}
#endif

#endif /* GMHD_H_ */
