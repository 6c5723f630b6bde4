// Host-side launch helpers shared by the kernel instantiation units.
#pragma once

#include <cuda_runtime.h>

#include "fused_step.cuh"

namespace gmhd
{

// Launch the fused step for configuration C. Returns a cudaError_t (0 on success) or -1 when the
// tile does not divide the block.
// Resident CTAs of configuration C on the whole device (persistent variants), set by prepare_fused.
template <class C>
int &
resident_ctas()
{
  static int n = 0;
  return n;
}

template <class C>
int
launch_fused(StepArgs a, cudaStream_t stream)
{
  if (a.bx % C::TX || a.by % C::TY || (C::DIM == 3 && a.bz % C::TZ))
    return -1;
  a.tiles_x = a.bx / C::TX;
  a.tiles_y = a.by / C::TY;
  a.tiles_z = C::DIM == 3 ? a.bz / C::TZ : 1;
  long long nblocks = a.tile_list ? (long long)a.n_list
                                  : (long long)(a.blk_list ? a.blk_count : a.n_owned) * a.tiles_x * a.tiles_y * a.tiles_z;
  if (nblocks <= 0)
    return 0;
  if constexpr (C::PIPE)
  {
    // one persistent CTA per resident slot, each looping over tiles (or over the pass's tile list)
    if (resident_ctas<C>() <= 0)
      return -1;
    nblocks = nblocks < resident_ctas<C>() ? nblocks : resident_ctas<C>();
  }
  fused_step_kernel<C><<<(unsigned)nblocks, C::NT, C::SMEM_BYTES, stream>>>(a);
  return (int)cudaGetLastError();
}

// Opt configuration C into its dynamic shared-memory size on the current device and record how
// many CTAs of it the device holds. Called when a context is created, so that no attribute call
// happens while a stream is being captured.
template <class C>
int
prepare_fused()
{
  cudaError_t e = cudaFuncSetAttribute(fused_step_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)C::SMEM_BYTES);
  if (e != cudaSuccess || !C::PIPE)
    return (int)e;
  int dev = 0, sms = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
      (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fused_step_kernel<C>, C::NT, C::SMEM_BYTES)) !=
        cudaSuccess)
    return (int)e;
  resident_ctas<C>() = sms * (per_sm > 0 ? per_sm : 1);
  return 0;
}

// Tile choice: a.tile when it is one of the configured tiles that divide the block (named by their
// x extent), else the largest that does. With a.src.viscosity the viscous variants run
// (launch_step_*_visc).
int launch_step_fp64(const StepArgs & a, int dim, cudaStream_t stream);
int launch_step_mixed(const StepArgs & a, int dim, cudaStream_t stream);
int launch_step_fp64_visc(const StepArgs & a, int dim, cudaStream_t stream);
int launch_step_mixed_visc(const StepArgs & a, int dim, cudaStream_t stream);
// configured tiles (x extents, largest first) that divide these blocks; returns their count (<= 3).
// Mixed 3D without viscosity on a conforming mesh (amr false) also offers 16: the column step
// (column_step.cuh, 16 x 8 columns through the block's z extent), listed after the 3D tiles.
int tile_candidates_fp64(int dim, int bx, int by, int bz, bool visc, int * out);
int tile_candidates_mixed(int dim, int bx, int by, int bz, bool visc, bool amr, int * out);
// the tile extents launch_step_* uses for these block sizes and request (column step: 16, 8, bz)
void tile_shape_fp64(int dim, int bx, int by, int bz, bool visc, int tile, int * t);
void tile_shape_mixed(int dim, int bx, int by, int bz, bool visc, bool amr, int tile, int * t);
// column step (step_column.cu): -1 when it does not apply to these blocks / this mesh
int launch_column(const StepArgs & a, cudaStream_t stream);
int prepare_column();

// the requested tile when it is a candidate, else the first (largest) candidate, 0 when none fits
inline int
pick_tile(const int * cand, int n, int req)
{
  for (int i = 0; i < n; ++i)
    if (cand[i] == req)
      return req;
  return n > 0 ? cand[0] : 0;
}
int prepare_fp64();
int prepare_mixed();
int prepare_fp64_visc();
int prepare_mixed_visc();

// coarse/fine ghost prepass (amr.cu): fills the virtual neighbour blocks read by the fused step
struct GhostArgs
{
  const double *  U;
  const double *  B;
  double *        Uv;
  double *        Bv;
  double *        Bccv;
  const int32_t * vmap;     // [n_virtual][2]: owner block, neighbour slot
  const int32_t * neighbor; // [n_blocks * 27] real ids (same-level, coarser or outside block)
  const int8_t *  kind;     // [n_owned * 27]
  const int32_t * fine;     // [n_blocks * 27 * 8]
  const int32_t * coord;    // [n_blocks * 3]
  int             n_virtual, dim, bx, by, bz, prolongation;
  int64_t         ncell, nfx, nfy, nface;
  unsigned int *  health;
};

int launch_ghost_prepass(const GhostArgs & g, cudaStream_t stream);

// regrid (amr.cu): refinement flags of the owned blocks and the remap to an adapted mesh
int launch_refine_flags(const double * U, const double * B, const int32_t * level, int n_owned, int dim, int bx,
                        int by, int bz, int64_t ncell, int64_t nfx, int64_t nfy, int64_t nface, double gamma0,
                        double smallr, double smallp, int criterion, int level_min, int level_max, int use_rho,
                        int use_pressure, double eps_refine, double eps_coarsen, double eps_lohner, double * scratch,
                        int8_t * flags, cudaStream_t stream);
int launch_remap(const GhostArgs & g, const int32_t * remap, int n_new, double * Un, double * Bn, cudaStream_t stream);

} // namespace gmhd
