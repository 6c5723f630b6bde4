// Host-side launch helpers shared by the kernel instantiation units.
#pragma once

#include <cuda_runtime.h>

#include "fused_step.cuh"

namespace gmhd
{

// Launch the fused step for configuration C. Returns a cudaError_t (0 on success) or -1 when the
// tile does not divide the block.
template <class C>
int
launch_fused(StepArgs a, cudaStream_t stream)
{
  if (a.bx % C::TX || a.by % C::TY || (C::DIM == 3 && a.bz % C::TZ))
    return -1;
  a.tiles_x = a.bx / C::TX;
  a.tiles_y = a.by / C::TY;
  a.tiles_z = C::DIM == 3 ? a.bz / C::TZ : 1;
  const long long nblocks = (long long)a.n_owned * a.tiles_x * a.tiles_y * a.tiles_z;
  if (nblocks <= 0)
    return 0;
  fused_step_kernel<C><<<(unsigned)nblocks, C::NT, C::SMEM_BYTES, stream>>>(a);
  return (int)cudaGetLastError();
}

// Opt configuration C into its dynamic shared-memory size on the current device. Called when a
// context is created, so that no attribute call happens while a stream is being captured.
template <class C>
int
prepare_fused()
{
  return (int)cudaFuncSetAttribute(fused_step_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)C::SMEM_BYTES);
}

// Tile choice: the largest configured tile that divides the block.
int launch_step_fp64(const StepArgs & a, int dim, cudaStream_t stream);
int launch_step_mixed(const StepArgs & a, int dim, cudaStream_t stream);
int prepare_fp64();
int prepare_mixed();

} // namespace gmhd
