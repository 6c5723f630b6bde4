// Column-step instantiation (mixed precision, 3D, conforming meshes): 16 x 8 columns, 256 threads,
// two CTAs per SM, persistent over the columns of the owned blocks.
#include "column_step.cuh"
#include "launch.cuh"

namespace gmhd
{
using COL_16x8 = ColCfg<16, 8, 256>;
static_assert(COL_16x8::SMEM_BYTES + 2048 <= 113 * 1024, "two column CTAs must fit in one SM's shared memory");

namespace
{
int g_column_ctas = 0; // resident column CTAs on the device (set by prepare_column)
}

int
launch_column(const StepArgs & a, cudaStream_t stream)
{
  using K = COL_16x8;
  if (a.bx % K::TX || a.by % K::TY || a.kind || a.tile_list)
    return -1;
  const long long n_work = (long long)(a.blk_list ? a.blk_count : a.n_owned) * (a.bx / K::TX) * (a.by / K::TY);
  if (n_work <= 0)
    return 0;
  if (g_column_ctas <= 0)
    return -1;
  const long long grid = n_work < g_column_ctas ? n_work : g_column_ctas;
  column_step_kernel<K><<<(unsigned)grid, K::NT, K::SMEM_BYTES, stream>>>(a);
  return (int)cudaGetLastError();
}

int
prepare_column()
{
  using K = COL_16x8;
  cudaError_t e = cudaFuncSetAttribute(column_step_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)K::SMEM_BYTES);
  if (e != cudaSuccess)
    return (int)e;
  int dev = 0, sms = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
      (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, column_step_kernel<K>, K::NT, K::SMEM_BYTES)) !=
        cudaSuccess)
    return (int)e;
  g_column_ctas = sms * (per_sm > 0 ? per_sm : 1);
  return 0;
}
} // namespace gmhd
