// FP64 instantiations of the fused step with viscous fluxes compiled in ([viscosity] enabled), in a
// unit of their own so that both sets compile in parallel. --fmad=false, as the other FP64 units.
#include <type_traits>

#include "launch.cuh"

namespace gmhd
{
using V64_3D_844 = Cfg<double, 3, 8, 4, 4, 256, true, false, true>;
using V64_3D_444 = Cfg<double, 3, 4, 4, 4, 64, true, false, true>;
using V64_2D_16 = Cfg<double, 2, 16, 16, 1, 256, true, false, true>;
using V64_2D_8 = Cfg<double, 2, 8, 8, 1, 64, true, false, true>;
using V64_2D_4 = Cfg<double, 2, 4, 4, 1, 32, true, false, true>;
using V64_3D_844_AMR = Cfg<double, 3, 8, 4, 4, 256, true, true, true>;
using V64_3D_444_AMR = Cfg<double, 3, 4, 4, 4, 64, true, true, true>;
using V64_2D_16_AMR = Cfg<double, 2, 16, 16, 1, 256, true, true, true>;
using V64_2D_8_AMR = Cfg<double, 2, 8, 8, 1, 64, true, true, true>;
using V64_2D_4_AMR = Cfg<double, 2, 4, 4, 1, 32, true, true, true>;

template <bool AMR>
int
launch_step_fp64_visc_cfg(const StepArgs & a, int dim, cudaStream_t stream)
{
  int       cand[3];
  const int x = pick_tile(cand, tile_candidates_fp64(dim, a.bx, a.by, a.bz, true, cand), a.tile);
  if (dim == 3)
  {
    if (x == 8)
      return launch_fused<std::conditional_t<AMR, V64_3D_844_AMR, V64_3D_844>>(a, stream);
    return launch_fused<std::conditional_t<AMR, V64_3D_444_AMR, V64_3D_444>>(a, stream);
  }
  if (x == 16)
    return launch_fused<std::conditional_t<AMR, V64_2D_16_AMR, V64_2D_16>>(a, stream);
  if (x == 8)
    return launch_fused<std::conditional_t<AMR, V64_2D_8_AMR, V64_2D_8>>(a, stream);
  return launch_fused<std::conditional_t<AMR, V64_2D_4_AMR, V64_2D_4>>(a, stream);
}

int
launch_step_fp64_visc(const StepArgs & a, int dim, cudaStream_t stream)
{
  return a.kind ? launch_step_fp64_visc_cfg<true>(a, dim, stream) : launch_step_fp64_visc_cfg<false>(a, dim, stream);
}

int
prepare_fp64_visc()
{
  int rc = 0;
  rc = rc ? rc : prepare_fused<V64_3D_844>();
  rc = rc ? rc : prepare_fused<V64_3D_444>();
  rc = rc ? rc : prepare_fused<V64_2D_16>();
  rc = rc ? rc : prepare_fused<V64_2D_8>();
  rc = rc ? rc : prepare_fused<V64_2D_4>();
  rc = rc ? rc : prepare_fused<V64_3D_844_AMR>();
  rc = rc ? rc : prepare_fused<V64_3D_444_AMR>();
  rc = rc ? rc : prepare_fused<V64_2D_16_AMR>();
  rc = rc ? rc : prepare_fused<V64_2D_8_AMR>();
  rc = rc ? rc : prepare_fused<V64_2D_4_AMR>();
  return rc;
}
} // namespace gmhd
