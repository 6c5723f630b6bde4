// Mixed-precision instantiations of the fused step with viscous fluxes compiled in ([viscosity]
// enabled). The 3D tile is 8x8x4: the t^n velocities the viscous fluxes keep do not fit next to an
// 8x8x8 tile in shared memory.
#include <type_traits>

#include "launch.cuh"

namespace gmhd
{
using VMX_3D_884 = Cfg<float, 3, 8, 8, 4, 256, false, false, true>;
using VMX_3D_444 = Cfg<float, 3, 4, 4, 4, 64, false, false, true>;
using VMX_2D_16 = Cfg<float, 2, 16, 16, 1, 256, false, false, true>;
using VMX_2D_8 = Cfg<float, 2, 8, 8, 1, 64, false, false, true>;
using VMX_2D_4 = Cfg<float, 2, 4, 4, 1, 32, false, false, true>;
using VMX_3D_884_AMR = Cfg<float, 3, 8, 8, 4, 256, false, true, true>;
using VMX_3D_444_AMR = Cfg<float, 3, 4, 4, 4, 64, false, true, true>;
using VMX_2D_16_AMR = Cfg<float, 2, 16, 16, 1, 256, false, true, true>;
using VMX_2D_8_AMR = Cfg<float, 2, 8, 8, 1, 64, false, true, true>;
using VMX_2D_4_AMR = Cfg<float, 2, 4, 4, 1, 32, false, true, true>;

template <bool AMR>
int
launch_step_mixed_visc_cfg(const StepArgs & a, int dim, cudaStream_t stream)
{
  int       cand[3];
  const int x = pick_tile(cand, tile_candidates_mixed(dim, a.bx, a.by, a.bz, true, AMR, cand), a.tile);
  if (dim == 3)
  {
    if (x == 8)
      return launch_fused<std::conditional_t<AMR, VMX_3D_884_AMR, VMX_3D_884>>(a, stream);
    return launch_fused<std::conditional_t<AMR, VMX_3D_444_AMR, VMX_3D_444>>(a, stream);
  }
  if (x == 16)
    return launch_fused<std::conditional_t<AMR, VMX_2D_16_AMR, VMX_2D_16>>(a, stream);
  if (x == 8)
    return launch_fused<std::conditional_t<AMR, VMX_2D_8_AMR, VMX_2D_8>>(a, stream);
  return launch_fused<std::conditional_t<AMR, VMX_2D_4_AMR, VMX_2D_4>>(a, stream);
}

int
launch_step_mixed_visc(const StepArgs & a, int dim, cudaStream_t stream)
{
  return a.kind ? launch_step_mixed_visc_cfg<true>(a, dim, stream) : launch_step_mixed_visc_cfg<false>(a, dim, stream);
}

int
prepare_mixed_visc()
{
  int rc = 0;
  rc = rc ? rc : prepare_fused<VMX_3D_884>();
  rc = rc ? rc : prepare_fused<VMX_3D_444>();
  rc = rc ? rc : prepare_fused<VMX_2D_16>();
  rc = rc ? rc : prepare_fused<VMX_2D_8>();
  rc = rc ? rc : prepare_fused<VMX_2D_4>();
  rc = rc ? rc : prepare_fused<VMX_3D_884_AMR>();
  rc = rc ? rc : prepare_fused<VMX_3D_444_AMR>();
  rc = rc ? rc : prepare_fused<VMX_2D_16_AMR>();
  rc = rc ? rc : prepare_fused<VMX_2D_8_AMR>();
  rc = rc ? rc : prepare_fused<VMX_2D_4_AMR>();
  return rc;
}
} // namespace gmhd
