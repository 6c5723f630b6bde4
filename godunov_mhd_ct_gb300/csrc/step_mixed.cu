// Mixed-precision instantiations of the fused step: FP32 slopes, predictor, Riemann solvers and
// EMFs; FP64 conserved/face-B accumulation, CT curl and low-beta pressure recovery.
#include "launch.cuh"

namespace gmhd
{
using MX_3D_888 = Cfg<float, 3, 8, 8, 8, 512, false>;
using MX_3D_444 = Cfg<float, 3, 4, 4, 4, 64, false>;
using MX_2D_16 = Cfg<float, 2, 16, 16, 1, 256, false>;
using MX_2D_8 = Cfg<float, 2, 8, 8, 1, 64, false>;
using MX_2D_4 = Cfg<float, 2, 4, 4, 1, 32, false>;

int
launch_step_mixed(const StepArgs & a, int dim, cudaStream_t stream)
{
  if (dim == 3)
  {
    if (a.bx % 8 == 0 && a.by % 8 == 0 && a.bz % 8 == 0)
      return launch_fused<MX_3D_888>(a, stream);
    return launch_fused<MX_3D_444>(a, stream);
  }
  if (a.bx % 16 == 0 && a.by % 16 == 0)
    return launch_fused<MX_2D_16>(a, stream);
  if (a.bx % 8 == 0 && a.by % 8 == 0)
    return launch_fused<MX_2D_8>(a, stream);
  return launch_fused<MX_2D_4>(a, stream);
}

int
prepare_mixed()
{
  int rc = 0;
  rc = rc ? rc : prepare_fused<MX_3D_888>();
  rc = rc ? rc : prepare_fused<MX_3D_444>();
  rc = rc ? rc : prepare_fused<MX_2D_16>();
  rc = rc ? rc : prepare_fused<MX_2D_8>();
  rc = rc ? rc : prepare_fused<MX_2D_4>();
  return rc;
}
} // namespace gmhd
