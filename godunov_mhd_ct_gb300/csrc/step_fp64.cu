// FP64 instantiations of the fused step: the drop-in path. This unit is compiled with
// --fmad=false so that every a*b+c stays unfused, matching the reference formulas' FP64 rounding.
#include <type_traits>

#include "launch.cuh"

namespace gmhd
{
using F64_3D_844 = Cfg<double, 3, 8, 4, 4, 256, true>;
using F64_3D_444 = Cfg<double, 3, 4, 4, 4, 64, true>;
using F64_2D_16 = Cfg<double, 2, 16, 16, 1, 256, true>;
using F64_2D_8 = Cfg<double, 2, 8, 8, 1, 64, true>;
using F64_2D_4 = Cfg<double, 2, 4, 4, 1, 32, true>;
using F64_3D_844_AMR = Cfg<double, 3, 8, 4, 4, 256, true, true>;
using F64_3D_444_AMR = Cfg<double, 3, 4, 4, 4, 64, true, true>;
using F64_2D_16_AMR = Cfg<double, 2, 16, 16, 1, 256, true, true>;
using F64_2D_8_AMR = Cfg<double, 2, 8, 8, 1, 64, true, true>;
using F64_2D_4_AMR = Cfg<double, 2, 4, 4, 1, 32, true, true>;

template <bool AMR>
int
launch_step_fp64_cfg(const StepArgs & a, int dim, cudaStream_t stream)
{
  int       cand[3];
  const int x = pick_tile(cand, tile_candidates_fp64(dim, a.bx, a.by, a.bz, false, cand), a.tile);
  if (dim == 3)
  {
    if (x == 8)
      return launch_fused<std::conditional_t<AMR, F64_3D_844_AMR, F64_3D_844>>(a, stream);
    return launch_fused<std::conditional_t<AMR, F64_3D_444_AMR, F64_3D_444>>(a, stream);
  }
  if (x == 16)
    return launch_fused<std::conditional_t<AMR, F64_2D_16_AMR, F64_2D_16>>(a, stream);
  if (x == 8)
    return launch_fused<std::conditional_t<AMR, F64_2D_8_AMR, F64_2D_8>>(a, stream);
  return launch_fused<std::conditional_t<AMR, F64_2D_4_AMR, F64_2D_4>>(a, stream);
}

int
launch_step_fp64(const StepArgs & a, int dim, cudaStream_t stream)
{
  if (a.src.viscosity)
    return launch_step_fp64_visc(a, dim, stream);
  return a.kind ? launch_step_fp64_cfg<true>(a, dim, stream) : launch_step_fp64_cfg<false>(a, dim, stream);
}

int
tile_candidates_fp64(int dim, int bx, int by, int bz, bool /*visc: same tiles*/, int * out)
{
  int n = 0;
  if (dim == 3)
  {
    // 8x4x4 tiles, then 4x4x4
    if (bx % 8 == 0 && by % 4 == 0 && bz % 4 == 0)
      out[n++] = 8;
    if (bx % 4 == 0 && by % 4 == 0 && bz % 4 == 0)
      out[n++] = 4;
    return n;
  }
  for (int t : {16, 8, 4})
    if (bx % t == 0 && by % t == 0)
      out[n++] = t;
  return n;
}

void
tile_shape_fp64(int dim, int bx, int by, int bz, bool visc, int tile, int * t)
{
  int       cand[3];
  const int x = pick_tile(cand, tile_candidates_fp64(dim, bx, by, bz, visc, cand), tile);
  if (dim == 3)
  {
    t[0] = x == 8 ? 8 : 4;
    t[1] = 4;
    t[2] = 4;
    return;
  }
  const int n = x ? x : 4;
  t[0] = t[1] = n;
  t[2] = 1;
}

int
prepare_fp64()
{
  int rc = 0;
  rc = rc ? rc : prepare_fused<F64_3D_844>();
  rc = rc ? rc : prepare_fused<F64_3D_444>();
  rc = rc ? rc : prepare_fused<F64_2D_16>();
  rc = rc ? rc : prepare_fused<F64_2D_8>();
  rc = rc ? rc : prepare_fused<F64_2D_4>();
  rc = rc ? rc : prepare_fused<F64_3D_844_AMR>();
  rc = rc ? rc : prepare_fused<F64_3D_444_AMR>();
  rc = rc ? rc : prepare_fused<F64_2D_16_AMR>();
  rc = rc ? rc : prepare_fused<F64_2D_8_AMR>();
  rc = rc ? rc : prepare_fused<F64_2D_4_AMR>();
  return rc;
}
} // namespace gmhd

namespace gmhd
{
// ComputeDtMHDFunctor::compute_cfl (scheme/ComputeDtMHDFunctor.cpp:86-151) over the owned blocks,
// one CTA per block, max-reduced per problem. FP64 with the reference operand order.
__global__ void __launch_bounds__(256)
inv_dt_kernel(const double * __restrict__ U, const double * __restrict__ B, const int32_t * __restrict__ level,
              const int32_t * __restrict__ problem, int dim, int bx, int by, int bz, int64_t ncell, int64_t nfx,
              int64_t nfy, int64_t nface, double gamma0, double smallr, double smallp, double scaling_factor,
              Sources src, unsigned long long * invdt)
{
  const int     blk = blockIdx.x;
  const double  dx = (1.0 / (double)((int64_t)bx << level[blk])) * scaling_factor;
  const double *Ub = U + (int64_t)blk * 5 * ncell;
  const double *Bb = B + (int64_t)blk * nface;
  double        m = 0.0;
  for (int64_t c = threadIdx.x; c < ncell; c += blockDim.x)
  {
    const int i = (int)(c % bx), j = (int)((c / bx) % by), k = (int)(c / ((int64_t)bx * by));
    m = fmax(m, cell_inv_dt_fp64(Ub, Bb, dim, bx, by, i, j, k, c, ncell, nfx, nfy, dx, gamma0, smallr, smallp, src));
  }
  __shared__ double red[8];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
    m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0)
    red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0)
  {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      m = fmax(m, red[w]);
    atomicMax(&invdt[problem ? problem[blk] : 0], (unsigned long long)__double_as_longlong(m));
  }
}

int
launch_inv_dt(const double * U, const double * B, const int32_t * level, const int32_t * problem, int n_owned, int dim,
              int bx, int by, int bz, int64_t ncell, int64_t nfx, int64_t nfy, int64_t nface, double gamma0,
              double smallr, double smallp, double scaling_factor, const Sources & src, unsigned long long * invdt,
              cudaStream_t stream)
{
  if (n_owned <= 0)
    return 0;
  inv_dt_kernel<<<n_owned, 256, 0, stream>>>(U, B, level, problem, dim, bx, by, bz, ncell, nfx, nfy, nface, gamma0,
                                             smallr, smallp, scaling_factor, src, invdt);
  return (int)cudaGetLastError();
}
} // namespace gmhd
