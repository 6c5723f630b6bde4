// Mixed-precision instantiations of the fused step: FP32 slopes, predictor, Riemann solvers and
// EMFs; FP64 conserved/face-B accumulation, CT curl and low-beta pressure recovery.
#include <type_traits>

#include "launch.cuh"

namespace gmhd
{
using MX_3D_888 = Cfg<float, 3, 8, 8, 8, 512, false>;
using MX_3D_444 = Cfg<float, 3, 4, 4, 4, 64, false>;
using MX_2D_16 = Cfg<float, 2, 16, 16, 1, 256, false>;
using MX_2D_8 = Cfg<float, 2, 8, 8, 1, 64, false>;
using MX_2D_4 = Cfg<float, 2, 4, 4, 1, 32, false>;
using MX_3D_888_AMR = Cfg<float, 3, 8, 8, 8, 512, false, true>;
using MX_3D_444_AMR = Cfg<float, 3, 4, 4, 4, 64, false, true>;
using MX_2D_16_AMR = Cfg<float, 2, 16, 16, 1, 256, false, true>;
using MX_2D_8_AMR = Cfg<float, 2, 8, 8, 1, 64, false, true>;
using MX_2D_4_AMR = Cfg<float, 2, 4, 4, 1, 32, false, true>;

template <bool AMR>
int
launch_step_mixed_cfg(const StepArgs & a, int dim, cudaStream_t stream)
{
  int       cand[3];
  const int x = pick_tile(cand, tile_candidates_mixed(dim, a.bx, a.by, a.bz, false, AMR, cand), a.tile);
  if (dim == 3)
  {
    if (x == 16)
      return launch_column(a, stream);
    if (x == 8)
      return launch_fused<std::conditional_t<AMR, MX_3D_888_AMR, MX_3D_888>>(a, stream);
    return launch_fused<std::conditional_t<AMR, MX_3D_444_AMR, MX_3D_444>>(a, stream);
  }
  if (x == 16)
    return launch_fused<std::conditional_t<AMR, MX_2D_16_AMR, MX_2D_16>>(a, stream);
  if (x == 8)
    return launch_fused<std::conditional_t<AMR, MX_2D_8_AMR, MX_2D_8>>(a, stream);
  return launch_fused<std::conditional_t<AMR, MX_2D_4_AMR, MX_2D_4>>(a, stream);
}

int
launch_step_mixed(const StepArgs & a, int dim, cudaStream_t stream)
{
  if (a.src.viscosity)
    return launch_step_mixed_visc(a, dim, stream);
  return a.kind ? launch_step_mixed_cfg<true>(a, dim, stream) : launch_step_mixed_cfg<false>(a, dim, stream);
}

int
tile_candidates_mixed(int dim, int bx, int by, int bz, bool visc, bool amr, int * out)
{
  int n = 0;
  if (dim == 3)
  {
    // 8x8x8 tiles (8x8x4 with the viscous velocities), then 4x4x4, then 16 x 8 columns
    if (bx % 8 == 0 && by % 8 == 0 && bz % (visc ? 4 : 8) == 0)
      out[n++] = 8;
    if (bx % 4 == 0 && by % 4 == 0 && bz % 4 == 0)
      out[n++] = 4;
    if (!visc && !amr && bx % 16 == 0 && by % 8 == 0)
      out[n++] = 16;
    return n;
  }
  for (int t : {16, 8, 4})
    if (bx % t == 0 && by % t == 0)
      out[n++] = t;
  return n;
}

void
tile_shape_mixed(int dim, int bx, int by, int bz, bool visc, bool amr, int tile, int * t)
{
  int       cand[3];
  const int x = pick_tile(cand, tile_candidates_mixed(dim, bx, by, bz, visc, amr, cand), tile);
  if (dim == 3)
  {
    if (x == 16)
    {
      t[0] = 16;
      t[1] = 8;
      t[2] = bz;
      return;
    }
    const int n = x == 8 ? 8 : 4;
    t[0] = t[1] = n;
    t[2] = visc ? 4 : n;
    return;
  }
  const int n = x ? x : 4;
  t[0] = t[1] = n;
  t[2] = 1;
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
  rc = rc ? rc : prepare_fused<MX_3D_888_AMR>();
  rc = rc ? rc : prepare_fused<MX_3D_444_AMR>();
  rc = rc ? rc : prepare_fused<MX_2D_16_AMR>();
  rc = rc ? rc : prepare_fused<MX_2D_8_AMR>();
  rc = rc ? rc : prepare_fused<MX_2D_4_AMR>();
  rc = rc ? rc : prepare_column();
  return rc;
}
} // namespace gmhd

namespace gmhd
{
// FP32 estimate of ComputeDtMHDFunctor::compute_cfl (scheme/ComputeDtMHDFunctor.cpp:86-151) for
// the mixed path's solver loop: one CTA per owned block, max-reduced per problem.
__global__ void __launch_bounds__(256)
inv_dt_mixed_kernel(const double * __restrict__ U, const double * __restrict__ B, const int32_t * __restrict__ level,
                    const int32_t * __restrict__ problem, int dim, int bx, int by, int bz, int64_t ncell,
                    int64_t nfx, int64_t nfy, int64_t nface, float gamma0, float smallr, float smallp,
                    double scaling_factor, Sources src, unsigned long long * invdt)
{
  const int     blk = blockIdx.x;
  const double  dx = (1.0 / (double)((int64_t)bx << level[blk])) * scaling_factor;
  const float   idx = d2f_bits(1.0 / dx);
  const double *Ub = U + (int64_t)blk * 5 * ncell;
  const double *Bb = B + (int64_t)blk * nface;
  float         m = 0.0f;
  for (int64_t c = threadIdx.x; c < ncell; c += blockDim.x)
  {
    const int   i = (int)(c % bx), j = (int)((c / bx) % by), k = (int)(c / ((int64_t)bx * by));
    const float Ax = 0.5f * (d2f_bits(Bb[i + (int64_t)(bx + 1) * (j + (int64_t)by * k)]) +
                             d2f_bits(Bb[i + 1 + (int64_t)(bx + 1) * (j + (int64_t)by * k)]));
    const float Ay = 0.5f * (d2f_bits(Bb[nfx + i + (int64_t)bx * (j + (int64_t)(by + 1) * k)]) +
                             d2f_bits(Bb[nfx + i + (int64_t)bx * (j + 1 + (int64_t)(by + 1) * k)]));
    const float Az = dim == 3 ? 0.5f * (d2f_bits(Bb[nfx + nfy + i + (int64_t)bx * (j + (int64_t)by * k)]) +
                                        d2f_bits(Bb[nfx + nfy + i + (int64_t)bx * (j + (int64_t)by * (k + 1))]))
                              : d2f_bits(Bb[nfx + nfy + c]);
    const float r = fmaxf(d2f_bits(Ub[c]), smallr);
    const float ir = 1.0f / r;
    const float vx = d2f_bits(Ub[2 * ncell + c]) * ir, vy = d2f_bits(Ub[3 * ncell + c]) * ir,
                vz = d2f_bits(Ub[4 * ncell + c]) * ir;
    const float ekin = 0.5f * r * (vx * vx + vy * vy + vz * vz);
    const float emag = 0.5f * (Ax * Ax + Ay * Ay + Az * Az);
    const float p = fmaxf((gamma0 - 1.0f) * (d2f_bits(Ub[ncell + c]) - emag - ekin), r * smallp);
    const float c2 = gamma0 * p * ir;
    const float d2 = 0.5f * (2.0f * emag * ir + c2);
    const float cfx = sqrtf(d2 + sqrtf(fmaxf(d2 * d2 - c2 * Ax * Ax * ir, 0.0f))) + fabsf(vx);
    const float cfy = sqrtf(d2 + sqrtf(fmaxf(d2 * d2 - c2 * Ay * Ay * ir, 0.0f))) + fabsf(vy);
    const float cfz = dim == 3 ? sqrtf(d2 + sqrtf(fmaxf(d2 * d2 - c2 * Az * Az * ir, 0.0f))) + fabsf(vz) : 0.0f;
    m = fmaxf(m, cfl_inv_dt_fp32(dim, cfx, cfy, cfz, (float)dx, idx, d2f_bits(Ub[c]), src));
  }
  __shared__ float red[8];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
    m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0)
    red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0)
  {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      m = fmaxf(m, red[w]);
    atomicMax(&invdt[problem ? problem[blk] : 0], (unsigned long long)__double_as_longlong(f2d_bits(m)));
  }
}

int
launch_inv_dt_mixed(const double * U, const double * B, const int32_t * level, const int32_t * problem, int n_owned,
                    int dim, int bx, int by, int bz, int64_t ncell, int64_t nfx, int64_t nfy, int64_t nface,
                    double gamma0, double smallr, double smallp, double scaling_factor, const Sources & src,
                    unsigned long long * invdt, cudaStream_t stream)
{
  if (n_owned <= 0)
    return 0;
  inv_dt_mixed_kernel<<<n_owned, 256, 0, stream>>>(U, B, level, problem, dim, bx, by, bz, ncell, nfx, nfy, nface,
                                                   (float)gamma0, (float)smallr, (float)smallp, scaling_factor, src,
                                                   invdt);
  return (int)cudaGetLastError();
}
} // namespace gmhd
