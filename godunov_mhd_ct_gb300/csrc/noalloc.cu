// Allocation-free CFL reduction: gmhd_inv_dt_noalloc (declared in include/gmhd.h).
//
// Some callers cannot call cudaMalloc: code running while a stream is being captured into a CUDA
// graph, host frameworks that own every device allocation (a memory pool they must account for),
// or processes whose allocations are fenced off after start-up. gmhd_inv_dt needs a context, and a
// context allocates device memory for its mesh tables and its reduction slots. This entry point
// needs neither: the caller passes the state (U, B), the per-block problem ids (or none) and a
// device output buffer, and the reduction accumulator lives in the fixed array below.
//
// The array g_inv_dt_scratch has GMHD_NOALLOC_MAX_PROBLEMS 64-bit slots (8 KB). Every GPU that
// loads this library holds it until the process exits. All calls on a device share it and it keeps
// the last call's contents, so each call clears the slots it uses before reducing into them; calls
// that overlap on the GPU (on different streams, without ordering between them) race on it.
// Compiled with --fmad=false: the per-cell arithmetic is the FP64 reference formula order, so the
// result equals gmhd_inv_dt's.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/gmhd.h"
#include "mhd_math.cuh"

namespace
{
using gmhd::cfl_inv_dt_fp64;
using gmhd::Sources;

__device__ __align__(256) unsigned long long g_inv_dt_scratch[GMHD_NOALLOC_MAX_PROBLEMS];

constexpr int kMaxDevices = 64;
std::mutex    g_setup_mutex;
void *        g_scratch_addr[kMaxDevices] = {};

// Device address of g_inv_dt_scratch on the current device. Host code cannot use the symbol
// itself (its host-side name is only a stand-in), so the address is looked up once per device.
int
scratch_address(void ** out)
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return GMHD_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev])
  {
    void * p = nullptr;
    if (cudaGetSymbolAddress(&p, g_inv_dt_scratch) != cudaSuccess || !p)
      return GMHD_ERR_CUDA;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return GMHD_OK;
}

__global__ void
clear_slots_kernel(unsigned long long * slots, int n)
{
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
    slots[p] = 0ull;
}

// compute_cfl (scheme/ComputeDtMHDFunctor.cpp:86-151) per owned cell, one CTA per block, max per
// problem into slots[]. All blocks at one level (cell size dx).
__global__ void __launch_bounds__(256)
inv_dt_noalloc_kernel(const double * __restrict__ U, const double * __restrict__ B,
                      const int32_t * __restrict__ problem, int dim, int bx, int by, int bz, int64_t ncell,
                      int64_t nfx, int64_t nfy, int64_t nface, double dx, double gamma0, double smallr,
                      double smallp, Sources src, unsigned long long * slots)
{
  const int     blk = blockIdx.x;
  const double *Ub = U + (int64_t)blk * 5 * ncell;
  const double *Bb = B + (int64_t)blk * nface;
  double        m = 0.0;
  for (int64_t c = threadIdx.x; c < ncell; c += blockDim.x)
  {
    const int i = (int)(c % bx), j = (int)((c / bx) % by), k = (int)(c / ((int64_t)bx * by));
    const double Ax = 0.5 * (Bb[i + (int64_t)(bx + 1) * (j + (int64_t)by * k)] +
                             Bb[i + 1 + (int64_t)(bx + 1) * (j + (int64_t)by * k)]);
    const double Ay = 0.5 * (Bb[nfx + i + (int64_t)bx * (j + (int64_t)(by + 1) * k)] +
                             Bb[nfx + i + (int64_t)bx * (j + 1 + (int64_t)(by + 1) * k)]);
    double Az;
    if (dim == 3)
      Az = 0.5 * (Bb[nfx + nfy + i + (int64_t)bx * (j + (int64_t)by * k)] +
                  Bb[nfx + nfy + i + (int64_t)bx * (j + (int64_t)by * (k + 1))]);
    else
      Az = 0.5 * (Bb[nfx + nfy + c] + Bb[nfx + nfy + c]);
    // compute_primitives (models/mhd_utils.h:449-515) and find_speed_info (:340-394)
    const double r = fmax(Ub[c], smallr);
    const double vx = Ub[2 * ncell + c] / r, vy = Ub[3 * ncell + c] / r, vz = Ub[4 * ncell + c] / r;
    const double eken = 0.5 * (vx * vx + vy * vy + vz * vz);
    const double emag = 0.5 * (Ax * Ax + Ay * Ay + Az * Az);
    const double eint = (Ub[ncell + c] - emag) / r - eken;
    const double p = fmax((gamma0 - 1.0) * r * eint, r * smallp);
    const double b2 = Ax * Ax + Ay * Ay + Az * Az;
    const double c2 = gamma0 * p / r;
    const double d2 = 0.5 * (b2 / r + c2);
    const double cfx = sqrt(d2 + sqrt(d2 * d2 - c2 * Ax * Ax / r)) + fabs(vx);
    const double cfy = sqrt(d2 + sqrt(d2 * d2 - c2 * Ay * Ay / r)) + fabs(vy);
    const double cfz = dim == 3 ? sqrt(d2 + sqrt(d2 * d2 - c2 * Az * Az / r)) + fabs(vz) : 0.0;
    m = fmax(m, cfl_inv_dt_fp64(dim, cfx, cfy, cfz, dx, Ub[c], src));
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
    // positive doubles order like their bit patterns
    atomicMax(&slots[problem ? problem[blk] : 0], (unsigned long long)__double_as_longlong(m));
  }
}

__global__ void
write_out_kernel(const unsigned long long * slots, double * out, int n)
{
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
    out[p] = __longlong_as_double((long long)slots[p]);
}
} // namespace

extern "C" int
gmhd_inv_dt_noalloc(const gmhd_params * params, int32_t dim, int32_t bx, int32_t by, int32_t bz, int32_t n_blocks,
                    int32_t level, const int32_t * problem, int32_t n_problems, const double * U, const double * B,
                    double * inv_dt, void * stream)
{
  if (!params || !U || !B || !inv_dt)
    return GMHD_ERR_ARGUMENT;
  if ((dim != 2 && dim != 3) || bx < 1 || by < 1 || (dim == 3 && bz < 1) || (dim == 2 && bz != 1) || n_blocks < 0 ||
      level < 0 || level > 30 || !(params->gamma0 > 1.0) || !(params->scaling_factor > 0.0))
    return GMHD_ERR_ARGUMENT;
  const int np = problem ? n_problems : 1;
  if (np < 1)
    return GMHD_ERR_ARGUMENT;
  if (np > GMHD_NOALLOC_MAX_PROBLEMS)
    return GMHD_ERR_TOO_LARGE;
  void * addr = nullptr;
  int    rc = scratch_address(&addr);
  if (rc != GMHD_OK)
    return rc;
  unsigned long long * slots = static_cast<unsigned long long *>(addr);
  cudaStream_t         s = (cudaStream_t)stream;
  const int64_t        ncell = (int64_t)bx * by * bz;
  const int64_t        nfx = (int64_t)(bx + 1) * by * bz;
  const int64_t        nfy = (int64_t)bx * (by + 1) * bz;
  const int64_t        nfz = dim == 3 ? (int64_t)bx * by * (bz + 1) : ncell;
  const int64_t        nface = nfx + nfy + nfz;
  const double         dx = (1.0 / (double)((int64_t)bx << level)) * params->scaling_factor;
  const double         smallp = params->smallc * params->smallc / params->gamma0;
  Sources src;
  src.gravity = params->gravity_enabled != 0;
  for (int d = 0; d < 3; ++d)
    src.g[d] = src.gravity ? params->gravity[d] : 0.0;
  src.viscosity = params->viscosity_enabled != 0;
  src.mu = src.viscosity ? params->viscosity_mu : 0.0;
  src.visc_predictor = 0;
  clear_slots_kernel<<<(np + 255) / 256, 256, 0, s>>>(slots, np);
  if (n_blocks > 0)
    inv_dt_noalloc_kernel<<<n_blocks, 256, 0, s>>>(U, B, problem, dim, bx, by, bz, ncell, nfx, nfy, nface, dx,
                                                   params->gamma0, params->smallr, smallp, src, slots);
  write_out_kernel<<<(np + 255) / 256, 256, 0, s>>>(slots, inv_dt, np);
  return cudaGetLastError() == cudaSuccess ? GMHD_OK : GMHD_ERR_CUDA;
}
