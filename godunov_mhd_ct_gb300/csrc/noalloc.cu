// Allocation-free CFL reduction: gmhd_inv_dt_noalloc (declared in include/gmhd.h).
//
// Some callers cannot call cudaMalloc: code running while a stream is being captured into a CUDA
// graph, host frameworks that own every device allocation (a memory pool they must account for),
// or processes whose allocations are fenced off after start-up. gmhd_inv_dt needs a context, and a
// context allocates device memory for its mesh tables and its reduction slots. This entry point
// needs neither: the caller passes the state (U, B), the per-block problem ids (or none) and a
// device output buffer, and the reduction accumulator lives in the fixed array below.
//
// The array g_inv_dt_scratch has GMHD_NOALLOC_MAX_PROBLEMS 64-bit slots (8 KB) plus one flag slot.
// Every GPU that loads this library holds it until the process exits. All calls on a device share it
// and it keeps the last call's contents, so each call clears the slots it uses (and the flag) before
// reducing into them; calls that overlap on the GPU (on different streams, without ordering between
// them) race on it. A block whose problem id is outside [0, n_problems) is skipped and sets the flag
// slot, and the call then writes NaN to every output: the ids live on the device, so the host cannot
// check them without a copy, and the kernel never indexes the array with them.
// Compiled with --fmad=false and sharing cell_inv_dt_fp64 with gmhd_inv_dt, so the result equals
// gmhd_inv_dt's.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/gmhd.h"
#include "mhd_math.cuh"

namespace
{
using gmhd::Sources;

// [0, GMHD_NOALLOC_MAX_PROBLEMS): per-problem maxima; [GMHD_NOALLOC_MAX_PROBLEMS]: bad-id flag
constexpr int kFlagSlot = GMHD_NOALLOC_MAX_PROBLEMS;
__device__ __align__(256) unsigned long long g_inv_dt_scratch[GMHD_NOALLOC_MAX_PROBLEMS + 1];

constexpr int kMaxDevices = 64;
std::mutex    g_setup_mutex;
void *        g_scratch_addr[kMaxDevices] = {};

// Device address of g_inv_dt_scratch on device `dev` (the current device). Host code cannot use the
// symbol itself (its host-side name is only a stand-in), so the address is looked up once per device.
int
scratch_address(int dev, void ** out)
{
  if (dev < 0 || dev >= kMaxDevices)
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

// Clears slots [0, n) and the bad-id flag.
__global__ void
clear_slots_kernel(unsigned long long * slots, int n)
{
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
    slots[p] = 0ull;
  if (blockIdx.x == 0 && threadIdx.x == 0)
    slots[kFlagSlot] = 0ull;
}

// compute_cfl (scheme/ComputeDtMHDFunctor.cpp:86-151) per owned cell, one CTA per block, max per
// problem into slots[]. All blocks at one level (cell size dx). A block whose problem id is not in
// [0, np) does no work and sets the flag slot.
__global__ void __launch_bounds__(256)
inv_dt_noalloc_kernel(const double * __restrict__ U, const double * __restrict__ B,
                      const int32_t * __restrict__ problem, int np, int dim, int bx, int by, int bz, int64_t ncell,
                      int64_t nfx, int64_t nfy, int64_t nface, double dx, double gamma0, double smallr,
                      double smallp, Sources src, unsigned long long * slots)
{
  const int blk = blockIdx.x;
  const int pid = problem ? problem[blk] : 0;
  if ((unsigned)pid >= (unsigned)np)
  {
    // uniform over the CTA: every thread leaves before any barrier
    if (threadIdx.x == 0)
      atomicExch(&slots[kFlagSlot], 1ull);
    return;
  }
  const double *Ub = U + (int64_t)blk * 5 * ncell;
  const double *Bb = B + (int64_t)blk * nface;
  double        m = 0.0;
  for (int64_t c = threadIdx.x; c < ncell; c += blockDim.x)
  {
    const int i = (int)(c % bx), j = (int)((c / bx) % by), k = (int)(c / ((int64_t)bx * by));
    m = fmax(m, gmhd::cell_inv_dt_fp64(Ub, Bb, dim, bx, by, i, j, k, c, ncell, nfx, nfy, dx, gamma0, smallr, smallp,
                                       src));
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
    atomicMax(&slots[pid], (unsigned long long)__double_as_longlong(m));
  }
}

// Per-problem results, or NaN everywhere when some block had a problem id out of range.
__global__ void
write_out_kernel(const unsigned long long * slots, double * out, int n)
{
  const bool bad = slots[kFlagSlot] != 0ull;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
    out[p] = bad ? __longlong_as_double(0x7ff8000000000000LL) : __longlong_as_double((long long)slots[p]);
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
  cudaStream_t s = (cudaStream_t)stream;
  // the array looked up below is the current device's: the stream must belong to that device
  int dev = -1, sdev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess)
    return GMHD_ERR_CUDA;
  if (s && (cudaStreamGetDevice(s, &sdev) != cudaSuccess || sdev != dev))
    return GMHD_ERR_ARGUMENT;
  void * addr = nullptr;
  int    rc = scratch_address(dev, &addr);
  if (rc != GMHD_OK)
    return rc;
  unsigned long long * slots = static_cast<unsigned long long *>(addr);
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
  // an error left by earlier, unrelated work is not this call's: clear it so that the check after the
  // launches reports only these
  (void)cudaGetLastError();
  clear_slots_kernel<<<(np + 255) / 256, 256, 0, s>>>(slots, np);
  if (n_blocks > 0)
    inv_dt_noalloc_kernel<<<n_blocks, 256, 0, s>>>(U, B, problem, np, dim, bx, by, bz, ncell, nfx, nfy, nface, dx,
                                                   params->gamma0, params->smallr, smallp, src, slots);
  write_out_kernel<<<(np + 255) / 256, 256, 0, s>>>(slots, inv_dt, np);
  return cudaGetLastError() == cudaSuccess ? GMHD_OK : GMHD_ERR_CUDA;
}
