// C ABI of the GB300 MHD stage (declared in include/gmhd.h): context, mesh tables, the step,
// the CFL reduction, the outside-block fill and a graph-captured multi-step loop.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <unordered_map>
#include <vector>

#include "../../include/gmhd.h"
#include "launch.cuh"

namespace gmhd
{
int launch_inv_dt(const double * U, const double * B, const int32_t * level, const int32_t * problem,
                  int n_owned, int dim, int bx, int by, int bz, int64_t ncell, int64_t nfx, int64_t nfy,
                  int64_t nface, double gamma0, double smallr, double smallp, double scaling_factor,
                  const Sources & src, unsigned long long * invdt, cudaStream_t stream);
int launch_inv_dt_mixed(const double * U, const double * B, const int32_t * level, const int32_t * problem,
                        int n_owned, int dim, int bx, int by, int bz, int64_t ncell, int64_t nfx, int64_t nfy,
                        int64_t nface, double gamma0, double smallr, double smallp, double scaling_factor,
                        const Sources & src, unsigned long long * invdt, cudaStream_t stream);
} // namespace gmhd

struct gmhd_ctx
{
  gmhd_params p;
  double      smallp;
  int         device;
  // mesh
  bool    has_mesh = false;
  int     dim = 0, bx = 0, by = 0, bz = 0, n_blocks = 0, n_owned = 0, n_problems = 1, n_outside = 0;
  int64_t ncell = 0, nfx = 0, nfy = 0, nfz = 0, nface = 0;
  int     bc[6] = {0, 0, 0, 0, 0, 0};
  int32_t *d_neighbor = nullptr, *d_level = nullptr, *d_problem = nullptr;
  int32_t *d_out_src = nullptr, *d_out_normal = nullptr;
  // scratch
  unsigned long long * d_invdt = nullptr; // [3][n_problems]
  double *             d_dt = nullptr;    // [n_problems]
  double *             d_t = nullptr;     // [n_problems]
  double *             d_tend = nullptr;  // [n_problems]
  int32_t *            d_counter = nullptr;
  unsigned int *       d_health = nullptr;
  double *             d_dtlog = nullptr;
  int64_t              dtlog_cap = 0;
  // host-variant staging
  double *d_U = nullptr, *d_U2 = nullptr, *d_B = nullptr, *d_B2 = nullptr;
  // RK2_SSP stage buffers of gmhd_advance
  double *d_Urk = nullptr, *d_Brk = nullptr;
  // asynchronous host-variant pipeline: two staging sets, copy-in / step / copy-out streams
  double *     a_U[2] = {nullptr, nullptr}, *a_U2[2] = {nullptr, nullptr};
  double *     a_B[2] = {nullptr, nullptr}, *a_B2[2] = {nullptr, nullptr};
  cudaStream_t a_in = nullptr, a_run = nullptr, a_out = nullptr;
  cudaEvent_t  a_in_done[2] = {nullptr, nullptr}, a_run_done[2] = {nullptr, nullptr}, a_out_done[2] = {nullptr, nullptr};
  int          a_next = 0;
  // chunked gmhd_step_host on conforming meshes without outside blocks (plan_host_chunks): hp_k chunks
  // of owned blocks, hp_blocks[hp_off[k] .. hp_off[k+1]) (ascending ids; on the device in d_hp_blocks),
  // copied as the strided runs hp_copy[hp_coff[k] .. hp_coff[k+1]); chunk k steps once chunks
  // 0 .. hp_dep[k] are in (its blocks' neighbours lie there), in the order hp_order, and its copy-out
  // follows its step
  struct HostRuns
  {
    int start, len, stride, count; // blocks start + i * stride .. + len, i < count
  };
  static constexpr int  HP_MAX = 8;
  int                   hp_k = 0;
  std::vector<int>      hp_off, hp_coff, hp_dep, hp_order;
  std::vector<int32_t>  hp_blocks;
  std::vector<HostRuns> hp_copy;
  int32_t *             d_hp_blocks = nullptr;
  cudaEvent_t           hp_in[HP_MAX] = {}, hp_run[HP_MAX] = {}, hp_start = nullptr, hp_end = nullptr;
  // per owned block: its chunk, and the chunk of the block in each of its 27 neighbour slots (-1: none)
  std::vector<int8_t>   hp_chunk, hp_nchunk;
  // tile-level schedule for the current tile choice: group k (launched once chunks 0 .. k are in) is
  // d_hp_tiles[hp_toff[k] .. hp_toff[k+1]); chunk c's results are complete after group hp_done[c]
  int                   hp_tile_key = -1;
  std::vector<int>      hp_toff, hp_done;
  int32_t *             d_hp_tiles = nullptr;
  // the launches of the tile-level schedule: group k's tiles of chunk c's blocks, d_hp_tiles[off .. off + n);
  // the launch that completes a chunk comes first within its group
  struct HostLaunch
  {
    int k, c, off, n;
  };
  std::vector<HostLaunch> hp_launch;
  // own stream for graph capture when the caller passes the legacy stream
  cudaStream_t own_stream = nullptr;
  // cached graph of two steps
  cudaGraphExec_t graph_exec = nullptr;
  const void *    graph_key[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  int             mesh_version = 0, graph_mesh_version = -1;
  uint64_t        bytes = 0;
  int             last_cuda = 0;
  // bytes reserved behind every device buffer of the context (buffers are reused across meshes)
  std::unordered_map<const void *, size_t> cap;
  // coarse/fine meshes: virtual neighbour blocks, two-pass tile lists, fine-side data
  bool      amr = false;
  int       n_virtual = 0, n_list1 = 0, n_list2 = 0, flux_face_stride = 0;
  int8_t *  d_kind = nullptr;
  int32_t * d_fine = nullptr;
  // the children list of gmhd_mesh (fine_at, fine_id), scattered into d_fine after the uploads
  int64_t * d_fine_at = nullptr;
  int32_t * d_fine_id = nullptr;
  int64_t   fine_scatter = 0; // entries still to scatter at the next up_flush
  int32_t * d_coord = nullptr;
  int32_t * d_vmap = nullptr;
  int32_t * d_nbr_real = nullptr;
  int32_t * d_list1 = nullptr;
  int32_t * d_list2 = nullptr;
  int32_t * d_flux_slot = nullptr;
  int32_t * d_emf_slot = nullptr;
  double *  d_Uv = nullptr;
  double *  d_Bv = nullptr;
  double *  d_Bccv = nullptr;
  double *  d_flux_side = nullptr;
  double *  d_emf_side = nullptr;
  // gmhd_refine_flags scratch
  double * d_rf_q = nullptr;
  int8_t * d_rf_flags = nullptr;
  // gmhd_set_mesh uploads: recorded, then staged through one page-locked buffer (kept, grown as
  // needed) and issued asynchronously on own_stream, which set_mesh waits for before it returns
  struct Upload
  {
    void *       dst;
    const void * src; // null: a memset of `fill`
    size_t       bytes;
    int          fill;
  };
  std::vector<Upload> uploads;
  char *              h_stage = nullptr;
  size_t              h_stage_cap = 0;
  // host tables of the coarse/fine setup (kept so that their storage outlives the upload)
  std::vector<int8_t>  h_kind;
  std::vector<int32_t> h_knbr, h_vmap, h_list1, h_list2, h_flux_slot, h_emf_slot;
  // tile x extent the step asks for (0: the largest configured tile that divides the block; set by
  // gmhd_autotune, kept across meshes)
  int tile = 0;
};

namespace
{
int
cuda_fail(gmhd_ctx * c, cudaError_t e)
{
  if (e == cudaSuccess)
    return GMHD_OK;
  c->last_cuda = (int)e;
  return GMHD_ERR_CUDA;
}

// record a host->device copy / a memset for the batched upload of gmhd_set_mesh
void
up_copy(gmhd_ctx * c, void * dst, const void * src, size_t bytes)
{
  if (bytes)
    c->uploads.push_back(gmhd_ctx::Upload{dst, src, bytes, 0});
}
void
up_set(gmhd_ctx * c, void * dst, int fill, size_t bytes)
{
  if (bytes)
    c->uploads.push_back(gmhd_ctx::Upload{dst, nullptr, bytes, fill});
}
// children-list entries of a coarse/fine mesh into the dense table (indices checked on the host)
__global__ void
fine_scatter_kernel(const int64_t * __restrict__ at, const int32_t * __restrict__ id, int64_t n, int32_t * fine)
{
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    fine[at[i]] = id[i];
}

// stage the recorded copies through the page-locked buffer, issue everything on own_stream and wait
int
up_flush(gmhd_ctx * c)
{
  auto   rounded = [](size_t b) { return (b + 255) & ~(size_t)255; };
  size_t total = 0;
  for (const gmhd_ctx::Upload & u : c->uploads)
    if (u.src)
      total += rounded(u.bytes);
  cudaError_t e = cudaSuccess;
  if (total > c->h_stage_cap)
  {
    if (c->h_stage)
      cudaFreeHost(c->h_stage);
    c->h_stage = nullptr;
    c->h_stage_cap = 0;
    const size_t cap = total + total / 4;
    if ((e = cudaHostAlloc((void **)&c->h_stage, cap, cudaHostAllocDefault)) != cudaSuccess)
    {
      c->h_stage = nullptr;
      c->uploads.clear();
      return cuda_fail(c, e);
    }
    c->h_stage_cap = cap;
  }
  size_t off = 0;
  for (const gmhd_ctx::Upload & u : c->uploads)
  {
    if (!u.src)
      e = cudaMemsetAsync(u.dst, u.fill, u.bytes, c->own_stream);
    else
    {
      std::memcpy(c->h_stage + off, u.src, u.bytes);
      e = cudaMemcpyAsync(u.dst, c->h_stage + off, u.bytes, cudaMemcpyHostToDevice, c->own_stream);
      off += rounded(u.bytes);
    }
    if (e != cudaSuccess)
      break;
  }
  c->uploads.clear();
  if (e == cudaSuccess && c->fine_scatter > 0)
  {
    const int64_t n = c->fine_scatter;
    const int     grid = (int)std::min<int64_t>((n + 255) / 256, 152 * 8);
    fine_scatter_kernel<<<grid, 256, 0, c->own_stream>>>(c->d_fine_at, c->d_fine_id, n, c->d_fine);
    e = cudaGetLastError();
  }
  c->fine_scatter = 0;
  const cudaError_t e2 = cudaStreamSynchronize(c->own_stream);
  return cuda_fail(c, e != cudaSuccess ? e : e2);
}

#define GMHD_CUDA(call)                                                                           \
  do                                                                                              \
  {                                                                                               \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess)                                                                        \
      return cuda_fail(ctx, e_);                                                                  \
  } while (0)

template <typename T>
void
drelease(gmhd_ctx * ctx, T ** ptr)
{
  if (!*ptr)
    return;
  auto it = ctx->cap.find((const void *)*ptr);
  if (it != ctx->cap.end())
  {
    ctx->bytes -= it->second;
    ctx->cap.erase(it);
  }
  cudaFree((void *)*ptr);
  *ptr = nullptr;
}

// Device buffers outlive a mesh: a buffer is reallocated only when the new size does not fit, then
// with a quarter of headroom, so that an AMR cycle every few steps costs no cudaMalloc / cudaFree.
template <typename T>
int
dalloc(gmhd_ctx * ctx, T ** ptr, size_t count)
{
  const size_t need = count * sizeof(T);
  size_t       take = need;
  if (*ptr)
  {
    const auto   it = ctx->cap.find((const void *)*ptr);
    const size_t have = it != ctx->cap.end() ? it->second : 0;
    if (need <= have)
      return GMHD_OK;
    take = need + need / 4;
    drelease(ctx, ptr);
  }
  if (count == 0)
    return GMHD_OK;
  GMHD_CUDA(cudaMalloc((void **)ptr, take));
  ctx->cap[(const void *)*ptr] = take;
  ctx->bytes += take;
  return GMHD_OK;
}

void
release_amr(gmhd_ctx * c)
{
  drelease(c, &c->d_kind);
  drelease(c, &c->d_fine);
  drelease(c, &c->d_fine_at);
  drelease(c, &c->d_fine_id);
  drelease(c, &c->d_coord);
  drelease(c, &c->d_vmap);
  drelease(c, &c->d_nbr_real);
  drelease(c, &c->d_list1);
  drelease(c, &c->d_list2);
  drelease(c, &c->d_flux_slot);
  drelease(c, &c->d_emf_slot);
  drelease(c, &c->d_Uv);
  drelease(c, &c->d_Bv);
  drelease(c, &c->d_Bccv);
  drelease(c, &c->d_flux_side);
  drelease(c, &c->d_emf_side);
}

// forget the mesh (tables, graph, coarse/fine state) but keep the device buffers
void
reset_mesh(gmhd_ctx * c)
{
  c->amr = false;
  c->n_virtual = c->n_list1 = c->n_list2 = c->flux_face_stride = 0;
  if (c->graph_exec)
  {
    cudaGraphExecDestroy(c->graph_exec);
    c->graph_exec = nullptr;
  }
  c->has_mesh = false;
}

void
release_all(gmhd_ctx * c)
{
  reset_mesh(c);
  for (int32_t ** p : {&c->d_neighbor, &c->d_level, &c->d_problem, &c->d_out_src, &c->d_out_normal, &c->d_counter,
                       &c->d_hp_blocks, &c->d_hp_tiles})
    drelease(c, p);
  drelease(c, &c->d_invdt);
  for (double ** p : {&c->d_dt, &c->d_t, &c->d_tend, &c->d_dtlog, &c->d_U, &c->d_U2, &c->d_B, &c->d_B2, &c->d_Urk,
                      &c->d_Brk})
    drelease(c, p);
  for (int k = 0; k < 2; ++k)
    for (double ** p : {&c->a_U[k], &c->a_U2[k], &c->a_B[k], &c->a_B2[k]})
      drelease(c, p);
  release_amr(c);
  drelease(c, &c->d_rf_q);
  drelease(c, &c->d_rf_flags);
  c->dtlog_cap = 0;
}

gmhd::Sources
sources_of(const gmhd_params & p)
{
  gmhd::Sources src;
  std::memset(&src, 0, sizeof src);
  src.gravity = p.gravity_enabled != 0;
  for (int d = 0; d < 3; ++d)
    src.g[d] = src.gravity ? p.gravity[d] : 0.0;
  src.viscosity = p.viscosity_enabled != 0;
  src.mu = src.viscosity ? p.viscosity_mu : 0.0;
  src.visc_predictor = src.viscosity && p.viscous_predictor != 0;
  return src;
}

gmhd::StepArgs
make_args(const gmhd_ctx * c, const double * U, double * U2, const double * B, double * B2)
{
  gmhd::StepArgs a;
  std::memset(&a, 0, sizeof a);
  a.U = U;
  a.U2 = U2;
  a.B = B;
  a.B2 = B2;
  a.neighbor = c->d_neighbor;
  a.level = c->d_level;
  a.problem = c->d_problem;
  a.n_owned = c->n_owned;
  a.tile = c->tile;
  a.bx = c->bx;
  a.by = c->by;
  a.bz = c->bz;
  a.ncell = c->ncell;
  a.nfx = c->nfx;
  a.nfy = c->nfy;
  a.nface = c->nface;
  a.gamma0 = c->p.gamma0;
  a.smallr = c->p.smallr;
  a.smallc = c->p.smallc;
  a.smallp = c->smallp;
  a.slope_type = c->p.slope_type;
  a.scaling_factor = c->p.scaling_factor;
  a.cfl = c->p.cfl;
  a.riemann = c->p.riemann;
  a.gamma0_f = (float)a.gamma0;
  a.smallr_f = (float)a.smallr;
  a.smallc_f = (float)a.smallc;
  a.smallp_f = (float)a.smallp;
  a.slope_type_f = (float)a.slope_type;
  a.rk2 = c->p.time_integrator == GMHD_TIME_RK2_SSP;
  a.health = c->d_health;
  a.n_blocks = c->n_blocks;
  a.src = sources_of(c->p);
  return a;
}

int
launch_one(gmhd_ctx * ctx, const gmhd::StepArgs & a, cudaStream_t s)
{
  const int rc = ctx->p.precision == GMHD_PRECISION_MIXED ? gmhd::launch_step_mixed(a, ctx->dim, s)
                                                          : gmhd::launch_step_fp64(a, ctx->dim, s);
  if (rc == -1)
    return GMHD_ERR_ARGUMENT;
  if (rc != 0)
    return cuda_fail(ctx, (cudaError_t)rc);
  return GMHD_OK;
}

// One do_time_step. On coarse/fine meshes: the ghost prepass (virtual neighbour blocks from U, B),
// then pass 1 (tiles without finer neighbours; fine-side fluxes and EMFs) and pass 2 (tiles next to
// finer blocks, reading them).
int
launch_step(gmhd_ctx * ctx, const gmhd::StepArgs & a0, cudaStream_t s)
{
  if (!ctx->amr)
    return launch_one(ctx, a0, s);
  gmhd::GhostArgs g;
  std::memset(&g, 0, sizeof g);
  g.U = a0.U;
  g.B = a0.B;
  g.Uv = ctx->d_Uv;
  g.Bv = ctx->d_Bv;
  g.Bccv = ctx->d_Bccv;
  g.vmap = ctx->d_vmap;
  g.neighbor = ctx->d_nbr_real;
  g.kind = ctx->d_kind;
  g.fine = ctx->d_fine;
  g.coord = ctx->d_coord;
  g.n_virtual = ctx->n_virtual;
  g.dim = ctx->dim;
  g.bx = ctx->bx;
  g.by = ctx->by;
  g.bz = ctx->bz;
  g.prolongation = ctx->p.prolongation;
  g.ncell = ctx->ncell;
  g.nfx = ctx->nfx;
  g.nfy = ctx->nfy;
  g.nface = ctx->nface;
  g.health = ctx->d_health;
  int rc = gmhd::launch_ghost_prepass(g, s);
  if (rc != 0)
    return cuda_fail(ctx, (cudaError_t)rc);
  gmhd::StepArgs a = a0;
  a.kind = ctx->d_kind;
  a.fine = ctx->d_fine;
  a.Uv = ctx->d_Uv;
  a.Bv = ctx->d_Bv;
  a.Bccv = ctx->d_Bccv;
  a.prolongation = ctx->p.prolongation;
  a.flux_side = ctx->d_flux_side;
  a.flux_slot = ctx->d_flux_slot;
  a.flux_face_stride = ctx->flux_face_stride;
  a.emf_side = ctx->d_emf_side;
  a.emf_slot = ctx->d_emf_slot;
  if (ctx->n_list1 > 0)
  {
    a.pass = 1;
    a.tile_list = ctx->d_list1;
    a.n_list = ctx->n_list1;
    if ((rc = launch_one(ctx, a, s)))
      return rc;
  }
  if (ctx->n_list2 > 0)
  {
    a.pass = 2;
    a.tile_list = ctx->d_list2;
    a.n_list = ctx->n_list2;
    if ((rc = launch_one(ctx, a, s)))
      return rc;
  }
  return GMHD_OK;
}

// the fused step reads U and B in 16-byte pairs
bool
misaligned(const void * p)
{
  return ((uintptr_t)p & 15u) != 0;
}

bool
overlaps(const void * a, size_t na, const void * b, size_t nb)
{
  const char * pa = (const char *)a;
  const char * pb = (const char *)b;
  return pa < pb + nb && pb < pa + na;
}

// ---- outside-block fill (border_conditions/FillOutside.cpp:97-395) ---------------------------
struct FillArgs
{
  double *        U;
  double *        B;
  const int32_t * src;
  const int32_t * normal;
  int             n_owned, n_outside, dim, bx, by, bz;
  int64_t         ncell, nfx, nfy, nfz, nface;
  int             bc[6];
};

__global__ void
fill_outside_hydro_kernel(FillArgs a)
{
  const int64_t total = (int64_t)a.n_outside * a.ncell;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x)
  {
    const int     o = (int)(g / a.ncell);
    const int64_t c = g - (int64_t)o * a.ncell;
    const int     out_blk = a.n_owned + o;
    const int     in_blk = a.src[o];
    int           co[3] = {(int)(c % a.bx), (int)((c / a.bx) % a.by), (int)(c / ((int64_t)a.bx * a.by))};
    const int     bs[3] = {a.bx, a.by, a.bz};
    for (int face = 0; face < 2 * a.dim; ++face)
    {
      const int d = face / 2;
      const int nrm = a.normal[3 * o + d];
      // the inside block touches the domain border of this face and the outside block lies across it
      const bool applies = (face % 2 == 0) ? (nrm > 0) : (nrm < 0);
      if (!applies)
        continue;
      int ci[3] = {co[0], co[1], co[2]};
      if (a.bc[face] == GMHD_BC_ZERO_GRADIENT)
        ci[d] = (face % 2 == 0) ? 0 : bs[d] - 1;
      else if (a.bc[face] == GMHD_BC_WALL)
        ci[d] = bs[d] - 1 - co[d];
      else
        continue;
      const int64_t cin = ci[0] + (int64_t)a.bx * (ci[1] + (int64_t)a.by * ci[2]);
      for (int v = 0; v < 5; ++v)
        a.U[((int64_t)out_blk * 5 + v) * a.ncell + c] = a.U[((int64_t)in_blk * 5 + v) * a.ncell + cin];
      if (a.bc[face] == GMHD_BC_WALL)
        a.U[((int64_t)out_blk * 5 + 2 + d) * a.ncell + c] *= -1;
    }
  }
}

__global__ void
fill_outside_faces_kernel(FillArgs a)
{
  const int64_t total = (int64_t)a.n_outside * a.nface;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x)
  {
    const int     o = (int)(g / a.nface);
    const int64_t f = g - (int64_t)o * a.nface;
    const int     out_blk = a.n_owned + o;
    const int     in_blk = a.src[o];
    // unravel (component, i, j, k) of the face
    int  comp;
    int64_t r;
    int  nx, ny;
    if (f < a.nfx)
    {
      comp = 0; r = f; nx = a.bx + 1; ny = a.by;
    }
    else if (f < a.nfx + a.nfy)
    {
      comp = 1; r = f - a.nfx; nx = a.bx; ny = a.by + 1;
    }
    else
    {
      comp = 2; r = f - a.nfx - a.nfy; nx = a.bx; ny = a.by;
    }
    int       idx[3] = {(int)(r % nx), (int)((r / nx) % ny), (int)(r / ((int64_t)nx * ny))};
    const int fsz[3] = {nx, ny, comp == 2 && a.dim == 3 ? a.bz + 1 : a.bz};
    for (int d = 0; d < a.dim; ++d)
    {
      const int nrm = a.normal[3 * o + d];
      if (nrm > 0 && a.bc[2 * d] == GMHD_BC_ZERO_GRADIENT)
        idx[d] = 0;
      else if (nrm < 0 && a.bc[2 * d + 1] == GMHD_BC_ZERO_GRADIENT)
        idx[d] = fsz[d] - 1;
      // WALL: the reference leaves the index unchanged (a TODO), i.e. copies the same face
    }
    const int64_t fin = idx[0] + (int64_t)nx * (idx[1] + (int64_t)ny * idx[2]);
    const int64_t base = comp == 0 ? 0 : (comp == 1 ? a.nfx : a.nfx + a.nfy);
    a.B[(int64_t)out_blk * a.nface + f] = a.B[(int64_t)in_blk * a.nface + base + fin];
  }
}

// ---- device-side time control of gmhd_advance -----------------------------------------------
__global__ void
advance_time_kernel(const unsigned long long * invdt, double cfl, double * t, const double * t_end, double * dt_cur,
                    double * dt_log, int32_t * counter, int np, int64_t log_cap, int skip_ok)
{
  const int n = *counter;
  for (int p = threadIdx.x; p < np; p += blockDim.x)
  {
    double dt = cfl / __longlong_as_double((long long)invdt[p]);
    if (t_end)
    {
      const double rem = t_end[p] - t[p];
      if (dt > rem)
        dt = rem;
      if (!(rem > 0.0))
        dt = 0.0;
    }
    if ((int64_t)(n + 1) * np <= log_cap)
      dt_log[(int64_t)n * np + p] = dt;
    // A problem past its end time is copied through by the step (dt = +0). After one such step both
    // state buffers of the ping-pong hold its final state, so the next steps leave it alone: dt = -0
    // tells the step to skip its tiles (Hancock loop only; gmhd_advance resets dt_cur to NaN when it
    // starts, so the first step of a call always copies through).
    if (skip_ok && dt == 0.0 && dt_cur[p] == 0.0)
      dt = -0.0;
    dt_cur[p] = dt;
    t[p] += dt;
  }
  __syncthreads();
  if (threadIdx.x == 0)
    *counter = n + 1;
}

int
enqueue_fill(gmhd_ctx * ctx, double * U, double * B, cudaStream_t s)
{
  if (ctx->n_outside == 0)
    return GMHD_OK;
  FillArgs f;
  f.U = U;
  f.B = B;
  f.src = ctx->d_out_src;
  f.normal = ctx->d_out_normal;
  f.n_owned = ctx->n_owned;
  f.n_outside = ctx->n_outside;
  f.dim = ctx->dim;
  f.bx = ctx->bx;
  f.by = ctx->by;
  f.bz = ctx->bz;
  f.ncell = ctx->ncell;
  f.nfx = ctx->nfx;
  f.nfy = ctx->nfy;
  f.nfz = ctx->nfz;
  f.nface = ctx->nface;
  for (int i = 0; i < 6; ++i)
    f.bc[i] = ctx->bc[i];
  const int64_t nh = (int64_t)ctx->n_outside * ctx->ncell;
  const int64_t nf = (int64_t)ctx->n_outside * ctx->nface;
  const int     gh = (int)((nh + 255) / 256 < 65535 ? (nh + 255) / 256 : 65535);
  const int     gf = (int)((nf + 255) / 256 < 65535 ? (nf + 255) / 256 : 65535);
  // hydro and faces touch disjoint arrays: one after the other on the same stream
  fill_outside_hydro_kernel<<<gh, 256, 0, s>>>(f);
  fill_outside_faces_kernel<<<gf, 256, 0, s>>>(f);
  GMHD_CUDA(cudaGetLastError());
  return GMHD_OK;
}

// exact: FP64 with the reference operand order (gmhd_inv_dt); otherwise the precision of the
// context's step (the mixed solver loop seeds dt with an FP32 estimate)
int
enqueue_inv_dt(gmhd_ctx * ctx, const double * U, const double * B, unsigned long long * slot, cudaStream_t s,
               bool exact = true)
{
  GMHD_CUDA(cudaMemsetAsync(slot, 0, sizeof(unsigned long long) * ctx->n_problems, s));
  auto launch = (exact || ctx->p.precision != GMHD_PRECISION_MIXED) ? gmhd::launch_inv_dt : gmhd::launch_inv_dt_mixed;
  const int rc = launch(U, B, ctx->d_level, ctx->d_problem, ctx->n_owned, ctx->dim, ctx->bx, ctx->by,
                                     ctx->bz, ctx->ncell, ctx->nfx, ctx->nfy, ctx->nface, ctx->p.gamma0,
                                     ctx->p.smallr, ctx->smallp, ctx->p.scaling_factor, sources_of(ctx->p), slot, s);
  if (rc != 0)
    return cuda_fail(ctx, (cudaError_t)rc);
  return GMHD_OK;
}

// LinearCombination (core; SolverGodunovMHD.cpp:617-621): out = c0 * a + c1 * out over the owned blocks
__global__ void
lincomb_kernel(const double * __restrict__ a, double * __restrict__ out, int64_t n, double c0, double c1)
{
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = c0 * a[i] + c1 * out[i];
}

int
enqueue_lincomb(gmhd_ctx * ctx, const double * a, double * out, int64_t n, double c0, double c1, cudaStream_t s)
{
  if (n <= 0)
    return GMHD_OK;
  const int64_t want = (n + 255) / 256;
  lincomb_kernel<<<(int)(want < 152 * 64 ? want : 152 * 64), 256, 0, s>>>(a, out, n, c0, c1);
  GMHD_CUDA(cudaGetLastError());
  return GMHD_OK;
}

// one RK2_SSP iteration of gmhd_advance (SolverGodunovMHD.cpp:551-647): U_RK = U + L(U);
// U2 = U_RK + L(U_RK); U2 = 1/2 U + 1/2 U2; CFL of U2 for the next iteration. The stage-1 combination
// (coefficients 0 and 1) leaves U_RK unchanged and is not launched.
int
enqueue_iteration_rk2(gmhd_ctx * ctx, const double * Uc, double * Un, const double * Bc, double * Bn, int slot_in,
                      cudaStream_t s, bool has_tend)
{
  const int np = ctx->n_problems;
  advance_time_kernel<<<1, 256, 0, s>>>(ctx->d_invdt + (size_t)slot_in * np, ctx->p.cfl, ctx->d_t,
                                        has_tend ? ctx->d_tend : nullptr, ctx->d_dt, ctx->d_dtlog, ctx->d_counter,
                                        np, ctx->dtlog_cap, 0);
  GMHD_CUDA(cudaGetLastError());
  int rc = enqueue_fill(ctx, const_cast<double *>(Uc), const_cast<double *>(Bc), s);
  if (rc)
    return rc;
  gmhd::StepArgs a = make_args(ctx, Uc, ctx->d_Urk, Bc, ctx->d_Brk);
  a.dt_dev = ctx->d_dt;
  if ((rc = launch_step(ctx, a, s)))
    return rc;
  if ((rc = enqueue_fill(ctx, ctx->d_Urk, ctx->d_Brk, s)))
    return rc;
  a = make_args(ctx, ctx->d_Urk, Un, ctx->d_Brk, Bn);
  a.dt_dev = ctx->d_dt;
  if ((rc = launch_step(ctx, a, s)))
    return rc;
  if ((rc = enqueue_lincomb(ctx, Uc, Un, (int64_t)ctx->n_owned * 5 * ctx->ncell, 0.5, 0.5, s)) ||
      (rc = enqueue_lincomb(ctx, Bc, Bn, (int64_t)ctx->n_owned * ctx->nface, 0.5, 0.5, s)))
    return rc;
  return enqueue_inv_dt(ctx, Un, Bn, ctx->d_invdt + (size_t)(1 - slot_in) * np, s,
                        ctx->p.precision != GMHD_PRECISION_MIXED);
}

// one solver iteration of gmhd_advance: time control, outside fill, fused step + CFL
int
enqueue_iteration(gmhd_ctx * ctx, const double * Uc, double * Un, const double * Bc, double * Bn, int slot_in,
                  cudaStream_t s, bool has_tend)
{
  if (ctx->p.time_integrator == GMHD_TIME_RK2_SSP)
    return enqueue_iteration_rk2(ctx, Uc, Un, Bc, Bn, slot_in, s, has_tend);
  const int np = ctx->n_problems;
  advance_time_kernel<<<1, 256, 0, s>>>(ctx->d_invdt + (size_t)slot_in * np, ctx->p.cfl, ctx->d_t,
                                        has_tend ? ctx->d_tend : nullptr, ctx->d_dt, ctx->d_dtlog, ctx->d_counter,
                                        np, ctx->dtlog_cap, 1);
  GMHD_CUDA(cudaGetLastError());
  unsigned long long * out = ctx->d_invdt + (size_t)(1 - slot_in) * np;
  GMHD_CUDA(cudaMemsetAsync(out, 0, sizeof(unsigned long long) * np, s));
  int rc = enqueue_fill(ctx, const_cast<double *>(Uc), const_cast<double *>(Bc), s);
  if (rc)
    return rc;
  gmhd::StepArgs a = make_args(ctx, Uc, Un, Bc, Bn);
  a.dt_dev = ctx->d_dt;
  a.invdt_out = out;
  return launch_step(ctx, a, s);
}

int
check_health(gmhd_ctx * ctx, cudaStream_t s, unsigned int * flags_out)
{
  unsigned int h = 0;
  GMHD_CUDA(cudaMemcpyAsync(&h, ctx->d_health, sizeof h, cudaMemcpyDeviceToHost, s));
  GMHD_CUDA(cudaMemsetAsync(ctx->d_health, 0, sizeof(unsigned int), s));
  GMHD_CUDA(cudaStreamSynchronize(s));
  if (flags_out)
    *flags_out = h;
  return GMHD_OK;
}

// The two-pass tile lists of a coarse/fine mesh for the context's tile choice: pass 1 takes the tiles
// without finer neighbours (and, marked ~id, the coarse-side stores of tiles that also border finer
// blocks), pass 2 the tiles next to finer blocks. Host side only (ctx->h_list1, ctx->h_list2).
void
build_tile_lists(gmhd_ctx * ctx, int dim, const std::vector<int8_t> & kind)
{
  int T[3];
  if (ctx->p.precision == GMHD_PRECISION_MIXED)
    gmhd::tile_shape_mixed(dim, ctx->bx, ctx->by, ctx->bz, ctx->p.viscosity_enabled != 0, true, ctx->tile, T);
  else
    gmhd::tile_shape_fp64(dim, ctx->bx, ctx->by, ctx->bz, ctx->p.viscosity_enabled != 0, ctx->tile, T);
  const int              nt[3] = {ctx->bx / T[0], ctx->by / T[1], dim == 3 ? ctx->bz / T[2] : 1};
  const int              tpb = nt[0] * nt[1] * nt[2];
  std::vector<int32_t> & list1 = ctx->h_list1;
  std::vector<int32_t> & list2 = ctx->h_list2;
  list1.clear();
  list2.clear();
  // the neighbour slots a tile touches depend only on where it sits in the block along each axis (first,
  // last, or both when the block is one tile wide, or neither): one 27-bit mask per position class
  auto cls_of = [&](int c, int n) { return (c == 0 ? 1 : 0) | (c == n - 1 ? 2 : 0); };
  uint32_t touch[64];
  for (int cz = 0; cz < 4; ++cz)
    for (int cy = 0; cy < 4; ++cy)
      for (int cx = 0; cx < 4; ++cx)
      {
        const int cl[3] = {cx, cy, cz};
        uint32_t  m = 0;
        for (int s = 0; s < 27; ++s)
        {
          if (s == 13 || (dim == 2 && s / 9 != 1))
            continue;
          const int o[3] = {s % 3 - 1, (s / 3) % 3 - 1, s / 9 - 1};
          bool      t = true;
          for (int d = 0; d < 3; ++d)
            if (o[d] != 0 && !(cl[d] & (o[d] < 0 ? 1 : 2)))
              t = false;
          if (t)
            m |= 1u << s;
        }
        touch[cx + 4 * (cy + 4 * cz)] = m;
      }
  for (int b = 0; b < ctx->n_owned; ++b)
  {
    uint32_t finer = 0, coarser = 0;
    for (int s = 0; s < 27; ++s)
    {
      finer |= (kind[(size_t)b * 27 + s] == gmhd::RK_FINER ? 1u : 0u) << s;
      coarser |= (kind[(size_t)b * 27 + s] == gmhd::RK_COARSER ? 1u : 0u) << s;
    }
    for (int t = 0; t < tpb; ++t)
    {
      const int      tc[3] = {t % nt[0], (t / nt[0]) % nt[1], t / (nt[0] * nt[1])};
      const uint32_t m = touch[cls_of(tc[0], nt[0]) + 4 * (cls_of(tc[1], nt[1]) + 4 * cls_of(tc[2], nt[2]))];
      const bool     fin = (finer & m) != 0, coa = (coarser & m) != 0;
      const int32_t  id = b * tpb + t;
      if (!fin)
        list1.push_back(id);
      else
      {
        if (coa)
          list1.push_back(~id);
        list2.push_back(id);
      }
    }
  }
}

// Make `tile` the context's tile request; on a coarse/fine mesh rebuild and upload the tile lists for
// it (the caller has made sure no step still reads them).
int
apply_tile(gmhd_ctx * ctx, int tile)
{
  ctx->tile = tile;
  if (!ctx->has_mesh || !ctx->amr)
    return GMHD_OK;
  build_tile_lists(ctx, ctx->dim, ctx->h_kind);
  int rc;
  if ((rc = dalloc(ctx, &ctx->d_list1, ctx->h_list1.size())) || (rc = dalloc(ctx, &ctx->d_list2, ctx->h_list2.size())))
    return rc;
  up_copy(ctx, ctx->d_list1, ctx->h_list1.data(), sizeof(int32_t) * ctx->h_list1.size());
  up_copy(ctx, ctx->d_list2, ctx->h_list2.data(), sizeof(int32_t) * ctx->h_list2.size());
  ctx->n_list1 = (int)ctx->h_list1.size();
  ctx->n_list2 = (int)ctx->h_list2.size();
  return up_flush(ctx);
}

// Coarse/fine tables: virtual blocks for every neighbour region read through the ghost prepass,
// the kernel's neighbour table pointing at them, fine-side data slots and the two tile lists.
int
setup_amr(gmhd_ctx * ctx, const gmhd_mesh * m, const std::vector<int8_t> & kind)
{
  auto lev = [](int k) { return k == gmhd::RK_COARSER ? -1 : (k == gmhd::RK_FINER ? 1 : (k == gmhd::RK_MISSING ? -100 : 0)); };
  auto slot_of = [](const int * o) { return (o[2] + 1) * 9 + (o[1] + 1) * 3 + (o[0] + 1); };
  const int              nown = m->n_owned;
  std::vector<int32_t> & knbr = ctx->h_knbr;
  std::vector<int32_t> & vmap = ctx->h_vmap;
  std::vector<int32_t> & flux_slot = ctx->h_flux_slot;
  std::vector<int32_t> & emf_slot = ctx->h_emf_slot;
  knbr.assign(m->neighbor, m->neighbor + (size_t)m->n_blocks * 27);
  vmap.clear();
  flux_slot.assign(nown, -1);
  emf_slot.assign(nown, -1);
  int n_flux = 0, n_emf = 0;
  for (int b = 0; b < nown; ++b)
  {
    bool coarser_face = false, coarser_any = false;
    for (int s = 0; s < 27; ++s)
    {
      if (s == 13 || (m->dim == 2 && s / 9 != 1))
        continue;
      const int o[3] = {s % 3 - 1, (s / 3) % 3 - 1, s / 9 - 1};
      const int k = kind[(size_t)b * 27 + s];
      bool      virt = k == gmhd::RK_COARSER || k == gmhd::RK_FINER;
      if (k == gmhd::RK_COARSER)
      {
        coarser_any = true;
        coarser_face = coarser_face || (std::abs(o[0]) + std::abs(o[1]) + std::abs(o[2]) == 1);
      }
      // a same-level region whose border faces (along a normal) must come from a finer region
      if (!virt && (k == gmhd::RK_SAME || k == gmhd::RK_OUTSIDE))
        for (int c = 0; c < m->dim && !virt; ++c)
        {
          if (o[c] != 0)
            continue;
          for (int sg = -1; sg <= 1 && !virt; sg += 2)
          {
            int o1[3] = {o[0], o[1], o[2]};
            o1[c] = sg;
            virt = lev(kind[(size_t)b * 27 + slot_of(o1)]) > lev(k);
          }
        }
      if (virt)
      {
        knbr[(size_t)b * 27 + s] = m->n_blocks + (int32_t)(vmap.size() / 2);
        vmap.push_back(b);
        vmap.push_back(s);
      }
    }
    if (coarser_face)
      flux_slot[b] = n_flux++;
    if (coarser_any)
      emf_slot[b] = n_emf++;
  }
  build_tile_lists(ctx, m->dim, kind);
  const int     nv = (int)(vmap.size() / 2);
  const int     ncomp = m->dim == 3 ? 3 : 1;
  const int64_t ne = (int64_t)(ctx->bx + 1) * (ctx->by + 1) * (m->dim == 3 ? ctx->bz + 1 : 1);
  // hydro flux vars of the update, plus the 4 viscous ones (E and the momenta) with viscosity
  const int     nfv = (m->dim == 3 ? 5 : 6) + (ctx->p.viscosity_enabled ? 4 : 0);
  ctx->flux_face_stride = m->dim == 3 ? std::max(ctx->by * ctx->bz, std::max(ctx->bx * ctx->bz, ctx->bx * ctx->by))
                                      : std::max(ctx->bx, ctx->by);
  int rc;
  if ((rc = dalloc(ctx, &ctx->d_kind, kind.size())) || (rc = dalloc(ctx, &ctx->d_nbr_real, knbr.size())) ||
      (rc = dalloc(ctx, &ctx->d_vmap, vmap.size())) || (rc = dalloc(ctx, &ctx->d_list1, ctx->h_list1.size())) ||
      (rc = dalloc(ctx, &ctx->d_list2, ctx->h_list2.size())) || (rc = dalloc(ctx, &ctx->d_flux_slot, (size_t)nown)) ||
      (rc = dalloc(ctx, &ctx->d_emf_slot, (size_t)nown)) || (rc = dalloc(ctx, &ctx->d_coord, (size_t)m->n_blocks * 3)) ||
      (rc = dalloc(ctx, &ctx->d_fine, (size_t)m->n_blocks * 27 * 8)) ||
      (rc = dalloc(ctx, &ctx->d_Uv, (size_t)nv * 5 * ctx->ncell)) || (rc = dalloc(ctx, &ctx->d_Bv, (size_t)nv * ctx->nface)) ||
      (rc = dalloc(ctx, &ctx->d_Bccv, (size_t)nv * 3 * ctx->ncell)) ||
      (rc = dalloc(ctx, &ctx->d_flux_side, (size_t)n_flux * 2 * m->dim * nfv * ctx->flux_face_stride)) ||
      (rc = dalloc(ctx, &ctx->d_emf_side, (size_t)n_emf * ncomp * ne)))
    return rc;
  up_copy(ctx, ctx->d_kind, kind.data(), kind.size());
  // the real table for the prepass; the kernel's table with the virtual ids
  up_copy(ctx, ctx->d_nbr_real, m->neighbor, sizeof(int32_t) * knbr.size());
  up_copy(ctx, ctx->d_neighbor, knbr.data(), sizeof(int32_t) * knbr.size());
  up_copy(ctx, ctx->d_vmap, vmap.data(), sizeof(int32_t) * vmap.size());
  up_copy(ctx, ctx->d_list1, ctx->h_list1.data(), sizeof(int32_t) * ctx->h_list1.size());
  up_copy(ctx, ctx->d_list2, ctx->h_list2.data(), sizeof(int32_t) * ctx->h_list2.size());
  up_copy(ctx, ctx->d_flux_slot, flux_slot.data(), sizeof(int32_t) * nown);
  up_copy(ctx, ctx->d_emf_slot, emf_slot.data(), sizeof(int32_t) * nown);
  if (m->coord)
    up_copy(ctx, ctx->d_coord, m->coord, sizeof(int32_t) * m->n_blocks * 3);
  else
    up_set(ctx, ctx->d_coord, 0, sizeof(int32_t) * m->n_blocks * 3);
  if (m->fine_neighbor)
    up_copy(ctx, ctx->d_fine, m->fine_neighbor, sizeof(int32_t) * m->n_blocks * 27 * 8);
  else
  {
    up_set(ctx, ctx->d_fine, 0xff, sizeof(int32_t) * m->n_blocks * 27 * 8);
    if (m->n_fine > 0)
    {
      if ((rc = dalloc(ctx, &ctx->d_fine_at, (size_t)m->n_fine)) || (rc = dalloc(ctx, &ctx->d_fine_id, (size_t)m->n_fine)))
        return rc;
      up_copy(ctx, ctx->d_fine_at, m->fine_at, sizeof(int64_t) * (size_t)m->n_fine);
      up_copy(ctx, ctx->d_fine_id, m->fine_id, sizeof(int32_t) * (size_t)m->n_fine);
      ctx->fine_scatter = m->n_fine;
    }
  }
  up_set(ctx, ctx->d_Uv, 0, sizeof(double) * (size_t)nv * 5 * ctx->ncell);
  up_set(ctx, ctx->d_Bv, 0, sizeof(double) * (size_t)nv * ctx->nface);
  up_set(ctx, ctx->d_Bccv, 0, sizeof(double) * (size_t)nv * 3 * ctx->ncell);
  ctx->amr = true;
  ctx->n_virtual = nv;
  ctx->n_list1 = (int)ctx->h_list1.size();
  ctx->n_list2 = (int)ctx->h_list2.size();
  return GMHD_OK;
}

} // namespace

extern "C" {

gmhd_ctx *
gmhd_create(const gmhd_params * params)
{
  if (!params || !(params->gamma0 > 1.0) || !(params->cfl > 0.0) || !(params->scaling_factor > 0.0))
    return nullptr;
  if (params->riemann < GMHD_RIEMANN_LLF || params->riemann > GMHD_RIEMANN_HLLD)
    return nullptr;
  if (params->precision != GMHD_PRECISION_FP64 && params->precision != GMHD_PRECISION_MIXED)
    return nullptr;
  if (params->prolongation != GMHD_PROLONG_SIMPLE_COPY && params->prolongation != GMHD_PROLONG_LINEAR_MINMOD)
    return nullptr;
  if (params->time_integrator != GMHD_TIME_HANCOCK && params->time_integrator != GMHD_TIME_RK2_SSP)
    return nullptr;
  if (params->gravity_enabled &&
      !(std::isfinite(params->gravity[0]) && std::isfinite(params->gravity[1]) && std::isfinite(params->gravity[2])))
    return nullptr;
  if (params->viscosity_enabled && !(params->viscosity_mu >= 0.0 && std::isfinite(params->viscosity_mu)))
    return nullptr;
  gmhd_ctx * c = new (std::nothrow) gmhd_ctx();
  if (!c)
    return nullptr;
  c->p = *params;
  c->smallp = params->smallc * params->smallc / params->gamma0;
  if (cudaGetDevice(&c->device) != cudaSuccess || cudaMalloc((void **)&c->d_health, sizeof(unsigned int)) != cudaSuccess ||
      cudaMemset(c->d_health, 0, sizeof(unsigned int)) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess)
  {
    if (c->d_health)
      cudaFree(c->d_health);
    delete c;
    return nullptr;
  }
  c->bytes = sizeof(unsigned int);
  if (gmhd::prepare_fp64() != 0 || gmhd::prepare_mixed() != 0 || gmhd::prepare_fp64_visc() != 0 ||
      gmhd::prepare_mixed_visc() != 0)
  {
    cudaFree(c->d_health);
    cudaStreamDestroy(c->own_stream);
    delete c;
    return nullptr;
  }
  return c;
}

void
gmhd_destroy(gmhd_ctx * ctx)
{
  if (!ctx)
    return;
  if (ctx->a_in)
    cudaStreamSynchronize(ctx->a_in);
  if (ctx->a_run)
    cudaStreamSynchronize(ctx->a_run);
  if (ctx->a_out)
    cudaStreamSynchronize(ctx->a_out);
  release_all(ctx);
  if (ctx->h_stage)
    cudaFreeHost(ctx->h_stage);
  if (ctx->d_health)
    cudaFree(ctx->d_health);
  if (ctx->own_stream)
    cudaStreamDestroy(ctx->own_stream);
  for (cudaStream_t st : {ctx->a_in, ctx->a_run, ctx->a_out})
    if (st)
      cudaStreamDestroy(st);
  for (int k = 0; k < 2; ++k)
    for (cudaEvent_t ev : {ctx->a_in_done[k], ctx->a_run_done[k], ctx->a_out_done[k]})
      if (ev)
        cudaEventDestroy(ev);
  for (int k = 0; k < gmhd_ctx::HP_MAX; ++k)
    for (cudaEvent_t ev : {ctx->hp_in[k], ctx->hp_run[k]})
      if (ev)
        cudaEventDestroy(ev);
  for (cudaEvent_t ev : {ctx->hp_start, ctx->hp_end})
    if (ev)
      cudaEventDestroy(ev);
  delete ctx;
}

// The chunk plan of gmhd_step_host (conforming meshes without outside blocks, at least 16 owned
// blocks). With block coordinates the chunks are slabs along the last axis (z in 3D, y in 2D): bucket
// k of 8 holds the blocks whose coordinate falls in the k-th eighth of their problem's extent, so that
// a slab needs only its own and the two adjacent slabs and most slabs can step while later ones are
// still being copied in; without coordinates, up to 8 contiguous ranges of block ids. The copy-in runs
// in chunk order, so chunk k waits for chunk hp_dep[k] (the highest chunk holding a neighbour of one of
// its blocks); chunks step in the order of that readiness. A chunk's blocks are copied as runs of
// consecutive ids, runs of equal length at a constant stride merged into one strided copy.
static int
plan_host_chunks(gmhd_ctx * ctx, const gmhd_mesh * m, bool amr)
{
  ctx->hp_k = 0;
  ctx->hp_tile_key = -1;
  ctx->hp_off.clear();
  ctx->hp_coff.clear();
  ctx->hp_dep.clear();
  ctx->hp_order.clear();
  ctx->hp_blocks.clear();
  ctx->hp_copy.clear();
  const int n = m->n_owned;
  if (amr || m->n_blocks != n || n < 16)
    return GMHD_OK;
  constexpr int        NB = gmhd_ctx::HP_MAX;
  std::vector<int>     bucket(n);
  if (m->coord)
  {
    const int             a = m->dim - 1;
    const int             np = m->problem ? m->n_problems : 1;
    std::vector<int32_t>  ext(np, 0);
    for (int b = 0; b < n; ++b)
    {
      const int p = m->problem ? m->problem[b] : 0;
      ext[p] = std::max(ext[p], m->coord[3 * b + a] + 1);
    }
    for (int b = 0; b < n; ++b)
    {
      const int p = m->problem ? m->problem[b] : 0;
      const int c = std::max(0, m->coord[3 * b + a]);
      bucket[b] = (int)std::min<int64_t>(NB - 1, (int64_t)c * NB / std::max(1, ext[p]));
    }
  }
  else
    for (int b = 0; b < n; ++b)
      bucket[b] = (int)((int64_t)b * NB / n);
  // chunks: the non-empty buckets, in bucket order
  std::vector<int> chunk_of_bucket(NB, -1);
  std::vector<int> count(NB, 0);
  for (int b = 0; b < n; ++b)
    ++count[bucket[b]];
  int K = 0;
  for (int q = 0; q < NB; ++q)
    if (count[q])
      chunk_of_bucket[q] = K++;
  if (K < 2)
    return GMHD_OK;
  ctx->hp_off.assign(K + 1, 0);
  for (int q = 0; q < NB; ++q)
    if (count[q])
      ctx->hp_off[chunk_of_bucket[q] + 1] = count[q];
  for (int k = 0; k < K; ++k)
    ctx->hp_off[k + 1] += ctx->hp_off[k];
  ctx->hp_blocks.resize(n);
  std::vector<int> fill(ctx->hp_off.begin(), ctx->hp_off.end() - 1);
  std::vector<int> chunk_of(n);
  for (int b = 0; b < n; ++b) // ascending ids within each chunk
  {
    chunk_of[b] = chunk_of_bucket[bucket[b]];
    ctx->hp_blocks[fill[chunk_of[b]]++] = b;
  }
  ctx->hp_dep.assign(K, 0);
  for (int b = 0; b < n; ++b)
  {
    int & d = ctx->hp_dep[chunk_of[b]];
    d = std::max(d, chunk_of[b]);
    for (int sl = 0; sl < 27; ++sl)
    {
      const int nb = m->neighbor[(int64_t)b * 27 + sl];
      if (nb >= 0 && nb < n)
        d = std::max(d, chunk_of[nb]);
    }
  }
  ctx->hp_order.resize(K);
  for (int k = 0; k < K; ++k)
    ctx->hp_order[k] = k;
  std::stable_sort(ctx->hp_order.begin(), ctx->hp_order.end(),
                   [&](int x, int y) { return ctx->hp_dep[x] < ctx->hp_dep[y]; });
  ctx->hp_chunk.resize(n);
  ctx->hp_nchunk.assign((size_t)n * 27, (int8_t)-1);
  for (int b = 0; b < n; ++b)
  {
    ctx->hp_chunk[b] = (int8_t)chunk_of[b];
    for (int sl = 0; sl < 27; ++sl)
    {
      const int nb = m->neighbor[(int64_t)b * 27 + sl];
      if (nb >= 0 && nb < n)
        ctx->hp_nchunk[(size_t)b * 27 + sl] = (int8_t)chunk_of[nb];
    }
  }
  ctx->hp_tile_key = -1;
  // runs of consecutive ids, then runs of one length at one stride merged
  ctx->hp_coff.assign(1, 0);
  for (int k = 0; k < K; ++k)
  {
    std::vector<std::pair<int, int>> runs;
    for (int i = ctx->hp_off[k]; i < ctx->hp_off[k + 1]; ++i)
    {
      const int b = ctx->hp_blocks[i];
      if (!runs.empty() && runs.back().first + runs.back().second == b)
        ++runs.back().second;
      else
        runs.push_back({b, 1});
    }
    for (size_t r = 0; r < runs.size();)
    {
      gmhd_ctx::HostRuns h{runs[r].first, runs[r].second, 0, 1};
      size_t e = r + 1;
      if (e < runs.size() && runs[e].second == h.len)
      {
        h.stride = runs[e].first - h.start;
        while (e < runs.size() && runs[e].second == h.len && runs[e].first - runs[e - 1].first == h.stride)
          ++e;
        h.count = (int)(e - r);
      }
      ctx->hp_copy.push_back(h);
      r = e;
    }
    ctx->hp_coff.push_back((int)ctx->hp_copy.size());
  }
  int rc;
  if ((rc = dalloc(ctx, &ctx->d_hp_blocks, (size_t)n)))
    return rc;
  up_copy(ctx, ctx->d_hp_blocks, ctx->hp_blocks.data(), sizeof(int32_t) * (size_t)n);
  ctx->hp_k = K;
  return GMHD_OK;
}

int
gmhd_set_mesh(gmhd_ctx * ctx, const gmhd_mesh * m)
{
  if (!ctx || !m || !m->level || !m->neighbor)
    return GMHD_ERR_ARGUMENT;
  if ((m->dim != 2 && m->dim != 3) || m->bx < 4 || m->by < 4 || (m->dim == 3 && m->bz < 4) ||
      (m->dim == 2 && m->bz != 1))
    return GMHD_ERR_ARGUMENT;
  if (m->n_owned < 0 || m->n_blocks < m->n_owned)
    return GMHD_ERR_ARGUMENT;
  const int n_out = m->n_blocks - m->n_owned;
  if (n_out > 0 && (!m->outside_src || !m->outside_normal))
    return GMHD_ERR_ARGUMENT;
  const int np = m->problem ? m->n_problems : 1;
  if (np < 1)
    return GMHD_ERR_ARGUMENT;
  // validate tables on the host: indices in range, one level (uniform mesh) per problem
  for (int64_t i = 0; i < (int64_t)m->n_blocks * 27; ++i)
    if (m->neighbor[i] < -1 || m->neighbor[i] >= m->n_blocks)
      return GMHD_ERR_MESH;
  for (int b = 0; b < m->n_blocks; ++b)
  {
    if (m->level[b] < 0 || m->level[b] > 30)
      return GMHD_ERR_MESH;
    if (m->problem && (m->problem[b] < 0 || m->problem[b] >= np))
      return GMHD_ERR_MESH;
  }
  // the children list (read when there is no dense table): every entry checked, and the slots that have
  // children marked
  const bool           fine_list = !m->fine_neighbor && m->n_fine > 0;
  std::vector<uint8_t> has_child;
  if (!m->fine_neighbor && m->n_fine < 0)
    return GMHD_ERR_ARGUMENT;
  if (fine_list)
  {
    if (!m->fine_at || !m->fine_id)
      return GMHD_ERR_ARGUMENT;
    has_child.assign((size_t)m->n_owned * 27, 0);
    for (int64_t i = 0; i < m->n_fine; ++i)
    {
      const int64_t at = m->fine_at[i];
      const int64_t bs = at / 8;
      const int     b = (int)(bs / 27), c = (int)(at % 8), id = m->fine_id[i];
      if (at < 0 || b >= m->n_owned || c >= (1 << m->dim) || id < 0 || id >= m->n_owned)
        return GMHD_ERR_MESH;
      if (m->level[id] != m->level[b] + 1 || (m->problem && m->problem[id] != m->problem[b]))
        return GMHD_ERR_MESH;
      has_child[(size_t)bs] = 1;
    }
  }
  // kind of every neighbour region of the owned blocks (same level, one coarser, one finer, outside);
  // the fine-neighbour entries are checked where they are read (regions without a same-level or
  // coarser neighbour)
  ctx->uploads.clear();
  ctx->fine_scatter = 0;
  std::vector<int8_t> & kind = ctx->h_kind;
  kind.assign((size_t)m->n_owned * 27, (int8_t)gmhd::RK_MISSING);
  bool amr = false;
  for (int b = 0; b < m->n_owned; ++b)
    for (int s = 0; s < 27; ++s)
    {
      int8_t & k = kind[(size_t)b * 27 + s];
      if (s == 13)
      {
        k = gmhd::RK_SAME;
        continue;
      }
      if (m->dim == 2 && s / 9 != 1)
        continue;
      const int nb = m->neighbor[(int64_t)b * 27 + s];
      if (nb >= 0)
      {
        if (m->problem && m->problem[nb] != m->problem[b])
          return GMHD_ERR_MESH;
        if (nb >= m->n_owned)
        {
          if (m->level[nb] != m->level[b])
            return GMHD_ERR_MESH; // outside blocks are at the level of the block they serve
          k = gmhd::RK_OUTSIDE;
        }
        else if (m->level[nb] == m->level[b])
          k = gmhd::RK_SAME;
        else if (m->level[nb] == m->level[b] - 1 && m->coord)
        {
          k = gmhd::RK_COARSER;
          amr = true;
        }
        else
          return GMHD_ERR_MESH; // not 2:1 balanced, or a coarser neighbour without coordinates
        continue;
      }
      if (fine_list)
      {
        if (has_child[(size_t)b * 27 + s])
        {
          k = gmhd::RK_FINER;
          amr = true;
        }
        continue;
      }
      if (!m->fine_neighbor)
        continue;
      bool any = false;
      for (int c = 0; c < (1 << m->dim); ++c)
      {
        const int id = m->fine_neighbor[((int64_t)b * 27 + s) * 8 + c];
        if (id < -1 || id >= m->n_owned)
          return GMHD_ERR_MESH;
        if (id < 0)
          continue;
        if (m->level[id] != m->level[b] + 1 || (m->problem && m->problem[id] != m->problem[b]))
          return GMHD_ERR_MESH;
        any = true;
      }
      if (any)
      {
        k = gmhd::RK_FINER;
        amr = true;
      }
    }
  if (amr && (m->bx % 2 || m->by % 2 || (m->dim == 3 && m->bz % 2)))
    return GMHD_ERR_MESH;
  for (int o = 0; o < n_out; ++o)
    if (m->outside_src[o] < 0 || m->outside_src[o] >= m->n_owned)
      return GMHD_ERR_MESH;

  // work queued on any stream may still read the old tables: wait for it before reusing the buffers
  GMHD_CUDA(cudaDeviceSynchronize());
  reset_mesh(ctx);
  if (!amr)
    release_amr(ctx);
  if (!m->problem)
    drelease(ctx, &ctx->d_problem);
  ctx->dim = m->dim;
  ctx->bx = m->bx;
  ctx->by = m->by;
  ctx->bz = m->dim == 3 ? m->bz : 1;
  ctx->n_blocks = m->n_blocks;
  ctx->n_owned = m->n_owned;
  ctx->n_outside = n_out;
  ctx->n_problems = np;
  ctx->ncell = (int64_t)ctx->bx * ctx->by * ctx->bz;
  ctx->nfx = (int64_t)(ctx->bx + 1) * ctx->by * ctx->bz;
  ctx->nfy = (int64_t)ctx->bx * (ctx->by + 1) * ctx->bz;
  ctx->nfz = ctx->dim == 3 ? (int64_t)ctx->bx * ctx->by * (ctx->bz + 1) : ctx->ncell;
  ctx->nface = ctx->nfx + ctx->nfy + ctx->nfz;
  for (int i = 0; i < 6; ++i)
    ctx->bc[i] = m->bc[i];
  int rc;
  if ((rc = dalloc(ctx, &ctx->d_neighbor, (size_t)m->n_blocks * 27)) || (rc = dalloc(ctx, &ctx->d_level, (size_t)m->n_blocks)) ||
      (rc = dalloc(ctx, &ctx->d_invdt, (size_t)3 * np)) || (rc = dalloc(ctx, &ctx->d_dt, (size_t)np)) ||
      (rc = dalloc(ctx, &ctx->d_t, (size_t)np)) || (rc = dalloc(ctx, &ctx->d_tend, (size_t)np)) ||
      (rc = dalloc(ctx, &ctx->d_counter, 1)))
    return rc;
  up_copy(ctx, ctx->d_neighbor, m->neighbor, sizeof(int32_t) * m->n_blocks * 27);
  up_copy(ctx, ctx->d_level, m->level, sizeof(int32_t) * m->n_blocks);
  if (m->problem)
  {
    if ((rc = dalloc(ctx, &ctx->d_problem, (size_t)m->n_blocks)))
      return rc;
    up_copy(ctx, ctx->d_problem, m->problem, sizeof(int32_t) * m->n_blocks);
  }
  if (n_out > 0)
  {
    if ((rc = dalloc(ctx, &ctx->d_out_src, (size_t)n_out)) || (rc = dalloc(ctx, &ctx->d_out_normal, (size_t)3 * n_out)))
      return rc;
    up_copy(ctx, ctx->d_out_src, m->outside_src, sizeof(int32_t) * n_out);
    up_copy(ctx, ctx->d_out_normal, m->outside_normal, sizeof(int32_t) * 3 * n_out);
  }
  if (amr && (rc = setup_amr(ctx, m, kind)))
  {
    ctx->uploads.clear();
    return rc;
  }
  if ((rc = plan_host_chunks(ctx, m, amr)))
  {
    ctx->uploads.clear();
    return rc;
  }
  // all tables in one staged batch on own_stream, complete before any step reads them
  if ((rc = up_flush(ctx)))
    return rc;
  ctx->has_mesh = true;
  ctx->mesh_version++;
  return GMHD_OK;
}

uint64_t
gmhd_mem_bytes(const gmhd_ctx * ctx)
{
  return ctx ? ctx->bytes : 0;
}

int
gmhd_step(gmhd_ctx * ctx, const double * U, double * U2, const double * B, double * B2, double dt, void * stream)
{
  if (!ctx || !U || !U2 || !B || !B2)
    return GMHD_ERR_ARGUMENT;
  if (!ctx->has_mesh)
    return GMHD_ERR_MESH;
  if (!(dt >= 0.0) || misaligned(U) || misaligned(B))
    return GMHD_ERR_ARGUMENT;
  const size_t nu = sizeof(double) * (size_t)ctx->n_blocks * 5 * ctx->ncell;
  const size_t nb = sizeof(double) * (size_t)ctx->n_blocks * ctx->nface;
  if (overlaps(U, nu, U2, nu) || overlaps(B, nb, B2, nb) || overlaps(U2, nu, B, nb) || overlaps(B2, nb, U, nu))
    return GMHD_ERR_ALIAS;
  gmhd::StepArgs a = make_args(ctx, U, U2, B, B2);
  a.dt = dt;
  return launch_step(ctx, a, (cudaStream_t)stream);
}

int
gmhd_set_tile(gmhd_ctx * ctx, int32_t tile)
{
  if (!ctx || tile < 0)
    return GMHD_ERR_ARGUMENT;
  GMHD_CUDA(cudaDeviceSynchronize());
  const int rc = apply_tile(ctx, tile);
  ctx->mesh_version++; // cached step graphs hold the previous kernels
  return rc;
}

int
gmhd_autotune(gmhd_ctx * ctx, const double * U, double * U2, const double * B, double * B2, double dt,
              int32_t * tile_out, double * ms_out, void * stream)
{
  if (!ctx || !U || !U2 || !B || !B2)
    return GMHD_ERR_ARGUMENT;
  if (!ctx->has_mesh)
    return GMHD_ERR_MESH;
  if (!(dt >= 0.0) || misaligned(U) || misaligned(B))
    return GMHD_ERR_ARGUMENT;
  const size_t nu = sizeof(double) * (size_t)ctx->n_blocks * 5 * ctx->ncell;
  const size_t nb = sizeof(double) * (size_t)ctx->n_blocks * ctx->nface;
  if (overlaps(U, nu, U2, nu) || overlaps(B, nb, B2, nb) || overlaps(U2, nu, B, nb) || overlaps(B2, nb, U, nu))
    return GMHD_ERR_ALIAS;
  int       cand[3];
  const bool visc = ctx->p.viscosity_enabled != 0;
  const int n = ctx->p.precision == GMHD_PRECISION_MIXED
                  ? gmhd::tile_candidates_mixed(ctx->dim, ctx->bx, ctx->by, ctx->bz, visc, ctx->amr, cand)
                  : gmhd::tile_candidates_fp64(ctx->dim, ctx->bx, ctx->by, ctx->bz, visc, cand);
  if (n == 0)
    return GMHD_ERR_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t  e0 = nullptr, e1 = nullptr;
  // no step may still read the tile lists that a candidate replaces
  GMHD_CUDA(cudaDeviceSynchronize());
  GMHD_CUDA(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess)
  {
    cudaEventDestroy(e0);
    return cuda_fail(ctx, cudaErrorMemoryAllocation);
  }
  const int  prev = ctx->tile;
  int        best = cand[0], rc = GMHD_OK;
  double     best_ms = 0.0;
  auto       use_tile = [&](int tile) { return apply_tile(ctx, tile); };
  // every candidate: two steps to warm up, then five timed with events on the stream
  for (int i = 0; i < n && rc == GMHD_OK; ++i)
  {
    if ((rc = use_tile(cand[i])))
      break;
    gmhd::StepArgs a = make_args(ctx, U, U2, B, B2);
    a.dt = dt;
    for (int w = 0; w < 2 && rc == GMHD_OK; ++w)
      rc = launch_step(ctx, a, s);
    if (rc == GMHD_OK && (rc = cuda_fail(ctx, cudaEventRecord(e0, s))) == GMHD_OK)
    {
      for (int r = 0; r < 5 && rc == GMHD_OK; ++r)
        rc = launch_step(ctx, a, s);
    }
    if (rc == GMHD_OK && (rc = cuda_fail(ctx, cudaEventRecord(e1, s))) == GMHD_OK &&
        (rc = cuda_fail(ctx, cudaEventSynchronize(e1))) == GMHD_OK)
    {
      float ms = 0.0f;
      if ((rc = cuda_fail(ctx, cudaEventElapsedTime(&ms, e0, e1))) == GMHD_OK && (i == 0 || ms / 5.0 < best_ms))
      {
        best = cand[i];
        best_ms = ms / 5.0;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const cudaError_t es = cudaDeviceSynchronize();
  if (rc == GMHD_OK && es != cudaSuccess)
    rc = cuda_fail(ctx, es);
  const int rc2 = use_tile(rc == GMHD_OK ? best : prev);
  ctx->mesh_version++; // cached step graphs hold the previous kernels
  if (rc == GMHD_OK)
    rc = rc2;
  if (rc == GMHD_OK)
  {
    if (tile_out)
      *tile_out = best;
    if (ms_out)
      *ms_out = best_ms;
  }
  return rc;
}

int
gmhd_inv_dt(gmhd_ctx * ctx, const double * U, const double * B, double * inv_dt, void * stream)
{
  if (!ctx || !U || !B || !inv_dt)
    return GMHD_ERR_ARGUMENT;
  if (!ctx->has_mesh)
    return GMHD_ERR_MESH;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long * slot = ctx->d_invdt + (size_t)2 * ctx->n_problems;
  int                  rc = enqueue_inv_dt(ctx, U, B, slot, s);
  if (rc)
    return rc;
  std::vector<unsigned long long> h(ctx->n_problems);
  GMHD_CUDA(cudaMemcpyAsync(h.data(), slot, sizeof(unsigned long long) * ctx->n_problems, cudaMemcpyDeviceToHost, s));
  GMHD_CUDA(cudaStreamSynchronize(s));
  for (int p = 0; p < ctx->n_problems; ++p)
  {
    double v;
    std::memcpy(&v, &h[p], sizeof v);
    inv_dt[p] = v;
  }
  return GMHD_OK;
}

int
gmhd_fill_outside(gmhd_ctx * ctx, double * U, double * B, void * stream)
{
  if (!ctx || !U || !B)
    return GMHD_ERR_ARGUMENT;
  if (!ctx->has_mesh)
    return GMHD_ERR_MESH;
  return enqueue_fill(ctx, U, B, (cudaStream_t)stream);
}

int
gmhd_advance(gmhd_ctx * ctx, double * U, double * U2, double * B, double * B2, int32_t nsteps, double * t,
             const double * t_end, double * dt_log, int32_t use_graph, void * stream)
{
  if (!ctx || !U || !U2 || !B || !B2 || nsteps < 0)
    return GMHD_ERR_ARGUMENT;
  if (misaligned(U) || misaligned(U2) || misaligned(B) || misaligned(B2))
    return GMHD_ERR_ARGUMENT;
  if (!ctx->has_mesh)
    return GMHD_ERR_MESH;
  const size_t nu = sizeof(double) * (size_t)ctx->n_blocks * 5 * ctx->ncell;
  const size_t nb = sizeof(double) * (size_t)ctx->n_blocks * ctx->nface;
  if (overlaps(U, nu, U2, nu) || overlaps(B, nb, B2, nb) || overlaps(U2, nu, B, nb) || overlaps(B2, nb, U, nu))
    return GMHD_ERR_ALIAS;
  if (nsteps == 0)
    return GMHD_OK;
  const int np = ctx->n_problems;
  // work on a capturable stream, ordered after / before the caller's stream
  cudaStream_t caller = (cudaStream_t)stream;
  cudaStream_t s = caller ? caller : ctx->own_stream;
  cudaEvent_t  ev = nullptr;
  if (!caller)
  {
    GMHD_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    GMHD_CUDA(cudaEventRecord(ev, 0));
    GMHD_CUDA(cudaStreamWaitEvent(s, ev, 0));
  }
  int rc;
  if ((int64_t)nsteps * np > ctx->dtlog_cap)
  {
    if ((rc = dalloc(ctx, &ctx->d_dtlog, (size_t)nsteps * np)))
      return rc;
    ctx->dtlog_cap = (int64_t)nsteps * np;
    if (ctx->graph_exec)
    {
      cudaGraphExecDestroy(ctx->graph_exec);
      ctx->graph_exec = nullptr;
    }
  }
  if (ctx->p.time_integrator == GMHD_TIME_RK2_SSP)
  {
    if ((rc = dalloc(ctx, &ctx->d_Urk, (size_t)ctx->n_blocks * 5 * ctx->ncell)) ||
        (rc = dalloc(ctx, &ctx->d_Brk, (size_t)ctx->n_blocks * ctx->nface)))
      return rc;
  }
  std::vector<double> zeros(np, 0.0);
  GMHD_CUDA(cudaMemcpyAsync(ctx->d_t, t ? t : zeros.data(), sizeof(double) * np, cudaMemcpyHostToDevice, s));
  if (t_end)
    GMHD_CUDA(cudaMemcpyAsync(ctx->d_tend, t_end, sizeof(double) * np, cudaMemcpyHostToDevice, s));
  GMHD_CUDA(cudaMemsetAsync(ctx->d_counter, 0, sizeof(int32_t), s));
  // no step of this call has copied a finished problem through yet (NaN: not a dt of 0)
  GMHD_CUDA(cudaMemsetAsync(ctx->d_dt, 0xff, sizeof(double) * np, s));
  // CFL of the initial state into slot 0 (SolverGodunovMHD ctor: compute_dt, .cpp:180)
  if ((rc = enqueue_inv_dt(ctx, U, B, ctx->d_invdt, s, false)))
    return rc;
  const bool has_tend = t_end != nullptr;
  int        done = 0;
  if (use_graph && nsteps >= 2)
  {
    const void * key[5] = {U, U2, B, B2, (const void *)(intptr_t)(has_tend ? 1 : 0)};
    bool         same = ctx->graph_exec && ctx->graph_mesh_version == ctx->mesh_version;
    for (int i = 0; i < 5; ++i)
      same = same && key[i] == ctx->graph_key[i];
    if (!same)
    {
      if (ctx->graph_exec)
      {
        cudaGraphExecDestroy(ctx->graph_exec);
        ctx->graph_exec = nullptr;
      }
      cudaGraph_t g = nullptr;
      GMHD_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      int rc1 = enqueue_iteration(ctx, U, U2, B, B2, 0, s, has_tend);
      int rc2 = rc1 ? rc1 : enqueue_iteration(ctx, U2, U, B2, B, 1, s, has_tend);
      cudaError_t ec = cudaStreamEndCapture(s, &g);
      if (rc2)
      {
        if (g)
          cudaGraphDestroy(g);
        return rc2;
      }
      GMHD_CUDA(ec);
      cudaError_t ei = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
      cudaGraphDestroy(g);
      GMHD_CUDA(ei);
      for (int i = 0; i < 5; ++i)
        ctx->graph_key[i] = key[i];
      ctx->graph_mesh_version = ctx->mesh_version;
    }
    for (; done + 2 <= nsteps; done += 2)
      GMHD_CUDA(cudaGraphLaunch(ctx->graph_exec, s));
  }
  for (; done < nsteps; ++done)
  {
    const bool even = (done % 2) == 0;
    rc = even ? enqueue_iteration(ctx, U, U2, B, B2, 0, s, has_tend) : enqueue_iteration(ctx, U2, U, B2, B, 1, s, has_tend);
    if (rc)
      return rc;
  }
  if (nsteps % 2)
  {
    GMHD_CUDA(cudaMemcpyAsync(U, U2, nu, cudaMemcpyDeviceToDevice, s));
    GMHD_CUDA(cudaMemcpyAsync(B, B2, nb, cudaMemcpyDeviceToDevice, s));
  }
  if (t)
    GMHD_CUDA(cudaMemcpyAsync(t, ctx->d_t, sizeof(double) * np, cudaMemcpyDeviceToHost, s));
  if (dt_log)
    GMHD_CUDA(cudaMemcpyAsync(dt_log, ctx->d_dtlog, sizeof(double) * nsteps * np, cudaMemcpyDeviceToHost, s));
  unsigned int flags = 0;
  if ((rc = check_health(ctx, s, &flags)))
    return rc;
  if (ev)
  {
    cudaEventRecord(ev, s);
    cudaStreamWaitEvent(0, ev, 0);
    cudaEventDestroy(ev);
  }
  if (flags & (GMHD_HEALTH_BAD_DENSITY | GMHD_HEALTH_NONFINITE | GMHD_HEALTH_MISSING_NEIGHBOR | GMHD_HEALTH_LEVEL_JUMP))
    return GMHD_ERR_HEALTH;
  return GMHD_OK;
}

// gmhd_step_host in chunks (plan_host_chunks): copy-in on a_in, chunk steps on a compute stream as their
// inputs land, each chunk's copy-out on a_out right after its step, so that the copies in both
// directions overlap the steps. The compute stream is the caller's, or the context's own stream
// ordered after and before the legacy stream when the caller passes none.
static int
copy_runs(gmhd_ctx * ctx, int k, double * dst, const double * src, size_t per_block, cudaMemcpyKind kind,
          cudaStream_t st)
{
  const size_t bytes = per_block * sizeof(double);
  for (int g = ctx->hp_coff[k]; g < ctx->hp_coff[k + 1]; ++g)
  {
    const gmhd_ctx::HostRuns & h = ctx->hp_copy[g];
    const size_t               off = (size_t)h.start * per_block;
    if (h.count == 1)
      GMHD_CUDA(cudaMemcpyAsync(dst + off, src + off, (size_t)h.len * bytes, kind, st));
    else
    {
      const size_t pitch = (size_t)h.stride * bytes;
      GMHD_CUDA(cudaMemcpy2DAsync(dst + off, pitch, src + off, pitch, (size_t)h.len * bytes, (size_t)h.count, kind, st));
    }
  }
  return GMHD_OK;
}

// The tile-level schedule of the chunked host step for the context's tile choice: a tile reads the
// neighbour blocks in the slots its position in the block touches, so it can step once the highest chunk
// among its own and those blocks' chunks is in; tiles are grouped by that chunk (a slab's tiles away from its
// two neighbour slabs start as soon as the slab itself has arrived). Not used for the column step, whose
// columns span the whole block (block lists then, as planned per chunk).
static int
plan_host_tiles(gmhd_ctx * ctx)
{
  int T[3];
  const bool mixed = ctx->p.precision == GMHD_PRECISION_MIXED;
  const bool visc = ctx->p.viscosity_enabled != 0;
  if (mixed)
    gmhd::tile_shape_mixed(ctx->dim, ctx->bx, ctx->by, ctx->bz, visc, false, ctx->tile, T);
  else
    gmhd::tile_shape_fp64(ctx->dim, ctx->bx, ctx->by, ctx->bz, visc, ctx->tile, T);
  const int key = (T[0] << 16) | (T[1] << 8) | T[2];
  if (key == ctx->hp_tile_key)
    return GMHD_OK;
  const int K = ctx->hp_k, n = ctx->n_owned;
  ctx->hp_toff.assign(K + 1, 0);
  ctx->hp_done.assign(K, 0);
  const bool column = ctx->dim == 3 && T[2] == ctx->bz && T[0] == 16 && T[1] == 8 && mixed;
  if (column || ctx->bx % T[0] || ctx->by % T[1] || ctx->bz % T[2])
  {
    ctx->hp_tile_key = key;
    ctx->hp_toff.clear(); // block-level chunks
    return GMHD_OK;
  }
  const int nt[3] = {ctx->bx / T[0], ctx->by / T[1], ctx->dim == 3 ? ctx->bz / T[2] : 1};
  const int tpb = nt[0] * nt[1] * nt[2];
  // neighbour slots touched by a tile at each position class (first / last / both / neither per axis)
  auto     cls_of = [](int c, int nn) { return (c == 0 ? 1 : 0) | (c == nn - 1 ? 2 : 0); };
  uint32_t touch[64];
  for (int c = 0; c < 64; ++c)
  {
    const int cl[3] = {c & 3, (c >> 2) & 3, c >> 4};
    uint32_t  msk = 0;
    for (int sl = 0; sl < 27; ++sl)
    {
      const int o[3] = {sl % 3 - 1, (sl / 3) % 3 - 1, sl / 9 - 1};
      bool      t = true;
      for (int d = 0; d < 3; ++d)
        if (o[d] != 0 && !(cl[d] & (o[d] < 0 ? 1 : 2)))
          t = false;
      if (t)
        msk |= 1u << sl;
    }
    touch[c] = msk;
  }
  // tiles by (group, chunk of their block)
  std::vector<std::vector<int32_t>> groups((size_t)K * K);
  for (int k = 0; k < K; ++k)
    for (int i = ctx->hp_off[k]; i < ctx->hp_off[k + 1]; ++i)
    {
      const int b = ctx->hp_blocks[i];
      for (int t = 0; t < tpb; ++t)
      {
        const int      tc[3] = {t % nt[0], (t / nt[0]) % nt[1], t / (nt[0] * nt[1])};
        const uint32_t msk = touch[cls_of(tc[0], nt[0]) + 4 * (cls_of(tc[1], nt[1]) + 4 * cls_of(tc[2], nt[2]))];
        int            dep = k;
        for (int sl = 0; sl < 27; ++sl)
          if ((msk >> sl) & 1u)
            dep = std::max(dep, (int)ctx->hp_nchunk[(size_t)b * 27 + sl]);
        groups[(size_t)dep * K + k].push_back(b * tpb + t);
        ctx->hp_done[k] = std::max(ctx->hp_done[k], dep);
      }
    }
  // launches: per group, first the chunks this group completes (so that their copy-out starts early),
  // then the rest of the group's tiles
  std::vector<int32_t> all;
  all.reserve((size_t)n * tpb);
  ctx->hp_launch.clear();
  for (int k = 0; k < K; ++k)
  {
    ctx->hp_toff[k] = (int)all.size();
    for (int pass = 0; pass < 2; ++pass)
      for (int c = 0; c < K; ++c)
      {
        const std::vector<int32_t> & g = groups[(size_t)k * K + c];
        if (g.empty() || (ctx->hp_done[c] == k) != (pass == 0))
          continue;
        ctx->hp_launch.push_back(gmhd_ctx::HostLaunch{k, c, (int)all.size(), (int)g.size()});
        all.insert(all.end(), g.begin(), g.end());
      }
  }
  ctx->hp_toff[K] = (int)all.size();
  int rc;
  if ((rc = dalloc(ctx, &ctx->d_hp_tiles, all.size())))
    return rc;
  GMHD_CUDA(cudaMemcpy(ctx->d_hp_tiles, all.data(), all.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  ctx->hp_tile_key = key;
  return GMHD_OK;
}

static int
step_host_chunked(gmhd_ctx * ctx, const double * U, double * U2, const double * B, double * B2, double dt,
                  cudaStream_t caller)
{
  const int K = ctx->hp_k;
  if (!ctx->a_in)
  {
    GMHD_CUDA(cudaStreamCreateWithFlags(&ctx->a_in, cudaStreamNonBlocking));
    GMHD_CUDA(cudaStreamCreateWithFlags(&ctx->a_run, cudaStreamNonBlocking));
    GMHD_CUDA(cudaStreamCreateWithFlags(&ctx->a_out, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k)
    {
      GMHD_CUDA(cudaEventCreateWithFlags(&ctx->a_in_done[k], cudaEventDisableTiming));
      GMHD_CUDA(cudaEventCreateWithFlags(&ctx->a_run_done[k], cudaEventDisableTiming));
      GMHD_CUDA(cudaEventCreateWithFlags(&ctx->a_out_done[k], cudaEventDisableTiming));
    }
  }
  if (!ctx->hp_start)
  {
    GMHD_CUDA(cudaEventCreateWithFlags(&ctx->hp_start, cudaEventDisableTiming));
    GMHD_CUDA(cudaEventCreateWithFlags(&ctx->hp_end, cudaEventDisableTiming));
    for (int k = 0; k < gmhd_ctx::HP_MAX; ++k)
    {
      GMHD_CUDA(cudaEventCreateWithFlags(&ctx->hp_in[k], cudaEventDisableTiming));
      GMHD_CUDA(cudaEventCreateWithFlags(&ctx->hp_run[k], cudaEventDisableTiming));
    }
  }
  int rc;
  if ((rc = plan_host_tiles(ctx)))
    return rc;
  cudaStream_t s = caller ? caller : ctx->own_stream;
  const size_t cu = (size_t)5 * ctx->ncell, cb = (size_t)ctx->nface; // doubles per block
  // the copies and steps start after the work queued before this call on the caller's stream
  GMHD_CUDA(cudaEventRecord(ctx->hp_start, caller));
  GMHD_CUDA(cudaStreamWaitEvent(ctx->a_in, ctx->hp_start, 0));
  GMHD_CUDA(cudaStreamWaitEvent(ctx->a_out, ctx->hp_start, 0));
  if (s != caller)
    GMHD_CUDA(cudaStreamWaitEvent(s, ctx->hp_start, 0));
  for (int k = 0; k < K; ++k)
  {
    if ((rc = copy_runs(ctx, k, ctx->d_U, U, cu, cudaMemcpyHostToDevice, ctx->a_in)) ||
        (rc = copy_runs(ctx, k, ctx->d_B, B, cb, cudaMemcpyHostToDevice, ctx->a_in)))
      return rc;
    GMHD_CUDA(cudaEventRecord(ctx->hp_in[k], ctx->a_in));
  }
  auto copy_out = [&](int c) -> int {
    int r;
    if ((r = copy_runs(ctx, c, U2, ctx->d_U2, cu, cudaMemcpyDeviceToHost, ctx->a_out)) ||
        (r = copy_runs(ctx, c, B2, ctx->d_B2, cb, cudaMemcpyDeviceToHost, ctx->a_out)))
      return r;
    return GMHD_OK;
  };
  if (!ctx->hp_toff.empty())
  {
    // tile groups in chunk order; each chunk's copy-out right after the launch that completes it
    int waited = -1;
    for (const gmhd_ctx::HostLaunch & L : ctx->hp_launch)
    {
      if (L.k != waited)
      {
        GMHD_CUDA(cudaStreamWaitEvent(s, ctx->hp_in[L.k], 0));
        waited = L.k;
      }
      gmhd::StepArgs a = make_args(ctx, ctx->d_U, ctx->d_U2, ctx->d_B, ctx->d_B2);
      a.dt = dt;
      a.tile_list = ctx->d_hp_tiles + L.off;
      a.n_list = L.n;
      if ((rc = launch_step(ctx, a, s)))
        return rc;
      if (ctx->hp_done[L.c] == L.k)
      {
        GMHD_CUDA(cudaEventRecord(ctx->hp_run[L.c], s));
        GMHD_CUDA(cudaStreamWaitEvent(ctx->a_out, ctx->hp_run[L.c], 0));
        if ((rc = copy_out(L.c)))
          return rc;
      }
    }
  }
  else
    for (int i = 0; i < K; ++i)
    {
      // (column step) whole chunks in the order of their readiness
      const int      k = ctx->hp_order[i];
      gmhd::StepArgs a = make_args(ctx, ctx->d_U, ctx->d_U2, ctx->d_B, ctx->d_B2);
      a.dt = dt;
      GMHD_CUDA(cudaStreamWaitEvent(s, ctx->hp_in[ctx->hp_dep[k]], 0));
      a.blk_list = ctx->d_hp_blocks + ctx->hp_off[k];
      a.blk_count = ctx->hp_off[k + 1] - ctx->hp_off[k];
      if ((rc = launch_step(ctx, a, s)))
        return rc;
      GMHD_CUDA(cudaEventRecord(ctx->hp_run[k], s));
      GMHD_CUDA(cudaStreamWaitEvent(ctx->a_out, ctx->hp_run[k], 0));
      if ((rc = copy_out(k)))
        return rc;
    }
  GMHD_CUDA(cudaEventRecord(ctx->hp_end, ctx->a_out));
  GMHD_CUDA(cudaStreamWaitEvent(caller, ctx->hp_end, 0));
  GMHD_CUDA(cudaStreamSynchronize(caller));
  return GMHD_OK;
}

int
gmhd_step_host(gmhd_ctx * ctx, const double * U, double * U2, const double * B, double * B2, double dt, void * stream)
{
  if (!ctx || !U || !U2 || !B || !B2)
    return GMHD_ERR_ARGUMENT;
  if (!ctx->has_mesh)
    return GMHD_ERR_MESH;
  if (ctx->n_blocks == 0)
    return GMHD_OK; // nothing to copy or step
  const size_t nu = (size_t)ctx->n_blocks * 5 * ctx->ncell;
  const size_t nb = (size_t)ctx->n_blocks * ctx->nface;
  int          rc;
  {
    if ((rc = dalloc(ctx, &ctx->d_U, nu)) || (rc = dalloc(ctx, &ctx->d_U2, nu)) || (rc = dalloc(ctx, &ctx->d_B, nb)) ||
        (rc = dalloc(ctx, &ctx->d_B2, nb)))
      return rc;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (ctx->hp_k > 1)
  {
    if (!(dt >= 0.0))
      return GMHD_ERR_ARGUMENT;
    return step_host_chunked(ctx, U, U2, B, B2, dt, s);
  }
  GMHD_CUDA(cudaMemcpyAsync(ctx->d_U, U, nu * sizeof(double), cudaMemcpyHostToDevice, s));
  GMHD_CUDA(cudaMemcpyAsync(ctx->d_B, B, nb * sizeof(double), cudaMemcpyHostToDevice, s));
  if ((rc = gmhd_step(ctx, ctx->d_U, ctx->d_U2, ctx->d_B, ctx->d_B2, dt, stream)))
    return rc;
  const size_t nu_own = (size_t)ctx->n_owned * 5 * ctx->ncell;
  const size_t nb_own = (size_t)ctx->n_owned * ctx->nface;
  GMHD_CUDA(cudaMemcpyAsync(U2, ctx->d_U2, nu_own * sizeof(double), cudaMemcpyDeviceToHost, s));
  GMHD_CUDA(cudaMemcpyAsync(B2, ctx->d_B2, nb_own * sizeof(double), cudaMemcpyDeviceToHost, s));
  GMHD_CUDA(cudaStreamSynchronize(s));
  return GMHD_OK;
}

int
gmhd_step_host_async(gmhd_ctx * ctx, const double * U, double * U2, const double * B, double * B2, double dt,
                     void * stream)
{
  if (!ctx || !U || !U2 || !B || !B2)
    return GMHD_ERR_ARGUMENT;
  if (!ctx->has_mesh)
    return GMHD_ERR_MESH;
  if (!(dt >= 0.0))
    return GMHD_ERR_ARGUMENT;
  if (ctx->n_blocks == 0)
    return GMHD_OK; // nothing to copy or step
  const size_t nu = (size_t)ctx->n_blocks * 5 * ctx->ncell;
  const size_t nb = (size_t)ctx->n_blocks * ctx->nface;
  int          rc;
  if (!ctx->a_in)
  {
    GMHD_CUDA(cudaStreamCreateWithFlags(&ctx->a_in, cudaStreamNonBlocking));
    GMHD_CUDA(cudaStreamCreateWithFlags(&ctx->a_run, cudaStreamNonBlocking));
    GMHD_CUDA(cudaStreamCreateWithFlags(&ctx->a_out, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k)
    {
      GMHD_CUDA(cudaEventCreateWithFlags(&ctx->a_in_done[k], cudaEventDisableTiming));
      GMHD_CUDA(cudaEventCreateWithFlags(&ctx->a_run_done[k], cudaEventDisableTiming));
      GMHD_CUDA(cudaEventCreateWithFlags(&ctx->a_out_done[k], cudaEventDisableTiming));
    }
  }
  const int k = ctx->a_next;
  {
    if ((rc = dalloc(ctx, &ctx->a_U[k], nu)) || (rc = dalloc(ctx, &ctx->a_U2[k], nu)) ||
        (rc = dalloc(ctx, &ctx->a_B[k], nb)) || (rc = dalloc(ctx, &ctx->a_B2[k], nb)))
      return rc;
  }
  cudaStream_t caller = (cudaStream_t)stream;
  // copy in (U, B are complete in host memory when the call is made) once the step that last read this
  // input set is done; the input and output sets are released separately, so that the copy-in of one
  // call runs beside the copy-out of the call before it
  GMHD_CUDA(cudaStreamWaitEvent(ctx->a_in, ctx->a_run_done[k], 0));
  GMHD_CUDA(cudaMemcpyAsync(ctx->a_U[k], U, nu * sizeof(double), cudaMemcpyHostToDevice, ctx->a_in));
  GMHD_CUDA(cudaMemcpyAsync(ctx->a_B[k], B, nb * sizeof(double), cudaMemcpyHostToDevice, ctx->a_in));
  GMHD_CUDA(cudaEventRecord(ctx->a_in_done[k], ctx->a_in));
  // the step, once its inputs are in and the output set's last copy-out is done
  GMHD_CUDA(cudaStreamWaitEvent(ctx->a_run, ctx->a_in_done[k], 0));
  GMHD_CUDA(cudaStreamWaitEvent(ctx->a_run, ctx->a_out_done[k], 0));
  gmhd::StepArgs a = make_args(ctx, ctx->a_U[k], ctx->a_U2[k], ctx->a_B[k], ctx->a_B2[k]);
  a.dt = dt;
  if ((rc = launch_step(ctx, a, ctx->a_run)))
    return rc;
  GMHD_CUDA(cudaEventRecord(ctx->a_run_done[k], ctx->a_run));
  // copy out the owned blocks, then order the caller's stream after it
  GMHD_CUDA(cudaStreamWaitEvent(ctx->a_out, ctx->a_run_done[k], 0));
  GMHD_CUDA(cudaMemcpyAsync(U2, ctx->a_U2[k], (size_t)ctx->n_owned * 5 * ctx->ncell * sizeof(double),
                            cudaMemcpyDeviceToHost, ctx->a_out));
  GMHD_CUDA(cudaMemcpyAsync(B2, ctx->a_B2[k], (size_t)ctx->n_owned * ctx->nface * sizeof(double),
                            cudaMemcpyDeviceToHost, ctx->a_out));
  GMHD_CUDA(cudaEventRecord(ctx->a_out_done[k], ctx->a_out));
  GMHD_CUDA(cudaStreamWaitEvent(caller, ctx->a_out_done[k], 0));
  ctx->a_next = 1 - k;
  return GMHD_OK;
}

int
gmhd_refine_flags(gmhd_ctx * ctx, const double * U, const double * B, const gmhd_refine_params * params,
                  int8_t * flags, void * stream)
{
  if (!ctx || !U || !B || !params || !flags)
    return GMHD_ERR_ARGUMENT;
  if (!ctx->has_mesh)
    return GMHD_ERR_MESH;
  if ((params->criterion != GMHD_REFINE_SIMPLE_GRADIENT && params->criterion != GMHD_REFINE_LOHNER_UNSPLIT) ||
      (!params->use_rho && !params->use_pressure))
    return GMHD_ERR_ARGUMENT;
  const int     nvar = (params->use_rho ? 1 : 0) + (params->use_pressure ? 1 : 0);
  const size_t  nq = (size_t)nvar * ctx->n_owned * ctx->ncell;
  cudaStream_t  s = (cudaStream_t)stream;
  // scratch kept in the context (an AMR cycle every few steps allocates nothing)
  int rc;
  if ((rc = dalloc(ctx, &ctx->d_rf_q, nq > 0 ? nq : 1)) ||
      (rc = dalloc(ctx, &ctx->d_rf_flags, (size_t)(ctx->n_owned > 0 ? ctx->n_owned : 1))))
    return rc;
  rc = gmhd::launch_refine_flags(U, B, ctx->d_level, ctx->n_owned, ctx->dim, ctx->bx, ctx->by, ctx->bz, ctx->ncell,
                                 ctx->nfx, ctx->nfy, ctx->nface, ctx->p.gamma0, ctx->p.smallr, ctx->smallp,
                                 params->criterion, params->level_min, params->level_max, params->use_rho,
                                 params->use_pressure, params->eps_refine, params->eps_coarsen, params->eps_lohner,
                                 ctx->d_rf_q, ctx->d_rf_flags, s);
  if (rc == 0 && ctx->n_owned > 0)
    rc = (int)cudaMemcpyAsync(flags, ctx->d_rf_flags, (size_t)ctx->n_owned, cudaMemcpyDeviceToHost, s);
  if (rc == 0)
    rc = (int)cudaStreamSynchronize(s);
  return rc ? cuda_fail(ctx, (cudaError_t)rc) : GMHD_OK;
}

int
gmhd_remap(int32_t dim, int32_t bx, int32_t by, int32_t bz, int32_t n_old_blocks, int32_t n_new_owned,
           const int32_t * remap, const double * U_old, const double * B_old, double * U_new, double * B_new,
           void * stream)
{
  if ((dim != 2 && dim != 3) || bx < 4 || by < 4 || (dim == 3 && bz < 4) || (dim == 2 && bz != 1) || bx % 2 ||
      by % 2 || (dim == 3 && bz % 2) || n_new_owned < 0 || !remap || !U_old || !B_old || !U_new || !B_new)
    return GMHD_ERR_ARGUMENT;
  for (int64_t n = 0; n < n_new_owned; ++n)
  {
    const int32_t * rm = remap + n * 15;
    if (rm[0] < 0 || rm[0] > 2 || rm[1] < 0 || rm[1] >= n_old_blocks ||
        (rm[0] == 1 && (rm[2] < 0 || rm[2] >= (1 << dim))))
      return GMHD_ERR_ARGUMENT;
    if (rm[0] == 2)
      for (int c = 0; c < (1 << dim); ++c)
        if (rm[1 + c] < 0 || rm[1 + c] >= n_old_blocks)
          return GMHD_ERR_ARGUMENT;
    for (int f = 0; f < 6; ++f)
      if (rm[9 + f] < -1 || rm[9 + f] >= n_old_blocks || (f >= 2 * dim && rm[9 + f] != -1))
        return GMHD_ERR_ARGUMENT;
  }
  gmhd::GhostArgs g;
  std::memset(&g, 0, sizeof g);
  g.U = U_old;
  g.B = B_old;
  g.dim = dim;
  g.bx = bx;
  g.by = by;
  g.bz = dim == 3 ? bz : 1;
  g.ncell = (int64_t)bx * by * g.bz;
  g.nfx = (int64_t)(bx + 1) * by * g.bz;
  g.nfy = (int64_t)bx * (by + 1) * g.bz;
  g.nface = g.nfx + g.nfy + (dim == 3 ? (int64_t)bx * by * (g.bz + 1) : g.ncell);
  cudaStream_t s = (cudaStream_t)stream;
  int32_t *    dmap = nullptr;
  unsigned *   dh = nullptr;
  if (cudaMalloc((void **)&dmap, sizeof(int32_t) * 15 * (size_t)(n_new_owned > 0 ? n_new_owned : 1)) != cudaSuccess)
    return GMHD_ERR_CUDA;
  if (cudaMalloc((void **)&dh, sizeof(unsigned)) != cudaSuccess)
  {
    cudaFree(dmap);
    return GMHD_ERR_CUDA;
  }
  g.health = dh;
  int      rc = (int)cudaMemsetAsync(dh, 0, sizeof(unsigned), s);
  unsigned h = 0;
  if (rc == 0)
    rc = (int)cudaMemcpyAsync(dmap, remap, sizeof(int32_t) * 15 * (size_t)n_new_owned, cudaMemcpyHostToDevice, s);
  if (rc == 0)
    rc = gmhd::launch_remap(g, dmap, n_new_owned, U_new, B_new, s);
  if (rc == 0)
    rc = (int)cudaMemcpyAsync(&h, dh, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (rc == 0)
    rc = (int)cudaStreamSynchronize(s);
  cudaFree(dmap);
  cudaFree(dh);
  if (rc)
    return GMHD_ERR_CUDA;
  return h ? GMHD_ERR_MESH : GMHD_OK;
}

int
gmhd_last_status(gmhd_ctx * ctx, uint32_t * flags)
{
  if (!ctx || !flags)
    return GMHD_ERR_ARGUMENT;
  unsigned int h = 0;
  const int    rc = check_health(ctx, ctx->own_stream, &h);
  *flags = h;
  return rc;
}

int
gmhd_last_cuda_error(const gmhd_ctx * ctx)
{
  return ctx ? ctx->last_cuda : 0;
}

const char *
gmhd_error_string(int status)
{
  switch (status)
  {
    case GMHD_OK: return "ok";
    case GMHD_ERR_ARGUMENT: return "invalid argument";
    case GMHD_ERR_MESH: return "mesh not set or not supported";
    case GMHD_ERR_CUDA: return "CUDA error";
    case GMHD_ERR_ALIAS: return "output aliases an input";
    case GMHD_ERR_HEALTH: return "non-physical state produced";
    case GMHD_ERR_TOO_LARGE: return "request exceeds a fixed capacity";
    default: return "unknown status";
  }
}

int
gmhd_layout_check(const gmhd_mesh * m, int64_t u_var_stride, int64_t u_block_stride, int64_t b_block_stride)
{
  if (!m)
    return GMHD_ERR_ARGUMENT;
  const int64_t bz = m->dim == 3 ? m->bz : 1;
  const int64_t ncell = (int64_t)m->bx * m->by * bz;
  const int64_t nfz = m->dim == 3 ? (int64_t)m->bx * m->by * (bz + 1) : ncell;
  const int64_t nface = (int64_t)(m->bx + 1) * m->by * bz + (int64_t)m->bx * (m->by + 1) * bz + nfz;
  if (u_var_stride != ncell || u_block_stride != 5 * ncell || b_block_stride != nface)
    return GMHD_ERR_ARGUMENT;
  return GMHD_OK;
}

} // extern "C"
