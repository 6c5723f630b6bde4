// A C++ caller of the C ABI (include/gmhd.h) without Python or torch: what a GodunovImplemBase adapter in
// the reference's solver does. Builds a periodic 3D mesh with the library's forest, sets a 3D
// Orszag-Tang state (face B as the discrete curl of A_z, so div B = 0 exactly), runs the solver loop
// (gmhd_advance) on the FP64 and the mixed path, and checks mass conservation, div B, health flags and
// the mixed path against FP64. Exit status 0 on success.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

#include <cuda_runtime.h>

#include "gmhd.h"

namespace
{
constexpr double kPi = 3.14159265358979323846;

#define CHECK(cond, msg)                                                                           \
  do                                                                                               \
  {                                                                                                \
    if (!(cond))                                                                                   \
    {                                                                                              \
      std::fprintf(stderr, "FAIL: %s (%s:%d)\n", msg, __FILE__, __LINE__);                         \
      return 1;                                                                                    \
    }                                                                                              \
  } while (0)

struct Mesh
{
  int                  n_owned = 0, n_blocks = 0;
  std::vector<int32_t> level, coord, neighbor;
};

int
build_mesh(int level, int b, Mesh & m)
{
  // every leaf at `level` over one periodic root brick
  const int            side = 1 << level;
  std::vector<int32_t> keys;
  for (int z = 0; z < side; ++z)
    for (int y = 0; y < side; ++y)
      for (int x = 0; x < side; ++x)
      {
        keys.push_back(level);
        keys.push_back(x);
        keys.push_back(y);
        keys.push_back(z);
      }
  const int32_t  bricks[3] = {1, 1, 1}, periodic[3] = {1, 1, 1};
  gmhd_forest *  f = gmhd_forest_build(3, bricks, periodic, b, b, b, level, level, side * side * side, keys.data(), nullptr);
  CHECK(f, "gmhd_forest_build");
  int32_t no = 0, nb = 0, has_fine = 0;
  CHECK(gmhd_forest_sizes(f, &no, &nb, &has_fine) == GMHD_OK && !has_fine, "gmhd_forest_sizes");
  m.n_owned = no;
  m.n_blocks = nb;
  m.level.resize(nb);
  m.coord.resize(3 * (size_t)nb);
  m.neighbor.resize(27 * (size_t)nb);
  CHECK(gmhd_forest_tables(f, m.level.data(), m.coord.data(), m.neighbor.data(), nullptr, nullptr, nullptr, nullptr) ==
          GMHD_OK,
        "gmhd_forest_tables");
  gmhd_forest_destroy(f);
  return 0;
}

struct State
{
  std::vector<double> U, B;
};

// 3D Orszag-Tang (uniform in z), gamma 5/3, on blocks of b^3 cells; face B from A_z at cell corners
State
orszag_tang(const Mesh & m, int b)
{
  const int64_t ncell = (int64_t)b * b * b, nfx = (int64_t)(b + 1) * b * b, nface = 3 * nfx;
  State         s;
  s.U.assign((size_t)m.n_blocks * 5 * ncell, 0.0);
  s.B.assign((size_t)m.n_blocks * nface, 0.0);
  const double gamma = 5.0 / 3.0, B0 = 1.0 / std::sqrt(4.0 * kPi);
  const double rho = 25.0 / (36.0 * kPi), p = 5.0 / (12.0 * kPi);
  for (int blk = 0; blk < m.n_blocks; ++blk)
  {
    const double dx = 1.0 / (double)(b << m.level[blk]);
    const int    n = b << m.level[blk]; // cells per side
    const int    cx = m.coord[3 * blk] * b, cy = m.coord[3 * blk + 1] * b;
    // corners wrapped into [0, n): the two copies of a periodic border face get the same bits
    auto Az = [&](int i, int j) {
      const double x = ((cx + i) % n) * dx, y = ((cy + j) % n) * dx;
      return B0 * (std::cos(4.0 * kPi * x) / (4.0 * kPi) + std::cos(2.0 * kPi * y) / (2.0 * kPi));
    };
    double * Bx = &s.B[(size_t)blk * nface];
    double * By = Bx + nfx;
    double * U = &s.U[(size_t)blk * 5 * ncell];
    for (int k = 0; k < b; ++k)
      for (int j = 0; j < b; ++j)
        for (int i = 0; i <= b; ++i)
          Bx[i + (b + 1) * (j + (int64_t)b * k)] = (Az(i, j + 1) - Az(i, j)) / dx;
    for (int k = 0; k < b; ++k)
      for (int j = 0; j <= b; ++j)
        for (int i = 0; i < b; ++i)
          By[i + b * (j + (int64_t)(b + 1) * k)] = -(Az(i + 1, j) - Az(i, j)) / dx;
    for (int k = 0; k < b; ++k)
      for (int j = 0; j < b; ++j)
        for (int i = 0; i < b; ++i)
        {
          const int64_t c = i + b * (j + (int64_t)b * k);
          const double  x = (cx + i + 0.5) * dx, y = (cy + j + 0.5) * dx;
          const double  u = -std::sin(2.0 * kPi * y), v = std::sin(2.0 * kPi * x);
          const double  bxc = 0.5 * (Bx[i + (b + 1) * (j + (int64_t)b * k)] + Bx[i + 1 + (b + 1) * (j + (int64_t)b * k)]);
          const double  byc = 0.5 * (By[i + b * (j + (int64_t)(b + 1) * k)] + By[i + b * (j + 1 + (int64_t)(b + 1) * k)]);
          U[c] = rho;
          U[ncell + c] = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v) + 0.5 * (bxc * bxc + byc * byc);
          U[2 * ncell + c] = rho * u;
          U[3 * ncell + c] = rho * v;
          U[4 * ncell + c] = 0.0;
        }
  }
  return s;
}

// nsteps of the solver loop on one path; the final state comes back in s
int
run(const Mesh & m, int b, int precision, int nsteps, State & s)
{
  gmhd_params prm{};
  prm.gamma0 = 5.0 / 3.0;
  prm.cfl = 0.5;
  prm.slope_type = 2.0;
  prm.smallr = 1e-10;
  prm.smallc = 1e-10;
  prm.scaling_factor = 1.0;
  prm.riemann = GMHD_RIEMANN_HLLD;
  prm.precision = precision;
  prm.prolongation = GMHD_PROLONG_SIMPLE_COPY;
  prm.time_integrator = GMHD_TIME_HANCOCK;
  gmhd_ctx * ctx = gmhd_create(&prm);
  CHECK(ctx, "gmhd_create");
  gmhd_mesh gm{};
  gm.dim = 3;
  gm.bx = gm.by = gm.bz = b;
  gm.n_blocks = m.n_blocks;
  gm.n_owned = m.n_owned;
  gm.level = m.level.data();
  gm.neighbor = m.neighbor.data();
  gm.n_problems = 1;
  for (int f = 0; f < 6; ++f)
    gm.bc[f] = GMHD_BC_PERIODIC;
  gm.coord = m.coord.data();
  CHECK(gmhd_set_mesh(ctx, &gm) == GMHD_OK, "gmhd_set_mesh");
  double *U = nullptr, *U2 = nullptr, *B = nullptr, *B2 = nullptr;
  const size_t nu = s.U.size() * sizeof(double), nb = s.B.size() * sizeof(double);
  CHECK(cudaMalloc(&U, nu) == cudaSuccess && cudaMalloc(&U2, nu) == cudaSuccess && cudaMalloc(&B, nb) == cudaSuccess &&
          cudaMalloc(&B2, nb) == cudaSuccess,
        "cudaMalloc");
  CHECK(cudaMemcpy(U, s.U.data(), nu, cudaMemcpyHostToDevice) == cudaSuccess &&
          cudaMemcpy(B, s.B.data(), nb, cudaMemcpyHostToDevice) == cudaSuccess,
        "copy in");
  double t = 0.0;
  std::vector<double> dts(nsteps);
  CHECK(gmhd_advance(ctx, U, U2, B, B2, nsteps, &t, nullptr, dts.data(), 1, nullptr) == GMHD_OK, "gmhd_advance");
  uint32_t health = 0;
  CHECK(gmhd_last_status(ctx, &health) == GMHD_OK && (health & ~GMHD_HEALTH_LOW_BETA_FP64) == 0, "health flags");
  CHECK(cudaMemcpy(s.U.data(), U, nu, cudaMemcpyDeviceToHost) == cudaSuccess &&
          cudaMemcpy(s.B.data(), B, nb, cudaMemcpyDeviceToHost) == cudaSuccess,
        "copy out");
  CHECK(t > 0.0 && dts[0] > 0.0, "time advanced");
  cudaFree(U);
  cudaFree(U2);
  cudaFree(B);
  cudaFree(B2);
  gmhd_destroy(ctx);
  return 0;
}

double
max_div_b(const Mesh & m, int b, const State & s)
{
  const int64_t nfx = (int64_t)(b + 1) * b * b, nface = 3 * nfx;
  double        mx = 0.0;
  for (int blk = 0; blk < m.n_owned; ++blk)
  {
    const double   dx = 1.0 / (double)(b << m.level[blk]);
    const double * Bx = &s.B[(size_t)blk * nface];
    const double * By = Bx + nfx;
    const double * Bz = By + nfx;
    for (int k = 0; k < b; ++k)
      for (int j = 0; j < b; ++j)
        for (int i = 0; i < b; ++i)
        {
          const double d = (Bx[i + 1 + (b + 1) * (j + (int64_t)b * k)] - Bx[i + (b + 1) * (j + (int64_t)b * k)]) +
                           (By[i + b * (j + 1 + (int64_t)(b + 1) * k)] - By[i + b * (j + (int64_t)(b + 1) * k)]) +
                           (Bz[i + b * (j + (int64_t)b * (k + 1))] - Bz[i + b * (j + (int64_t)b * k)]);
          mx = std::fmax(mx, std::fabs(d) / dx);
        }
  }
  return mx;
}

double
total(const Mesh & m, int b, const State & s, int var)
{
  // compensated (Kahan) sum, so that the check sees the update's round-off, not the summation's
  const int64_t ncell = (int64_t)b * b * b;
  double        sum = 0.0, comp = 0.0;
  for (int blk = 0; blk < m.n_owned; ++blk)
    for (int64_t c = 0; c < ncell; ++c)
    {
      const double y = s.U[((size_t)blk * 5 + var) * ncell + c] - comp;
      const double t = sum + y;
      comp = (t - sum) - y;
      sum = t;
    }
  return sum;
}
} // namespace

int
main()
{
  const int level = 2, b = 16, nsteps = 20; // 64^3 cells in 64 blocks of 16^3
  Mesh      m;
  if (build_mesh(level, b, m))
    return 1;
  CHECK(m.n_owned == 64 && m.n_blocks == 64, "mesh size");
  const State s0 = orszag_tang(m, b);
  State       s64 = s0, smx = s0;
  if (run(m, b, GMHD_PRECISION_FP64, nsteps, s64) || run(m, b, GMHD_PRECISION_MIXED, nsteps, smx))
    return 1;
  const double mass0 = total(m, b, s0, 0);
  const double dm64 = std::fabs(total(m, b, s64, 0) - mass0) / mass0, dmmx = std::fabs(total(m, b, smx, 0) - mass0) / mass0;
  const double div0 = max_div_b(m, b, s0), div64 = max_div_b(m, b, s64), divmx = max_div_b(m, b, smx);
  double l1 = 0.0, nrm = 0.0;
  const int64_t ncell = (int64_t)b * b * b;
  for (int blk = 0; blk < m.n_owned; ++blk)
    for (int64_t c = 0; c < ncell; ++c)
    {
      l1 += std::fabs(smx.U[(size_t)blk * 5 * ncell + c] - s64.U[(size_t)blk * 5 * ncell + c]);
      nrm += std::fabs(s64.U[(size_t)blk * 5 * ncell + c]);
    }
  std::printf("abi_demo: %d steps on 64^3; mass drift fp64 %.2e mixed %.2e; max div B initial %.2e fp64 %.2e "
              "mixed %.2e; L1(rho) mixed vs fp64 %.2e\n",
              nsteps, dm64, dmmx, div0, div64, divmx, l1 / nrm);
  CHECK(dm64 < 1e-11 && dmmx < 1e-11, "mass conserved to round-off");
  CHECK(div64 < 1e-10 && divmx < 1e-10, "div B at round-off");
  CHECK(l1 / nrm < 1e-6, "mixed within 1e-6 of FP64");
  return 0;
}
