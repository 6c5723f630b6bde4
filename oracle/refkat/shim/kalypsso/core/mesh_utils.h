// Stub of kalypsso-core's mesh enums used by the bridged functors: the domain faces (XMIN = 0, XMAX,
// YMIN, YMAX, ZMIN, ZMAX) and directions.
#pragma once
#include <kalypsso/core/kokkos_shared.h>

namespace kalypsso
{
enum FaceId : int
{
  XMIN = 0,
  XMAX = 1,
  YMIN = 2,
  YMAX = 3,
  ZMIN = 4,
  ZMAX = 5
};
namespace Face
{
using face_t = int;
template <std::size_t dim>
Kokkos::Array<face_t, 2 * dim>
get_all_faces()
{
  Kokkos::Array<face_t, 2 * dim> f;
  for (std::size_t i = 0; i < 2 * dim; ++i)
    f[i] = (face_t)i;
  return f;
}
inline bool
is_left_face(face_t f)
{
  return f % 2 == 0;
}
} // namespace Face
namespace Dir
{
using dir_t = int;
} // namespace Dir
} // namespace kalypsso
