// Stub of kalypsso-core's per-octant face status for the functor bridge: one bit per face (xmin,
// xmax, ymin, ymax, zmin, zmax), set where the neighbour across that face is finer. The bridge runs
// conforming blocks (all bits clear).
#pragma once
#include <cstdint>
#include <memory>
#include <vector>

namespace kalypsso
{
enum class conformal_neighbor_status : int
{
  NEIGHBOR_IS_NOT_FINER = 0,
  NEIGHBOR_IS_FINER = 1
};
template <std::size_t dim, typename device_t>
struct conformal_status_view_t
{
  std::shared_ptr<std::vector<uint8_t>> bits = std::make_shared<std::vector<uint8_t>>();
  uint8_t operator()(int i) const { return (*bits)[i]; }
};
template <std::size_t dim>
struct conformal_face_status_t
{
  static conformal_neighbor_status face(uint8_t s, int f)
  {
    return (s >> f) & 1 ? conformal_neighbor_status::NEIGHBOR_IS_FINER : conformal_neighbor_status::NEIGHBOR_IS_NOT_FINER;
  }
  static conformal_neighbor_status face_xmin(uint8_t s) { return face(s, 0); }
  static conformal_neighbor_status face_xmax(uint8_t s) { return face(s, 1); }
  static conformal_neighbor_status face_ymin(uint8_t s) { return face(s, 2); }
  static conformal_neighbor_status face_ymax(uint8_t s) { return face(s, 3); }
  static conformal_neighbor_status face_zmin(uint8_t s) { return face(s, 4); }
  static conformal_neighbor_status face_zmax(uint8_t s) { return face(s, 5); }
};
} // namespace kalypsso
