// Stub of kalypsso-core's orchard keys for the functor bridge. A key packs a leaf's level (bits 0-5),
// its outside-status bits along x, y, z (bits 6-8: the leaf lies beyond the domain along that axis)
// and its coordinates at its level (18 bits each from bit 9, offset by 2^17 so that the outside layer,
// at -1 or n, fits). A bare level is a valid key for the functors that only read levels.
#pragma once
#include <cstdint>
#include <memory>
#include <vector>

#include <kalypsso/core/kokkos_shared.h>

namespace kalypsso
{
template <typename device_t>
struct orchard_key_base_t
{
  struct view_t
  {
    std::shared_ptr<std::vector<uint64_t>> keys = std::make_shared<std::vector<uint64_t>>();
    uint64_t    operator()(int i) const { return (*keys)[i]; }
    std::size_t extent(int) const { return keys->size(); }
  };
};
template <std::size_t dim>
struct orchard_key_t
{
  static constexpr int64_t OFF = int64_t(1) << 17;

  static uint64_t
  pack(int level, const int64_t * c, unsigned outside_bits)
  {
    uint64_t k = (uint64_t)(level & 63) | ((uint64_t)(outside_bits & 7u) << 6);
    for (int a = 0; a < 3; ++a)
      k |= (uint64_t)((a < (int)dim ? c[a] : 0) + OFF) << (9 + 18 * a);
    return k;
  }
  static int      level(uint64_t key) { return (int)(key & 63); }
  static unsigned outside_bits(uint64_t key) { return (unsigned)((key >> 6) & 7); }
  static int64_t  coord(uint64_t key, int a) { return (int64_t)((key >> (9 + 18 * a)) & ((1u << 18) - 1)) - OFF; }
  // leaves along axis a at the key's level
  template <class BS>
  static int64_t extent(uint64_t key, BS const & bricks, int a)
  {
    return (int64_t)bricks[a] << level(key);
  }

  // the direction pointing from a leaf beyond the domain back into it (+1 below, -1 above, 0 inside)
  template <class BS, class P>
  static Kokkos::Array<int, dim> get_outside_normal(uint64_t key, BS const & bricks, P const &)
  {
    Kokkos::Array<int, dim> n;
    for (int a = 0; a < (int)dim; ++a)
    {
      const int64_t c = coord(key, a);
      n[a] = c < 0 ? 1 : (c >= extent(key, bricks, a) ? -1 : 0);
    }
    return n;
  }
  static int is_touching_face_X(uint64_t key) { return (outside_bits(key) >> 0) & 1; }
  static int is_touching_face_Y(uint64_t key) { return (outside_bits(key) >> 1) & 1; }
  static int is_touching_face_Z(uint64_t key) { return (outside_bits(key) >> 2) & 1; }
  static bool is_outside_dir(uint64_t key, int d) { return (outside_bits(key) >> d) & 1; }

  // the same-level leaf across offset o (the coordinates move; the outside bits are kept)
  template <class O, class BS, class P>
  static uint64_t get_neighbor_key_same_level(uint64_t key, O const & o, BS const &, P const &)
  {
    int64_t c[3] = {0, 0, 0};
    for (int a = 0; a < (int)dim; ++a)
      c[a] = coord(key, a) + o[a];
    return pack(level(key), c, outside_bits(key));
  }
  static void reset_outside_bits(uint64_t & key) { key &= ~(uint64_t(7) << 6); }

  // the leaf touches the domain border face f (0 xmin, 1 xmax, 2 ymin, ...)
  template <class BS>
  static bool is_at_domain_border(uint64_t key, int f, BS const & bricks)
  {
    const int     a = f / 2;
    const int64_t c = coord(key, a);
    return (f % 2 == 0) ? c == 0 : c == extent(key, bricks, a) - 1;
  }
};
} // namespace kalypsso
