// Stub of kalypsso-core's AMR hashmap for the functor bridge. The reference's StencilHelper finds
// neighbour leaves through a hashmap of orchard keys; here the "map" carries the bridge's mesh tables
// instead (the C ABI's neighbour tables), which the StencilHelper stub reads.
#pragma once
#include <cstdint>

namespace kalypsso
{
using iOct_t = int32_t;
// Mesh tables of the bridge: per block its level, the 27-slot neighbour table ((oz+1)*9 + (oy+1)*3 +
// (ox+1); a same-level or coarser leaf, an outside block, or -1), the children of neighbour regions
// split into finer leaves ([27][8] per block, x fastest; null on conforming meshes) and the block's
// coordinates at its level. Blocks [0, n_owned) are owned, the rest outside blocks.
struct BridgeMesh
{
  int             dim = 0, n_owned = 0, n_blocks = 0;
  const int32_t * level = nullptr;
  const int32_t * neighbor = nullptr;
  const int32_t * fine = nullptr;
  const int32_t * coord = nullptr;
  const uint64_t * keys = nullptr; // [n_blocks] orchard keys (outside leaves: coordinates beyond the domain)
};
template <typename device_t>
struct hashmap_base_t
{
  struct map_t
  {
    const BridgeMesh * mesh = nullptr;
  };
};
} // namespace kalypsso
