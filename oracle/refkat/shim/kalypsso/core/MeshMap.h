// Stub of kalypsso-core's key-to-leaf lookup: the block whose key (level and coordinates, outside
// bits ignored) equals `key`, searched in the bridge's key table.
#pragma once
#include <cstdint>
#include <utility>

#include <kalypsso/core/amr_hashmap.h>

namespace kalypsso
{
template <class Map>
std::pair<bool, int32_t>
key_to_value(uint64_t key, Map const & map)
{
  const uint64_t mask = ~(uint64_t(7) << 6);
  for (int b = 0; b < map.mesh->n_blocks; ++b)
    if ((map.mesh->keys[b] & mask) == (key & mask))
      return {true, b};
  return {false, -1};
}
} // namespace kalypsso
