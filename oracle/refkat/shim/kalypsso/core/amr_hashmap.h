// Stub: the functor bridge runs conforming single blocks; nothing of the AMR hashmap is used beyond
// its type names.
#pragma once
#include <cstdint>

namespace kalypsso
{
using iOct_t = int32_t;
template <typename device_t>
struct hashmap_base_t
{
  struct map_t
  {
  };
};
} // namespace kalypsso
