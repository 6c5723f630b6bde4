// Stub of kalypsso-core's orchard keys for the functor bridge: a key is just the leaf's level here.
#pragma once
#include <cstdint>
#include <memory>
#include <vector>

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
  static int level(uint64_t key) { return (int)key; }
};
} // namespace kalypsso
