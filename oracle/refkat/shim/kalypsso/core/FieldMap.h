// Stub of kalypsso-core's FieldMap (only what models/MHD.h needs to compile).
#pragma once
#include <map>
#include <string>
namespace kalypsso
{
using id2names_t = std::map<int, std::string>;
using names2id_t = std::map<std::string, int>;
template <typename Model>
struct FieldMap
{
  bool on[32] = {};
  void enable(int id) { on[id] = true; }
  bool enabled(int id) const { return on[id]; }
  int  operator[](int id) const { return id; }
};
} // namespace kalypsso
