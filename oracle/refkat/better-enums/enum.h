// Minimal stand-in for the better-enums BETTER_ENUM macro (the real library is not vendored in
// the reference). Supports what the bridged reference code uses: unary '+' to the enum class,
// equality, _from_string_nothrow, _to_string and _to_integral, with implicit 0-based values.
#pragma once
#include <cstring>
#include <optional>
#include <string>

namespace betterenum_stub
{
inline int
index_of(const char * list, const char * name)
{
  std::string s(list);
  int         idx = 0;
  size_t      pos = 0;
  while (pos <= s.size())
  {
    size_t      end = s.find(',', pos);
    std::string tok = s.substr(pos, end == std::string::npos ? std::string::npos : end - pos);
    size_t      a = tok.find_first_not_of(" \t\n");
    size_t      b = tok.find_last_not_of(" \t\n");
    tok = a == std::string::npos ? "" : tok.substr(a, b - a + 1);
    if (tok == name)
      return idx;
    if (end == std::string::npos)
      break;
    pos = end + 1;
    ++idx;
  }
  return -1;
}
} // namespace betterenum_stub

#define BETTER_ENUM(Name, Underlying, ...)                                                        \
  struct Name                                                                                     \
  {                                                                                               \
    enum _enumerated : Underlying                                                                 \
    {                                                                                             \
      __VA_ARGS__                                                                                 \
    };                                                                                            \
    _enumerated v;                                                                                \
    constexpr Name()                                                                              \
      : v(static_cast<_enumerated>(0))                                                            \
    {}                                                                                            \
    constexpr Name(_enumerated e)                                                                 \
      : v(e)                                                                                      \
    {}                                                                                            \
    constexpr Underlying _to_integral() const { return static_cast<Underlying>(v); }             \
    constexpr operator _enumerated() const { return v; }                                          \
    static std::optional<Name> _from_string_nothrow(const char * s)                               \
    {                                                                                             \
      int i = betterenum_stub::index_of(#__VA_ARGS__, s);                                         \
      if (i < 0)                                                                                  \
        return std::nullopt;                                                                      \
      return Name(static_cast<_enumerated>(i));                                                   \
    }                                                                                             \
    const char * _to_string() const { return #Name; }                                             \
  };                                                                                              \
  constexpr Name operator+(Name::_enumerated e) { return Name(e); }
