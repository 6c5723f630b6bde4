// Stub of kalypsso's ini-backed ConfigMap: a flat section/key -> string map.
#pragma once
#include <map>
#include <string>
namespace kalypsso
{
class ConfigMap
{
public:
  void set(const std::string & sec, const std::string & key, const std::string & val)
  {
    m[sec + "/" + key] = val;
  }
  double getReal(const std::string & sec, const std::string & key, double def) const
  {
    auto it = m.find(sec + "/" + key);
    return it == m.end() ? def : std::stod(it->second);
  }
  int getInteger(const std::string & sec, const std::string & key, int def) const
  {
    auto it = m.find(sec + "/" + key);
    return it == m.end() ? def : std::stoi(it->second);
  }
  bool getBool(const std::string & sec, const std::string & key, bool def) const
  {
    auto it = m.find(sec + "/" + key);
    return it == m.end() ? def : (it->second == "true" || it->second == "1");
  }
  std::string getString(const std::string & sec, const std::string & key, const std::string & def) const
  {
    auto it = m.find(sec + "/" + key);
    return it == m.end() ? def : it->second;
  }

private:
  std::map<std::string, std::string> m;
};
} // namespace kalypsso
