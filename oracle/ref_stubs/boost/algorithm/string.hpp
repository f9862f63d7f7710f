// Stand-in for the single Boost string routine the reference calls
// (case-insensitive equality of two std::strings, used to pick the logger).
#ifndef ST_ORACLE_BOOST_STRING_STUB
#define ST_ORACLE_BOOST_STRING_STUB
#include <string>
#include <cctype>
namespace boost {
inline bool iequals(const std::string& a, const std::string& b) {
  if (a.size() != b.size()) return false;
  for (std::size_t i = 0; i < a.size(); ++i)
    if (std::tolower(static_cast<unsigned char>(a[i])) != std::tolower(static_cast<unsigned char>(b[i]))) return false;
  return true;
}
}  // namespace boost
#endif
