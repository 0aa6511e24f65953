// Build-local replacement for the header the reference generates from
// include/ads/config.hpp.in (CMake's #cmakedefine lines dropped: no Galois,
// no MUMPS).  Test infrastructure only.
#ifndef ADS_CONFIG_HPP
#define ADS_CONFIG_HPP

#include <string_view>

namespace ads {

struct version_info {
    std::string_view core;
    std::string_view commit;
    std::string_view full;
    int major;
    int minor;
    int patch;
};

auto version() -> version_info;

}  // namespace ads

#endif  // ADS_CONFIG_HPP
