// Internal helpers shared between the C-ABI translation units.
#pragma once
#include <string>

namespace eff {
// Record `msg` as the calling thread's eff_last_error() and return `code`.
int set_error(int code, const std::string& msg);
}  // namespace eff
