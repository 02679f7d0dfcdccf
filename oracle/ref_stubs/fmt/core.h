// Minimal stand-in for <fmt/core.h>: the reference headers compiled by oracle/Makefile only name
// fmt::format inside uninstantiated error paths.
#pragma once
#include <string>
namespace fmt {
template <class... A>
std::string format(A&&...);
} // namespace fmt
