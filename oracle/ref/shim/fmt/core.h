// Stand-in for {fmt}: the reference headers only call fmt::format with literal
// format strings, which std::format (C++20) accepts unchanged.
#pragma once
#include <format>
namespace fmt {
using std::format;
}
