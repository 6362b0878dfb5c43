// Stand-in for boundcraft (fetched by Spira at GIT_TAG main, unpinned). Spira
// names boundcraft::policy::hybrid<32> in two type aliases and never uses them.
#pragma once
#include <cstddef>
namespace boundcraft::policy {
template <std::size_t N> struct hybrid {};
}
