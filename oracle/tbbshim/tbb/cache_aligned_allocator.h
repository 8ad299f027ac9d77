// Stand-in for tbb::cache_aligned_allocator (oracle-only test infrastructure).
#pragma once
#include <memory>
namespace tbb {
template <typename T>
using cache_aligned_allocator = std::allocator<T>;
}
