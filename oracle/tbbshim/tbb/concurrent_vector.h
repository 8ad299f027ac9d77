// Stand-in for tbb::concurrent_vector (oracle-only; used single-threaded here).
#pragma once
#include <vector>
#include <memory>
namespace tbb {
template <typename T, typename A = std::allocator<T>>
class concurrent_vector : public std::vector<T, A> {
public:
    using std::vector<T, A>::vector;
};
}
