// Stand-in for TBB's scalable allocator (oracle-only test infrastructure).
#pragma once
#include <cstdlib>
#include <cstddef>
inline void* scalable_malloc(size_t n) { return std::malloc(n ? n : 1); }
inline void scalable_free(void* p) { std::free(p); }
inline void* scalable_aligned_malloc(size_t n, size_t align) {
    if (align < sizeof(void*)) align = sizeof(void*);
    size_t sz = ((n ? n : 1) + align - 1) / align * align;
    return std::aligned_alloc(align, sz);
}
inline void scalable_aligned_free(void* p) { std::free(p); }
