// Zero-filling global operator new / delete, linked into the reference's
// module only (hidden visibility: calls inside that shared object bind here,
// nothing else in the process is affected).
//
// Why: the reference's BloomFilter (cpp/src/kernels/buffers.cuh:37-40) sizes
// its bitset from n_instances_ and num_sets_per_list_, but those members are
// declared after the bitset (buffers.cuh:133-136), so they are read before
// they are initialised.  The bitset size is then whatever the heap held: on a
// GB300 machine a 70,000-row session failed with std::bad_alloc.  With every
// allocation zero-filled the size is 0 on every run, so the filter is a
// deterministic no-op (check() returns false, add() stores nothing); all other
// behaviour is unchanged.  calloc / free underneath keep the allocations
// compatible with memory freed or allocated by the C++ runtime library.
#include <cstdlib>
#include <new>

#define REFSHIM_HIDDEN __attribute__((visibility("hidden")))

namespace {
void *zeroed(std::size_t n) {
  void *p = std::calloc(1, n ? n : 1);
  if (!p) throw std::bad_alloc();
  return p;
}
}  // namespace

REFSHIM_HIDDEN void *operator new(std::size_t n) { return zeroed(n); }
REFSHIM_HIDDEN void *operator new[](std::size_t n) { return zeroed(n); }
REFSHIM_HIDDEN void *operator new(std::size_t n, const std::nothrow_t &) noexcept {
  return std::calloc(1, n ? n : 1);
}
REFSHIM_HIDDEN void *operator new[](std::size_t n, const std::nothrow_t &) noexcept {
  return std::calloc(1, n ? n : 1);
}
REFSHIM_HIDDEN void operator delete(void *p) noexcept { std::free(p); }
REFSHIM_HIDDEN void operator delete[](void *p) noexcept { std::free(p); }
REFSHIM_HIDDEN void operator delete(void *p, std::size_t) noexcept { std::free(p); }
REFSHIM_HIDDEN void operator delete[](void *p, std::size_t) noexcept { std::free(p); }
