// Drives the reference's own queue implementations (cpp/src/queue.cuh,
// compiled in place from the reference tree) through a fixed script and
// prints every pop, one line per pop: "<queue> <requested> <ids...>".
// The output is committed as tests/golden/queue_golden.txt.
#include <cstdint>
#include <cstdio>
#include <vector>

#include "queue.cuh"

int main() {
  gpumap::InsertionQueue iq;
  gpumap::UpdateQueue uq;
  unsigned state = 12345u;
  auto next = [&]() {
    state = state * 1664525u + 1013904223u;
    return state >> 8;
  };
  for (int step = 0; step < 200; ++step) {
    const unsigned op = next() % 4u;
    if (op < 2) {
      std::vector<uint32_t> items;
      const unsigned m = next() % 40u;
      for (unsigned i = 0; i < m; ++i) items.push_back(next() % 64u);
      uq.push_batch(items);
      std::vector<uint32_t> seq;
      for (unsigned i = 0; i < m; ++i) seq.push_back(step * 100u + i);
      iq.push_batch(seq);
      std::printf("push %u", m);
      for (auto v : items) std::printf(" %u", v);
      std::printf("\n");
    } else {
      const unsigned req = next() % 50u;
      auto a = uq.pop_n(req);
      std::printf("upop %u", req);
      for (auto v : a) std::printf(" %u", v);
      std::printf("\n");
      auto b = iq.pop_n(req);
      std::printf("ipop %u", req);
      for (auto v : b) std::printf(" %u", v);
      std::printf("\n");
    }
  }
  std::printf("usize %zu\n", uq.size());
  return 0;
}
