// simt_selftest.cpp - checks of the SIMT emulation itself (simt_host.h).
// TEST INFRASTRUCTURE ONLY: tests/test_window_host.py runs it.
//   simt_selftest ok    - shuffles, CTA and split cluster barriers give the
//                         values a GPU gives; exits 0
//   simt_selftest skip  - one thread leaves before a __syncthreads that the
//                         others wait at; the emulation must abort with a
//                         barrier-deadlock report instead of hanging
//   simt_selftest split - threads of one CTA wait at two different
//                         __syncthreads (undefined on a GPU); the emulation
//                         must abort naming both
//   simt_selftest redzone - writes one element past the end of a graph
//                         arena's node-code region; a -fsanitize=address
//                         build with SPOA_GB300_HOST_REDZONE must report it
//   simt_selftest race  - thread 0 writes a shared value that thread 33
//                         reads with no barrier between them (a data race
//                         on a GPU); a -fsanitize=thread build must report
//                         it, while "ok" must run without a report
#include "simt_host.h"

#include "../../spoa_gb300/csrc/poa_device.cuh"

#include <cstdio>
#include <cstring>
#include <vector>

int main(int argc, char** argv) {
  const bool skip = argc > 1 && std::strcmp(argv[1], "skip") == 0;
  const bool race = argc > 1 && std::strcmp(argv[1], "race") == 0;
  if (argc > 1 && std::strcmp(argv[1], "redzone") == 0) {
    spoa_gb300::GraphCaps gc{100, 300, 300, 5, 4};
    spoa_gb300::GraphView G;
    std::vector<uint8_t> arena(spoa_gb300::graph_layout(nullptr, gc, &G));
    spoa_gb300::graph_layout(arena.data(), gc, &G);
    simt::launch(32, [&] {
      if (threadIdx.x == 0) G.code[gc.nodes] = 1;  // one past the region
    });
    std::printf("no red-zone access reported\n");
    return 0;
  }
  if (argc > 1 && std::strcmp(argv[1], "split") == 0) {
    simt::launch(64, [] {
      if (threadIdx.x < 32)
        __syncthreads();
      else
        __syncthreads();
    });
    std::printf("no split barrier reported\n");
    return 0;
  }
  if (race) {
    int shared_value = 0, seen = 0;
    simt::launch(64, [&] {
      if (threadIdx.x == 0) shared_value = 7;
      if (threadIdx.x == 33) seen = shared_value;  // no barrier: a race
      __syncthreads();
    });
    std::printf("read %d\n", seen);
    return 0;
  }
  if (skip) {
    simt::launch(64, [] {
      __syncthreads();
      if (threadIdx.x == 37) return;
      __syncthreads();
    });
    std::printf("no deadlock reported\n");
    return 0;
  }
  // warp inclusive prefix sum by shuffles, then a CTA-wide exchange
  std::vector<int> out(128), sh(128);
  simt::launch(128, [&] {
    int v = (int)threadIdx.x + 1;
    for (unsigned d = 1; d < 32; d *= 2) {
      const int u = __shfl_up_sync(0xffffffffu, v, d);
      if (threadIdx.x % 32 >= d) v += u;
    }
    sh[threadIdx.x] = v;
    __syncthreads();
    out[threadIdx.x] = sh[127 - threadIdx.x];
  });
  for (unsigned t = 0; t < 128; ++t) {
    const unsigned src = 127 - t, w0 = src / 32 * 32;
    int want = 0;
    for (unsigned k = w0; k <= src; ++k) want += (int)k + 1;
    if (out[t] != want) {
      std::printf("prefix sum: thread %u has %d, want %d\n", t, out[t], want);
      return 1;
    }
  }
  // a cluster of 4 CTAs: each publishes a value, arrives, does other work,
  // waits, then reads every peer's value through the distributed view
  struct Shared {
    int v;
  };
  std::vector<Shared> cs(4);
  std::vector<char*> scratch;
  for (auto& c : cs) scratch.push_back(reinterpret_cast<char*>(&c));
  std::vector<int> sums(4 * 32);
  simt::launch_cluster(4, 32, scratch, [&] {
    Shared& me = cs[simt::cta_rank];
    if (threadIdx.x == 0) me.v = 10 * ((int)simt::cta_rank + 1);
    simt::cluster_arrive();
    simt::cluster_wait();
    int s = 0;
    for (unsigned r = 0; r < 4; ++r) s += simt::peer(&me, r)->v;
    sums[simt::cta_rank * 32 + threadIdx.x] = s;
  });
  for (int s : sums)
    if (s != 100) {
      std::printf("cluster exchange: %d, want 100\n", s);
      return 1;
    }
  std::printf("ok\n");
  return 0;
}
