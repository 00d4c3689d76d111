// batch_mw_host.cpp - the W-windows-per-CTA batched loop
// (spoa_gb300/csrc/poa_batch_mw.cuh) run on the host by the SIMT emulation
// of simt_host.h: one CTA pulls every window of the batch from the queue.
// TEST INFRASTRUCTURE ONLY (tests/test_batch_mw_host.py compares it with
// the oracle).
#include "simt_host.h"

#include "../../spoa_gb300/csrc/poa_batch_mw.cuh"

using namespace spoa_gb300;

namespace {

template <int SUB, int W>
int32_t run(const Scoring& S, uint32_t n_windows, const uint32_t* wro, const char* seqs,
            const uint64_t* off, int32_t* scores, uint8_t* rev, char* cons,
            const uint64_t* cons_off, uint32_t* cons_len, int32_t* win_status,
            const int8_t* strands, const char* quals) {
  constexpr int CPT = 8;
  uint64_t maxsum = 1;
  uint32_t lmax = 1, maxreads = 1;
  for (uint32_t w = 0; w < n_windows; ++w) {
    maxsum = std::max<uint64_t>(maxsum, off[wro[w + 1]] - off[wro[w]]);
    maxreads = std::max(maxreads, wro[w + 1] - wro[w]);
    for (uint32_t r = wro[w]; r < wro[w + 1]; ++r)
      lmax = std::max<uint32_t>(lmax, (uint32_t)(off[r + 1] - off[r]));
  }
  const uint32_t nt = 32 * std::max<uint32_t>(1, (lmax + CPT * 32 - 1) / (CPT * 32));
  GraphCaps gc{(uint32_t)maxsum + 2, 2 * (uint32_t)maxsum + maxreads + 8,
               (uint32_t)maxsum + maxreads + 8, maxreads + 1, 31};
  DpCaps dc{gc.nodes + 1, CPT * nt, gc.edges + gc.nodes + 2, S.sub, 2};
  DpView D;
  GraphView Gs[W];
  int32_t* pairs[W];
  uint8_t* reads[W];
  uint32_t* pre[W];
  std::vector<uint8_t> arena(mw_layout(nullptr, W, gc, dc, &D, nullptr, nullptr, nullptr) + 256);
  mw_layout(arena.data(), W, gc, dc, &D, Gs, pairs, reads, pre);
  std::vector<uint32_t> work(n_windows);
  for (uint32_t w = 0; w < n_windows; ++w) work[w] = w;
  uint32_t queue = 0;
  unsigned long long cells[2] = {0, 0};
  BatchArgs a{};
  a.base = S;
  a.win_strand = strands;
  a.n_windows = n_windows;
  a.win_read_off = wro;
  a.seqs = reinterpret_cast<const uint8_t*>(seqs);
  a.seq_off = off;
  a.quals = reinterpret_cast<const uint8_t*>(quals);
  a.work = work.data();
  a.n_work = n_windows;
  a.queue = &queue;
  a.read_scores = scores;
  a.read_rev = rev;
  a.cons = reinterpret_cast<uint8_t*>(cons);
  a.cons_off = cons_off;
  a.cons_len = cons_len;
  a.win_status = win_status;
  a.cells = cells;
  a.pred_cells = cells + 1;
  BlockScratch sh;
  SharedState ss;
  // shared memory starts with arbitrary contents: so does the emulation
  MwSlot slot[W];
  MwShared m;
  std::memset(static_cast<void*>(slot), 0xAB, sizeof(slot));
  std::memset(static_cast<void*>(&m), 0xAB, sizeof(m));
  simt::launch(nt, [&] { batch_cta_mw<SUB, CPT, int16_t, W>(a, sh, ss, slot, Gs, D, pairs, reads, pre, m); });
  return kOk;
}

}  // namespace

extern "C" int32_t mw_run(int32_t type, int32_t m, int32_t n, int32_t g, int32_t e, int32_t q,
                          int32_t c, int32_t W, uint32_t n_windows, const uint32_t* wro,
                          const char* seqs, const uint64_t* off, const int8_t* strands,
                          int32_t* scores, uint8_t* rev, char* cons, const uint64_t* cons_off,
                          uint32_t* cons_len, int32_t* win_status, const char* quals) {
  const int32_t sub = g >= e ? kLinear : ((g <= q || e >= c) ? kAffine : kConvex);
  if (sub == kLinear) {
    e = g;
  } else if (sub == kAffine) {
    q = g;
    c = e;
  }
  const Scoring S{type, sub, m, n, g, e, q, c};
#define RUN(SUBV, WV) \
  return run<SUBV, WV>(S, n_windows, wro, seqs, off, scores, rev, cons, cons_off, cons_len, \
                       win_status, strands, quals)
#define BY_SUB(WV)                    \
  switch (sub) {                      \
    case kLinear: RUN(kLinear, WV);   \
    case kAffine: RUN(kAffine, WV);   \
    default: RUN(kConvex, WV);        \
  }
  if (W == 1) BY_SUB(1)
  if (W == 2) BY_SUB(2)
  BY_SUB(4)
#undef BY_SUB
#undef RUN
}
