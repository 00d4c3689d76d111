// window_host.cpp - one window through the device code of the batched
// kernel (spoa_gb300/csrc/poa_window.cuh: forward pass with its CTA scans,
// traceback, strand choice, AddAlignment, topological sort, consensus, MSA),
// run on the host by the SIMT emulation of simt_host.h: one emulated CTA
// (or cluster of CTAs) of `nt` threads runs all reads of the window in one
// launch, as the batched kernels do.  TEST INFRASTRUCTURE ONLY
// (tests/test_window_host.py compares it with the oracle); the product runs
// the same functions on the GPU.
#include "simt_host.h"

#include "../../spoa_gb300/csrc/poa_window.cuh"

using namespace spoa_gb300;

namespace {

template <int SUB, int CPT, typename T, int SEGS = 1, int NT = 0>
int32_t run(const Scoring& S, uint32_t n_reads, const char* seqs, const uint64_t* off,
            const char* quals, int32_t strand, uint32_t nt, int32_t* scores, int32_t* rev,
            int32_t* aln, uint64_t aln_cap, uint64_t* aln_off, char* cons, uint32_t cons_cap,
            uint32_t* cons_len, char* msa, uint64_t msa_cap, uint32_t* msa_dims) {
  uint64_t sum = 0;
  uint32_t lmax = 1;
  for (uint32_t r = 0; r < n_reads; ++r) {
    sum += off[r + 1] - off[r];
    lmax = std::max<uint32_t>(lmax, (uint32_t)(off[r + 1] - off[r]));
  }
  GraphCaps gc{(uint32_t)sum + 2, 2 * (uint32_t)sum + n_reads + 8, (uint32_t)sum + n_reads + 8,
               n_reads + 1, 31};
  GraphView G;
  std::vector<uint8_t> gbuf(graph_layout(nullptr, gc, &G) + 256);
  graph_layout(gbuf.data(), gc, &G);
  DpCaps dc{gc.nodes + 1, CPT * nt * SEGS, gc.edges + gc.nodes + 2, S.sub, sizeof(T)};
  DpView D;
  std::vector<uint8_t> dbuf(dp_layout(nullptr, dc, &D) + 256);
  dp_layout(dbuf.data(), dc, &D);
  BlockScratch sh;
  SharedState ss;
  // the whole window in one launch, read after read, as the batched kernel
  // (k_batch) runs it: a CTA barrier after each read's outputs, nothing
  // else between the reads
  uint64_t na = 0;
  int32_t status = kOk;
  int32_t score = 0, rv = 0;
  const int32_t* pairs = nullptr;
  uint32_t np = 0, s_dims[2];
  aln_off[0] = 0;
  simt::launch(nt, [&] {
    if (threadIdx.x == 0) g_reset(G);
    __syncthreads();
    for (uint32_t r = 0; r < n_reads; ++r) {
      const uint32_t L = (uint32_t)(off[r + 1] - off[r]);
      const uint8_t* seq = reinterpret_cast<const uint8_t*>(seqs) + off[r];
      const uint8_t* qual = quals ? reinterpret_cast<const uint8_t*>(quals) + off[r] : nullptr;
      window_read<SUB, CPT, T, SEGS, NT>(S, G, D, sh, ss, seq, L, qual, strand != 0, &score,
                                         &rv, &pairs, &np);
      if (ss.status != kOk) {
        if (threadIdx.x == 0) status = ss.status;
        return;
      }
      if (threadIdx.x == 0) {
        scores[r] = score;
        rev[r] = rv;
        if (na + np > aln_cap) {
          status = kCapacity;
        } else {
          for (uint32_t k = 0; k < 2 * np; ++k) aln[2 * na + k] = pairs[k];
          na += np;
          aln_off[r + 1] = na;
        }
      }
      __syncthreads();
      if (status != kOk) return;
    }
    if (threadIdx.x == 0)
      write_consensus(G, reinterpret_cast<uint8_t*>(cons), cons_cap, cons_len);
    __syncthreads();
    if (msa) {
      // the MSA as the batched kernel writes it: rows spread over the CTA
      const int32_t st = window_msa(G, false, reinterpret_cast<uint8_t*>(msa), msa_cap,
                                    &msa_dims[0], &msa_dims[1], s_dims);
      if (threadIdx.x == 0 && st != kOk) status = st;
    }
  });
  return status;
}

// One window through window_read_cl on a cluster of CL emulated CTAs of nt
// threads each (every CTA its own shared state, the row spread over them).
template <int SUB, int CPT, typename T, int CL>
int32_t run_cl(const Scoring& S, uint32_t n_reads, const char* seqs, const uint64_t* off,
               const char* quals, int32_t strand, uint32_t nt, int32_t* scores, int32_t* rev,
               int32_t* aln, uint64_t aln_cap, uint64_t* aln_off, char* cons, uint32_t cons_cap,
               uint32_t* cons_len) {
  uint64_t sum = 0;
  for (uint32_t r = 0; r < n_reads; ++r) sum += off[r + 1] - off[r];
  GraphCaps gc{(uint32_t)sum + 2, 2 * (uint32_t)sum + n_reads + 8, (uint32_t)sum + n_reads + 8,
               n_reads + 1, 31};
  GraphView G;
  std::vector<uint8_t> gbuf(graph_layout(nullptr, gc, &G) + 256);
  graph_layout(gbuf.data(), gc, &G);
  DpCaps dc{gc.nodes + 1, CPT * nt * CL, gc.edges + gc.nodes + 2, S.sub, sizeof(T)};
  DpView D;
  std::vector<uint8_t> dbuf(dp_layout(nullptr, dc, &D) + 256);
  dp_layout(dbuf.data(), dc, &D);
  struct CtaShared {
    BlockScratch sh;
    SharedState ss;
  };
  std::vector<CtaShared> cs(CL);
  std::vector<char*> scratch;
  for (auto& c : cs) scratch.push_back(reinterpret_cast<char*>(&c));
  // the whole window in one launch, as k_batch_cl runs it: the lead CTA's
  // thread 0 takes each read's outputs, no other barrier between reads
  uint64_t na = 0;
  int32_t status = kOk;
  int32_t score = 0, rv = 0;
  const int32_t* pairs = nullptr;
  uint32_t np = 0;
  aln_off[0] = 0;
  simt::launch_cluster(CL, nt, scratch, [&] {
    CtaShared& me = cs[simt::cta_rank];
    const bool lead = simt::cta_rank == 0;
    if (lead && threadIdx.x == 0) g_reset(G);
    cl_sync<CL>();
    for (uint32_t r = 0; r < n_reads; ++r) {
      const uint32_t L = (uint32_t)(off[r + 1] - off[r]);
      const uint8_t* seq = reinterpret_cast<const uint8_t*>(seqs) + off[r];
      const uint8_t* qual = quals ? reinterpret_cast<const uint8_t*>(quals) + off[r] : nullptr;
      const int32_t st = window_read_cl<SUB, CPT, T, CL>(S, G, D, me.sh, me.ss, seq, L, qual,
                                                         strand != 0, &score, &rv, &pairs, &np);
      if (st != kOk) {
        if (lead && threadIdx.x == 0) status = st;
        break;
      }
      if (lead && threadIdx.x == 0) {
        scores[r] = score;
        rev[r] = rv;
        if (na + np > aln_cap) {
          status = kCapacity;
        } else {
          for (uint32_t k = 0; k < 2 * np; ++k) aln[2 * na + k] = pairs[k];
          na += np;
          aln_off[r + 1] = na;
        }
      }
    }
    if (lead && threadIdx.x == 0 && status == kOk)
      write_consensus(G, reinterpret_cast<uint8_t*>(cons), cons_cap, cons_len);
    cl_sync<CL>();
  });
  return status;
}

}  // namespace

extern "C" int32_t wh_run(int32_t type, int32_t m, int32_t n, int32_t g, int32_t e, int32_t q,
                          int32_t c, int32_t wide, int32_t cpt, uint32_t nt, uint32_t n_reads,
                          const char* seqs, const uint64_t* off, const char* quals,
                          int32_t strand, int32_t* scores, int32_t* rev, int32_t* aln,
                          uint64_t aln_cap, uint64_t* aln_off, char* cons, uint32_t cons_cap,
                          uint32_t* cons_len, char* msa, uint64_t msa_cap, uint32_t* msa_dims) {
  // AlignmentEngine::Create's subtype and canonical penalties
  // (alignment_engine.cpp:57-66)
  const int32_t sub = g >= e ? kLinear : ((g <= q || e >= c) ? kAffine : kConvex);
  if (sub == kLinear) {
    e = g;
  } else if (sub == kAffine) {
    q = g;
    c = e;
  }
  const Scoring S{type, sub, m, n, g, e, q, c};
#define RUN(SUBV, C, TT, ...)                                                              \
  return run<SUBV, C, TT, ##__VA_ARGS__>(S, n_reads, seqs, off, quals, strand, nt, scores, rev, \
                                         aln, aln_cap, aln_off, cons, cons_cap, cons_len, msa, \
                                         msa_cap, msa_dims)
#define BY_SUB(C, TT)                   \
  switch (sub) {                        \
    case kLinear: RUN(kLinear, C, TT);  \
    case kAffine: RUN(kAffine, C, TT);  \
    default: RUN(kConvex, C, TT);       \
  }
  if (cpt == 8) {
    if (wide) BY_SUB(8, int32_t) else BY_SUB(8, int16_t)
  }
  if (cpt == 16 && nt == 32 && !wide) {  // the one-warp build of the forward pass (NT = 32)
    switch (sub) {
      case kLinear: RUN(kLinear, 16, int16_t, 1, 32);
      case kAffine: RUN(kAffine, 16, int16_t, 1, 32);
      default: RUN(kConvex, 16, int16_t, 1, 32);
    }
  }
  if (cpt == -12) {  // the segmented forward: two 12-column strips per thread, 32-bit lanes
    switch (sub) {
      case kLinear: RUN(kLinear, 12, int32_t, 2);
      case kAffine: RUN(kAffine, 12, int32_t, 2);
      default: RUN(kConvex, 12, int32_t, 2);
    }
  }
  if (wide) BY_SUB(16, int32_t) else BY_SUB(16, int16_t)
#undef BY_SUB
#undef RUN
}

// mq_path of the cluster forward (the best path of a Q' carry into E'),
// for a unit test against the brute-force maximum.
extern "C" int32_t wh_mq_path(int32_t u, int32_t c, int32_t e, int32_t lanes) {
  return mq_path(u, c, e, lanes);
}

// The cluster form (window_read_cl): cl CTAs of nt threads, 12 columns per
// thread, 32-bit lanes.
extern "C" int32_t wh_run_cl(int32_t type, int32_t m, int32_t n, int32_t g, int32_t e, int32_t q,
                             int32_t c, int32_t cl, uint32_t nt, uint32_t n_reads,
                             const char* seqs, const uint64_t* off, const char* quals,
                             int32_t strand, int32_t* scores, int32_t* rev, int32_t* aln,
                             uint64_t aln_cap, uint64_t* aln_off, char* cons, uint32_t cons_cap,
                             uint32_t* cons_len) {
  const int32_t sub = g >= e ? kLinear : ((g <= q || e >= c) ? kAffine : kConvex);
  if (sub == kLinear) {
    e = g;
  } else if (sub == kAffine) {
    q = g;
    c = e;
  }
  const Scoring S{type, sub, m, n, g, e, q, c};
#define RUNC(SUBV, CLV)                                                                     \
  return run_cl<SUBV, 12, int32_t, CLV>(S, n_reads, seqs, off, quals, strand, nt, scores, rev, \
                                        aln, aln_cap, aln_off, cons, cons_cap, cons_len)
#define BY_SUBC(CLV)                     \
  switch (sub) {                         \
    case kLinear: RUNC(kLinear, CLV);    \
    case kAffine: RUNC(kAffine, CLV);    \
    default: RUNC(kConvex, CLV);         \
  }
  if (cl == 2) BY_SUBC(2)
  if (cl == 8) BY_SUBC(8)
  BY_SUBC(4)
#undef BY_SUBC
#undef RUNC
}
