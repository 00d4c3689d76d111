// poa_window.cuh - device code of one window, shared by the kernels of
// poa_kernels.cuh: the per-read prologue, one read's alignment (both strands
// when asked), the strand choice and the graph update, the consensus and
// the MSA.  Device functions only (no kernels, no host API), so the same
// code can also be built for the host by the test harness.
#pragma once

#include <cstdint>

#include "poa_device.cuh"
#include "poa_dp.cuh"

namespace spoa_gb300 {

struct ReadOut {
  int32_t status;
  int32_t has_score;
  int32_t score;
  int32_t reversed;
  uint32_t n_pairs;
  int32_t lanes;
};

struct SharedState {
  int32_t status, mode, lanes, pad;
  int64_t max_i, max_j;
  int32_t score, has_f, score_f, has_r, score_r;
  uint32_t np_f, np_r;
};

// Align one read (seq, or its reverse complement staged in D.seq_rc) against
// the current graph; thread 0 leaves the pairs in `pairs` and returns
// has_score/score through `ss`.  Every thread must call it.
// T is the arithmetic of the kernel: int16 pairs when every read of the
// window passes the reference's int16 width rule (implementation.hpp:719-775),
// int32 otherwise.  An int32 kernel runs int16-width reads with the 16-lane
// semantics (vector starts of the convex E recurrence, -infinity of the NW
// row selection), which gives the same results.
template <int SUB, int CPT, typename T, int SEGS = 1, int NT = 0>
__device__ void read_align(const Scoring& S, const GraphView& G, DpView& D, BlockScratch& sh,
                           SharedState& ss, const uint8_t* seq, uint32_t L, int32_t lanes,
                           int32_t* pairs, int32_t* has, int32_t* score, uint32_t* np) {
  int64_t mi, mj;
  int32_t sc;
  const uint32_t V = G.hdr->n_nodes;
  if constexpr (SEGS == 1)
    dp_forward<SUB, CPT, T, NT>(S, D, seq, L, V, lanes, sh, &mi, &mj, &sc);
  else
    dp_forward_seg<SUB, CPT, T, SEGS>(S, D, seq, L, V, lanes, sh, &mi, &mj, &sc);
  if (threadIdx.x == 0) {
    *np = 0;
    *has = 0;
    if (mi >= 0) {
      *has = 1;
      *score = sc;
      const int32_t st =
          dp_traceback<SUB, CPT, T>(S, D, G, seq, L, V, mi, mj, pairs, np, blockDim.x * SEGS);
      if (st != kOk) ss.status = st;
    }
  }
  __syncthreads();
}

// Checks done before a read's DP (thread 0): mode 0 = empty alignment,
// 1 = run the DP; status on error.
__device__ inline void read_prologue(const Scoring& S, const GraphView& G, const DpView& D,
                                     uint32_t L, uint32_t nthreads_cols, bool wide_ok,
                                     SharedState& ss) {
  const uint32_t V = G.hdr->n_nodes;
  ss.status = kOk;
  ss.mode = 0;
  ss.lanes = 16;
  // every read is staged in buffers of caps.ld bytes (the reverse
  // complement, the multi-window slots), the first one too
  if (L > nthreads_cols || L > D.caps.ld) {
    ss.status = kCapacity;
    return;
  }
  if (V == 0 || L == 0) return;
  int32_t lanes = lanes_for(S, L, V);
  if (!lanes) {
    ss.status = kOverflow;
    return;
  }
  if (lanes == 8 && !wide_ok) {
    ss.status = kNeedWide;  // rerun the window with the int32 kernel
    return;
  }
  if (V + 1 > D.caps.rows || (uint64_t)G.hdr->n_edges + V + 1 > D.caps.preds) {
    ss.status = kCapacity;
    return;
  }
  ss.lanes = lanes;
  ss.mode = 1;
}

// One read of a window: align (both strands when asked), choose, add.
// NT: the CTA's threads when known at compile time (dp_forward).
template <int SUB, int CPT, typename T, int SEGS = 1, int NT = 0>
__device__ void window_read(const Scoring& S, GraphView& G, DpView& D, BlockScratch& sh,
                            SharedState& ss, const uint8_t* seq, uint32_t L,
                            const uint8_t* qual, bool strand, int32_t* out_score,
                            int32_t* out_rev, const int32_t** out_pairs, uint32_t* out_np) {
  if (threadIdx.x == 0) read_prologue(S, G, D, L, blockDim.x * CPT * SEGS, sizeof(T) == 4, ss);
  __syncthreads();
  if (ss.status != kOk) return;
  const bool dp = ss.mode == 1;
  if (threadIdx.x == 0) {
    ss.has_f = ss.has_r = 0;
    ss.score_f = ss.score_r = 0;
    ss.np_f = ss.np_r = 0;
  }
  if (dp) {
    dp_build_rows(G, D, sh);
    read_align<SUB, CPT, T, SEGS, NT>(S, G, D, sh, ss, seq, L, ss.lanes, D.aln_a, &ss.has_f,
                                      &ss.score_f, &ss.np_f);
  }
  if (strand) {
    for (uint32_t j = threadIdx.x; j < L; j += blockDim.x)
      D.seq_rc[j] = complement_base(seq[L - 1 - j]);
    __syncthreads();
    if (dp && ss.status == kOk)
      read_align<SUB, CPT, T, SEGS, NT>(S, G, D, sh, ss, D.seq_rc, L, ss.lanes, D.aln_b,
                                        &ss.has_r, &ss.score_r, &ss.np_r);
  }
  __syncthreads();
  if (ss.status == kOk) {
    // main.cpp:276-301: scores start at 0; keep forward if score >= score_rev
    const int32_t sf = ss.has_f ? ss.score_f : 0;
    const int32_t sr = ss.has_r ? ss.score_r : 0;
    const bool rev = strand && !(sf >= sr);
    const int32_t* pairs = rev ? D.aln_b : D.aln_a;
    const uint32_t np = rev ? ss.np_r : ss.np_f;
    const uint8_t* chosen = rev ? D.seq_rc : seq;
    // AddAlignment's read-only lookups on every thread, into the alignment
    // buffer the strand choice left unused (two words per pair fit it)
    uint32_t* pre = reinterpret_cast<uint32_t*>(rev ? D.aln_a : D.aln_b);
    g_add_prepass(G, pairs, np, chosen, L, pre);
    if (threadIdx.x == 0) {
      WeightSrc ws{nullptr, qual, L, rev ? 1u : 0u, 1u};
      int32_t st = g_add_alignment(G, pairs, np, chosen, L, ws, pre);
      if (st != kOk) ss.status = st;
      *out_score = rev ? sr : sf;
      *out_rev = rev ? 1 : 0;
      *out_pairs = pairs;
      *out_np = np;
    }
  }
  __syncthreads();
  if (ss.status == kOk && L > 0) {
    int* ret = &ss.pad;
    if (g_topo_sort_cta(G, ret) != 0 && threadIdx.x == 0) ss.status = kCapacity;
    __syncthreads();
  }
}

// One read of a window on a cluster of CL CTAs (long rows): every CTA of
// the cluster calls it.  The forward pass runs on all of them, each CTA a
// column range of the row (dp_forward with CL); the prologue, the row
// metadata, the traceback, the strand choice, AddAlignment and the sort run
// on CTA 0 (the lead), and every decision is read back from the lead's
// shared state after a cluster barrier, so each CTA takes the same path
// and meets the same barriers.  Returns the status (the same in every
// thread of the cluster); the lead's thread 0 gets the outputs.
template <int SUB, int CPT, typename T, int CL>
__device__ int32_t window_read_cl(const Scoring& S, GraphView& G, DpView& D, BlockScratch& sh,
                                  SharedState& ss, const uint8_t* seq, uint32_t L,
                                  const uint8_t* qual, bool strand, int32_t* out_score,
                                  int32_t* out_rev, const int32_t** out_pairs, uint32_t* out_np) {
  const bool lead = cl_rank<CL>() == 0;
  const uint32_t ntv = blockDim.x * CL;
  if (lead && threadIdx.x == 0) {
    read_prologue(S, G, D, L, ntv * CPT, sizeof(T) == 4, ss);
    ss.has_f = ss.has_r = 0;
    ss.score_f = ss.score_r = 0;
    ss.np_f = ss.np_r = 0;
  }
  cl_sync<CL>();
  int32_t st = cl_peek(&ss.status, 0);
  if (st != kOk) return st;
  const bool dp = cl_peek(&ss.mode, 0) == 1;
  const int32_t lanes = cl_peek(&ss.lanes, 0);
  // Read only when this read is aligned: a read that is only added (the
  // first one, without strands) reaches the lead's AddAlignment, which
  // rewrites the count, with no cluster barrier after this point.
  const uint32_t V = dp ? G.hdr->n_nodes : 0u;
  auto align = [&](const uint8_t* sq, int32_t* pairs, int32_t* has, int32_t* score,
                   uint32_t* np) {
    int64_t mi, mj;
    int32_t sc;
    dp_forward_cl<SUB, CPT, T, CL>(S, D, sq, L, V, lanes, sh, &mi, &mj, &sc);
    if (lead && threadIdx.x == 0) {
      *np = 0;
      *has = 0;
      if (mi >= 0) {
        *has = 1;
        *score = sc;
        const int32_t t = dp_traceback<SUB, CPT, T>(S, D, G, sq, L, V, mi, mj, pairs, np, ntv);
        if (t != kOk) ss.status = t;
      }
    }
    cl_sync<CL>();
  };
  if (dp) {
    if (lead) dp_build_rows(G, D, sh);
    cl_sync<CL>();
    align(seq, D.aln_a, &ss.has_f, &ss.score_f, &ss.np_f);
  }
  if (strand) {
    if (lead)
      for (uint32_t j = threadIdx.x; j < L; j += blockDim.x)
        D.seq_rc[j] = complement_base(seq[L - 1 - j]);
    cl_sync<CL>();
    st = cl_peek(&ss.status, 0);
    if (dp && st == kOk) align(D.seq_rc, D.aln_b, &ss.has_r, &ss.score_r, &ss.np_r);
  }
  if (lead && cl_peek(&ss.status, 0) == kOk) {
    // main.cpp:276-301: scores start at 0; keep forward if score >= score_rev
    const int32_t sf = ss.has_f ? ss.score_f : 0;
    const int32_t sr = ss.has_r ? ss.score_r : 0;
    const bool rev = strand && !(sf >= sr);
    const int32_t* pairs = rev ? D.aln_b : D.aln_a;
    const uint32_t np = rev ? ss.np_r : ss.np_f;
    const uint8_t* chosen = rev ? D.seq_rc : seq;
    uint32_t* pre = reinterpret_cast<uint32_t*>(rev ? D.aln_a : D.aln_b);
    g_add_prepass(G, pairs, np, chosen, L, pre);
    if (threadIdx.x == 0) {
      WeightSrc ws{nullptr, qual, L, rev ? 1u : 0u, 1u};
      const int32_t a = g_add_alignment(G, pairs, np, chosen, L, ws, pre);
      if (a != kOk) ss.status = a;
      *out_score = rev ? sr : sf;
      *out_rev = rev ? 1 : 0;
      *out_pairs = pairs;
      *out_np = np;
    }
    __syncthreads();
    if (ss.status == kOk && L > 0) {
      int* ret = &ss.pad;
      if (g_topo_sort_cta(G, ret) != 0 && threadIdx.x == 0) ss.status = kCapacity;
      __syncthreads();
    }
  }
  cl_sync<CL>();
  st = cl_peek(&ss.status, 0);
  // the lead rewrites ss for the next read only after every CTA has read it
  cl_sync<CL>();
  return st;
}

__device__ inline void write_consensus(GraphView& G, uint8_t* out, uint64_t cap, uint32_t* len) {
  g_consensus(G);
  const uint32_t n = G.hdr->n_consensus;
  for (uint32_t k = 0; k < n && k < cap; ++k)
    out[k] = (uint8_t)G.hdr->decoder[G.code[G.consensus[k]]];
  *len = n;
}

// MSA of the window into out[rows * cols]; every thread calls.
static __device__ __noinline__ int32_t window_msa(GraphView& G, bool include_consensus, uint8_t* out,
                                     uint64_t cap, uint32_t* rows_out, uint32_t* cols_out,
                                     uint32_t* s_dims) {
  if (threadIdx.x == 0) {
    s_dims[1] = g_msa_columns(G);
    if (include_consensus) g_consensus(G);
    s_dims[0] = G.hdr->n_seqs + (include_consensus ? 1 : 0);
    *rows_out = s_dims[0];
    *cols_out = s_dims[1];
  }
  __syncthreads();
  const uint32_t rows = s_dims[0], cols = s_dims[1];
  if ((uint64_t)rows * cols > cap) return kCapacity;
  for (uint64_t k = threadIdx.x; k < (uint64_t)rows * cols; k += blockDim.x) out[k] = '-';
  __syncthreads();
  const uint32_t ns = G.hdr->n_seqs;
  for (uint32_t s = threadIdx.x; s < ns; s += blockDim.x) {
    uint8_t* row = out + (uint64_t)s * cols;
    uint32_t it = G.seq_begin[s];
    uint32_t guard = 0;
    while (it != kNone && guard++ <= G.hdr->n_nodes) {
      row[G.column[it]] = (uint8_t)G.hdr->decoder[G.code[it]];
      it = g_successor(G, it, s);
    }
  }
  if (include_consensus && threadIdx.x == 0) {
    uint8_t* row = out + (uint64_t)ns * cols;
    for (uint32_t k = 0; k < G.hdr->n_consensus; ++k) {
      uint32_t it = G.consensus[k];
      row[G.column[it]] = (uint8_t)G.hdr->decoder[G.code[it]];
    }
  }
  __syncthreads();
  return kOk;
}

// Arguments of the persistent batched kernels.
struct BatchArgs {
  Scoring base;
  const int8_t* win_type;
  const int8_t* win_strand;
  uint32_t n_windows;
  const uint32_t* win_read_off;
  const uint8_t* seqs;
  const uint64_t* seq_off;
  const uint8_t* quals;
  const uint32_t* work;     // window ids to process (queue order)
  uint32_t n_work;
  uint32_t* queue;          // atomic cursor into work
  uint8_t* arena;
  uint64_t arena_stride;
  GraphCaps gcaps;
  DpCaps dcaps;
  int32_t* read_scores;
  uint8_t* read_rev;
  uint8_t* cons;
  const uint64_t* cons_off;
  uint32_t* cons_len;
  int32_t* win_status;
  int32_t* aln_out;         // optional
  const uint64_t* aln_off;
  uint32_t* aln_len;
  uint8_t* msa_out;         // optional
  const uint64_t* msa_off;
  uint32_t* msa_rows;
  uint32_t* msa_cols;
  unsigned long long* cells;       // sum of read length x graph nodes
  unsigned long long* pred_cells;  // sum of read length x predecessor entries
};

}  // namespace spoa_gb300
