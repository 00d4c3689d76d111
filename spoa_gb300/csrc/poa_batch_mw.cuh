// poa_batch_mw.cuh - the persistent batched loop with W windows per CTA.
//
// A CTA keeps W windows in flight.  Each round it aligns the next read of
// every one of them in turn (forward pass, traceback and strand choice: the
// whole CTA, one shared DP arena), keeping each chosen alignment and read in
// the window's own slot; then lane s of the first warp adds slot s's read to
// its graph and re-sorts it, so the W serial graph updates (pointer-chasing
// chains of dependent loads) run side by side instead of one after another;
// finished windows write their consensus and the slot takes the next window
// from the queue.  Results are those of the one-window loop, read by read.
#pragma once

#include <cstdint>

#include "poa_window.cuh"

namespace spoa_gb300 {

struct MwSlot {
  uint32_t w;             // window id, kNone when the slot is empty
  uint32_t r, r_end;      // next read, end of the window's reads
  int32_t status;
  int32_t type, strand;
  int32_t pending;        // an aligned read waits for its add
  int32_t score, rev;
  uint32_t np, L;
  unsigned long long cells, pred_cells;
};

// The CTA's arena: the DP arena, then per slot its graph arena, the chosen
// alignment (aln_cap pairs), the add's pre-pass results (two words per
// pair, g_add_prepass) and the chosen read (ld bytes).
__host__ __device__ inline uint64_t mw_layout(uint8_t* base, int W, const GraphCaps& gc,
                                              const DpCaps& dc, DpView* D, GraphView* Gs,
                                              int32_t** pairs, uint8_t** reads,
                                              uint32_t** pre = nullptr) {
  uint64_t off = align_up(dp_layout(base, dc, D), 256);
  for (int s = 0; s < W; ++s) {
    GraphView g;
    const uint64_t gb = align_up(graph_layout(base ? base + off : nullptr, gc, &g), 256);
    if (Gs) Gs[s] = g;
    off += gb;
    if (pairs) pairs[s] = base ? reinterpret_cast<int32_t*>(base + off) : nullptr;
    off += align_up(8 * D->aln_cap, 256);
    if (pre) pre[s] = base ? reinterpret_cast<uint32_t*>(base + off) : nullptr;
    off += align_up(8 * D->aln_cap, 256);
    if (reads) reads[s] = base ? base + off : nullptr;
    off += align_up(dc.ld, 256);
  }
  return off;
}

struct MwShared {
  uint32_t any;
  uint32_t dims[2];
};

// Every thread calls; Gs, slot_pairs, slot_reads and slot_pre have W
// entries each (shared memory), D is the CTA's DP view.
template <int SUB, int CPT, typename T, int W>
__device__ void batch_cta_mw(const BatchArgs& a, BlockScratch& sh, SharedState& ss, MwSlot* slot,
                             GraphView* Gs, DpView& D, int32_t** slot_pairs, uint8_t** slot_reads,
                             uint32_t** slot_pre, MwShared& m) {
  Scoring S = a.base;
  auto fill = [&](int s) {  // thread 0: the slot's next window
    const uint32_t k = atomicAdd(a.queue, 1u);
    MwSlot& q = slot[s];
    q.pending = 0;  // shared memory starts undefined: an empty slot must not add
    q.w = k < a.n_work ? a.work[k] : kNone;
    if (q.w == kNone) return;
    q.r = a.win_read_off[q.w];
    q.r_end = a.win_read_off[q.w + 1];
    q.status = kOk;
    q.type = a.win_type ? a.win_type[q.w] : a.base.type;
    q.strand = a.win_strand ? a.win_strand[q.w] != 0 : 0;
    q.pending = 0;
    q.cells = q.pred_cells = 0;
    g_reset(Gs[s]);
  };
  if (threadIdx.x == 0)
    for (int s = 0; s < W; ++s) fill(s);
  __syncthreads();
  while (true) {
    if (threadIdx.x == 0) {
      m.any = 0;
      for (int s = 0; s < W; ++s) m.any |= slot[s].w != kNone;
    }
    __syncthreads();
    if (!m.any) break;
    // align the next read of every active window (the whole CTA)
    for (int s = 0; s < W; ++s) {
      if (slot[s].w == kNone || slot[s].r == slot[s].r_end) continue;
      GraphView& G = Gs[s];
      const uint32_t r = slot[s].r;
      const uint64_t off = a.seq_off[r];
      const uint32_t L = (uint32_t)(a.seq_off[r + 1] - off);
      const uint8_t* seq = a.seqs + off;
      const bool strand = slot[s].strand != 0;
      S.type = slot[s].type;
      const uint32_t V0 = G.hdr->n_nodes;
      if (threadIdx.x == 0) {
        slot[s].cells += (unsigned long long)V0 * L * (strand ? 2u : 1u);
        read_prologue(S, G, D, L, blockDim.x * CPT, sizeof(T) == 4, ss);
        ss.has_f = ss.has_r = 0;
        ss.score_f = ss.score_r = 0;
        ss.np_f = ss.np_r = 0;
      }
      __syncthreads();
      if (ss.status == kOk) {
        const bool dp = ss.mode == 1;
        if (dp) {
          dp_build_rows(G, D, sh);
          read_align<SUB, CPT, T>(S, G, D, sh, ss, seq, L, ss.lanes, D.aln_a, &ss.has_f,
                                  &ss.score_f, &ss.np_f);
        }
        if (strand) {
          for (uint32_t j = threadIdx.x; j < L; j += blockDim.x)
            D.seq_rc[j] = complement_base(seq[L - 1 - j]);
          __syncthreads();
          if (dp && ss.status == kOk)
            read_align<SUB, CPT, T>(S, G, D, sh, ss, D.seq_rc, L, ss.lanes, D.aln_b, &ss.has_r,
                                    &ss.score_r, &ss.np_r);
        }
      }
      // keep the chosen alignment and read in the slot (main.cpp:276-301)
      const bool ok = ss.status == kOk;
      const int32_t sf = ss.has_f ? ss.score_f : 0;
      const int32_t sr = ss.has_r ? ss.score_r : 0;
      const bool rev = strand && !(sf >= sr);
      const int32_t* pairs = rev ? D.aln_b : D.aln_a;
      const uint32_t np = rev ? ss.np_r : ss.np_f;
      const uint8_t* chosen = rev ? D.seq_rc : seq;
      if (ok) {
        for (uint32_t k = threadIdx.x; k < 2 * np; k += blockDim.x) slot_pairs[s][k] = pairs[k];
        for (uint32_t k = threadIdx.x; k < L; k += blockDim.x) slot_reads[s][k] = chosen[k];
        if (threadIdx.x == 0 && V0 && ss.mode == 1)
          slot[s].pred_cells += (unsigned long long)D.pred_ptr[V0 + 1] * L * (strand ? 2u : 1u);
        // the add's read-only half on the whole CTA, before the graph changes
        g_add_prepass(G, pairs, np, chosen, L, slot_pre[s]);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        if (!ok) {
          slot[s].status = ss.status;
          slot[s].r = slot[s].r_end;
        } else {
          slot[s].pending = 1;
          slot[s].score = rev ? sr : sf;
          slot[s].rev = rev ? 1 : 0;
          slot[s].np = np;
          slot[s].L = L;
        }
      }
      __syncthreads();
    }
    // the graph updates side by side: lane s adds slot s's read and sorts
    if (threadIdx.x < (unsigned)W) {
      MwSlot& q = slot[threadIdx.x];
      if (q.pending) {
        q.pending = 0;
        GraphView& G = Gs[threadIdx.x];
        const uint32_t r = q.r;
        const uint8_t* qual = a.quals ? a.quals + a.seq_off[r] : nullptr;
        WeightSrc ws{nullptr, qual, q.L, q.rev ? 1u : 0u, 1u};
        int32_t st = g_add_alignment(G, slot_pairs[threadIdx.x], q.np, slot_reads[threadIdx.x],
                                     q.L, ws, slot_pre[threadIdx.x]);
        if (st == kOk && q.L > 0) {
          const uint32_t words = 3 * ((G.hdr->n_nodes + 31) / 32);
          for (uint32_t k = 0; k < words; ++k) G.sort_bits[k] = 0;
          if (g_topo_dfs(G) != 0) st = kCapacity;
        }
        if (st != kOk) {
          q.status = st;
          q.r = q.r_end;
        } else {
          a.read_scores[r] = q.score;
          a.read_rev[r] = (uint8_t)q.rev;
          if (a.aln_out) {
            const uint64_t cap = a.aln_off[r + 1] - a.aln_off[r];
            const uint32_t np = (uint32_t)min((uint64_t)q.np, cap);
            for (uint32_t k = 0; k < 2 * np; ++k)
              a.aln_out[2 * a.aln_off[r] + k] = slot_pairs[threadIdx.x][k];
            a.aln_len[r] = q.np;
          }
          ++q.r;
        }
      }
    }
    __syncthreads();
    // finished windows: consensus (lane s), MSA (CTA), status, next window
    if (threadIdx.x < (unsigned)W) {
      MwSlot& q = slot[threadIdx.x];
      if (q.w != kNone && q.r == q.r_end && q.status == kOk) {
        const uint64_t cap = a.cons_off[q.w + 1] - a.cons_off[q.w];
        write_consensus(Gs[threadIdx.x], a.cons + a.cons_off[q.w], cap, &a.cons_len[q.w]);
        if (a.cons_len[q.w] > cap) q.status = kCapacity;
      }
    }
    __syncthreads();
    if (a.msa_out) {
      for (int s = 0; s < W; ++s) {
        if (slot[s].w == kNone || slot[s].r != slot[s].r_end || slot[s].status != kOk) continue;
        const uint32_t w = slot[s].w;
        const int32_t st = window_msa(Gs[s], false, a.msa_out + a.msa_off[w],
                                      a.msa_off[w + 1] - a.msa_off[w], &a.msa_rows[w],
                                      &a.msa_cols[w], m.dims);
        if (threadIdx.x == 0 && st != kOk) slot[s].status = st;
        __syncthreads();
      }
    }
    if (threadIdx.x == 0) {
      for (int s = 0; s < W; ++s) {
        MwSlot& q = slot[s];
        if (q.w == kNone || q.r != q.r_end) continue;
        a.win_status[q.w] = q.status;
        if (a.cells) atomicAdd(a.cells, q.cells);
        if (a.pred_cells) atomicAdd(a.pred_cells, q.pred_cells);
        fill(s);
      }
    }
    __syncthreads();
  }
}

}  // namespace spoa_gb300
