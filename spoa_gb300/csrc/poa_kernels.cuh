// poa_kernels.cuh - kernel templates shared by the per-gap-model
// translation units (inst_linear.cu, inst_affine.cu, inst_convex.cu) and the
// host code (spoa_gb300.cu).  One CTA owns one window; the device functions
// live in poa_device.cuh and poa_dp.cuh.
#pragma once

#include <cuda_runtime.h>

#include "poa_device.cuh"
#include "poa_dp.cuh"
#include "poa_window.cuh"
#include "poa_batch_mw.cuh"

namespace spoa_gb300 {

template <int SUB, int CPT, typename T>
__global__ void __launch_bounds__(1024) k_align(Scoring S, GraphView G, DpView D,
                                                const uint8_t* seq, uint32_t L, ReadOut* out) {
  __shared__ BlockScratch sh;
  __shared__ SharedState ss;
  if (threadIdx.x == 0) read_prologue(S, G, D, L, blockDim.x * CPT, sizeof(T) == 4, ss);
  __syncthreads();
  if (ss.status != kOk || ss.mode == 0) {
    if (threadIdx.x == 0) {
      out->status = ss.status;
      out->has_score = 0;
      out->n_pairs = 0;
    }
    return;
  }
  dp_build_rows(G, D, sh);
  read_align<SUB, CPT, T>(S, G, D, sh, ss, seq, L, ss.lanes, D.aln_a, &ss.has_f, &ss.score_f,
                          &ss.np_f);
  if (threadIdx.x == 0) {
    out->status = ss.status;
    out->has_score = ss.has_f;
    out->score = ss.score_f;
    out->n_pairs = ss.np_f;
    out->lanes = ss.lanes;
  }
}

#ifdef SPOA_GB300_HOST_TU
__global__ void k_graph_reset(GraphView G) {
  if (threadIdx.x == 0 && blockIdx.x == 0) g_reset(G);
}
#endif

#ifdef SPOA_GB300_HOST_TU
__global__ void k_add(GraphView G, const int32_t* pairs, uint32_t n_pairs, const uint8_t* seq,
                      uint32_t L, const uint32_t* w, const uint8_t* qual, int32_t* status) {
  __shared__ int s_st;
  if (threadIdx.x == 0) {
    WeightSrc ws{w, qual, L, 0u, 1u};
    s_st = g_add_alignment(G, pairs, n_pairs, seq, L, ws);
  }
  __syncthreads();
  if (s_st == kOk && L > 0 && g_topo_sort_cta(G, &s_st) != 0) {
    if (threadIdx.x == 0) s_st = kCapacity;
  }
  __syncthreads();
  if (threadIdx.x == 0) *status = s_st;
}
#endif


template <int SUB, int CPT, typename T>
__global__ void __launch_bounds__(1024)
    k_align_add(Scoring S, GraphView G, DpView D, const uint8_t* seq, uint32_t L,
                const uint8_t* qual, int32_t strand, ReadOut* out, const ReadOut* prev) {
  __shared__ BlockScratch sh;
  __shared__ SharedState ss;
  __shared__ const int32_t* s_pairs;
  __shared__ int32_t s_score, s_rev;
  __shared__ uint32_t s_np;
  // in a chain of reads (one launch each, in stream order), a read after a
  // failed one is not added: it repeats the first failure's status
  if (prev) {
    if (threadIdx.x == 0) ss.pad = prev->status;
    __syncthreads();
    if (ss.pad != kOk) {
      if (threadIdx.x == 0) {
        out->status = ss.pad;
        out->score = 0;
        out->reversed = 0;
        out->n_pairs = 0;
      }
      return;
    }
  }
  window_read<SUB, CPT, T>(S, G, D, sh, ss, seq, L, qual, strand != 0, &s_score, &s_rev,
                           &s_pairs, &s_np);
  if (threadIdx.x == 0) {
    out->status = ss.status;
    out->score = s_score;
    out->reversed = s_rev;
    out->n_pairs = s_np;
  }
}


#ifdef SPOA_GB300_HOST_TU
__global__ void k_consensus(GraphView G, uint8_t* out, uint64_t cap, uint32_t* len) {
  if (threadIdx.x == 0) write_consensus(G, out, cap, len);
}
#endif


#ifdef SPOA_GB300_HOST_TU
__global__ void k_msa(GraphView G, int32_t include_consensus, uint8_t* out, uint64_t cap,
                      uint32_t* dims, int32_t* status) {
  __shared__ uint32_t s_dims[2];
  int32_t st = window_msa(G, include_consensus != 0, out, cap, &dims[0], &dims[1], s_dims);
  if (threadIdx.x == 0) *status = st;
}
#endif

struct ExportPtrs {
  uint8_t *chars, *codes;
  uint32_t *in_off, *in_edges, *out_off, *out_edges, *al_off, *al_nodes;
  uint32_t *e_tail, *e_head;
  int64_t* e_weight;
  uint32_t *lab_off, *labels, *rank, *seq_begin, *consensus;
  int32_t *coder, *decoder;
};

#ifdef SPOA_GB300_HOST_TU
__global__ void k_export(GraphView G, ExportPtrs x) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const GraphHeader* h = G.hdr;
  const uint32_t nn = h->n_nodes, ne = h->n_edges, K = G.caps.aligned;
  uint32_t io = 0, oo = 0, ao = 0;
  for (uint32_t v = 0; v < nn; ++v) {
    if (x.chars) x.chars[v] = (uint8_t)h->decoder[G.code[v]];
    if (x.codes) x.codes[v] = G.code[v];
    if (x.in_off) x.in_off[v] = io;
    for (uint32_t e = G.nlink[v].x; e != kNone; e = G.erec[e].z) {
      if (x.in_edges) x.in_edges[io] = e;
      ++io;
    }
    if (x.out_off) x.out_off[v] = oo;
    for (uint32_t e = G.nlink[v].z; e != kNone; e = G.erec[e].w) {
      if (x.out_edges) x.out_edges[oo] = e;
      ++oo;
    }
    if (x.al_off) x.al_off[v] = ao;
    for (uint32_t k = 0; k < G.n_aligned[v]; ++k) {
      if (x.al_nodes) x.al_nodes[ao] = G.aligned[(uint64_t)v * K + k];
      ++ao;
    }
    if (x.rank) x.rank[v] = G.rank_to_node[v];
  }
  if (x.in_off) x.in_off[nn] = io;
  if (x.out_off) x.out_off[nn] = oo;
  if (x.al_off) x.al_off[nn] = ao;
  uint32_t lo = 0;
  for (uint32_t e = 0; e < ne; ++e) {
    if (x.e_tail) x.e_tail[e] = G.erec[e].x;
    if (x.e_head) x.e_head[e] = G.erec[e].y;
    if (x.e_weight) x.e_weight[e] = G.e_weight[e];
    if (x.lab_off) x.lab_off[e] = lo;
    for (uint32_t l = G.e_lab_first[e]; l != kNone; l = G.lab_next[l]) {
      if (x.labels) x.labels[lo] = G.lab_seq[l];
      ++lo;
    }
  }
  if (x.lab_off) x.lab_off[ne] = lo;
  for (uint32_t s = 0; s < h->n_seqs; ++s)
    if (x.seq_begin) x.seq_begin[s] = G.seq_begin[s];
  for (uint32_t k = 0; k < h->n_consensus; ++k)
    if (x.consensus) x.consensus[k] = G.consensus[k];
  for (int k = 0; k < 256; ++k) {
    if (x.coder) x.coder[k] = h->coder[k];
    if (x.decoder) x.decoder[k] = h->decoder[k];
  }
}

// Graph::Subgraph (graph.cpp:541-595) of S into the empty graph D
// (g_subgraph_build), then the CTA sorts D.  gid (one word per node of S)
// and stack are scratch.  *status: kOk, or kCapacity when D or the stack is
// too small.
__global__ void k_subgraph(GraphView S, GraphView D, uint32_t begin, uint32_t end, uint32_t* gid,
                           uint32_t* stack, uint64_t stack_cap, uint32_t* map, int32_t* status) {
  __shared__ int s_st;
  const uint32_t nn = S.hdr->n_nodes;
  for (uint32_t v = threadIdx.x; v < nn; v += blockDim.x) gid[v] = kNone;
  __syncthreads();
  if (threadIdx.x == 0) s_st = g_subgraph_build(S, D, begin, end, gid, stack, stack_cap, map);
  __syncthreads();
  if (s_st == kOk && g_topo_sort_cta(D, &s_st) != 0) {
    if (threadIdx.x == 0) s_st = kCapacity;
  }
  __syncthreads();
  if (threadIdx.x == 0) *status = s_st;
}

// A saved graph rebuilt in G (g_import), thread 0; *status kOk or kCapacity.
__global__ void k_import(GraphView G, ImportArgs a, int32_t* status) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  *status = g_import(G, a);
}
#endif

// ---------------------------------------------------------------------------
// persistent batch kernel
// ---------------------------------------------------------------------------

// Register cap: 96 for int16 pairs gives 5 single-warp windows per SM
// sub-partition (20 per SM) and measured 6 % faster than 128 (16 per SM)
// despite more spilling in the forward pass; int32 pairs need twice the
// registers.
template <typename T>
constexpr int kBatchMaxRegs = sizeof(T) == 2 ? 96 : 128;

// MR: the register cap (the tile tuner also tries 128 for one-warp 16-bit
// tiles: fewer resident windows, no spills).
template <int SUB, int CPT, typename T, int SEGS = 1, int NT = 0, int MR = kBatchMaxRegs<T>>
__global__ void __maxnreg__(MR) k_batch(BatchArgs a) {
  __shared__ BlockScratch sh;
  __shared__ SharedState ss;
  __shared__ uint32_t s_w, s_dims[2];
  __shared__ const int32_t* s_pairs;
  __shared__ int32_t s_score, s_rev;
  __shared__ uint32_t s_np;
  // the arena views live in shared memory: each phase loads only the
  // pointers it uses instead of holding ~45 of them in registers
  __shared__ GraphView G;
  __shared__ DpView D;
  if (threadIdx.x == 0) {
    uint8_t* base = a.arena + a.arena_stride * blockIdx.x;
    const uint64_t gbytes = graph_layout(base, a.gcaps, &G);
    dp_layout(base + gbytes, a.dcaps, &D);
  }
  __syncthreads();
  Scoring S = a.base;
  while (true) {
    if (threadIdx.x == 0) {
      uint32_t k = atomicAdd(a.queue, 1u);
      s_w = k < a.n_work ? a.work[k] : kNone;
    }
    __syncthreads();
    const uint32_t w = s_w;
    if (w == kNone) break;
    if (threadIdx.x == 0) g_reset(G);
    S.type = a.win_type ? a.win_type[w] : a.base.type;
    const bool strand = a.win_strand ? a.win_strand[w] != 0 : false;
    __syncthreads();
    int32_t status = kOk;
    unsigned long long cells = 0, pred_cells = 0;
    for (uint32_t r = a.win_read_off[w]; r < a.win_read_off[w + 1]; ++r) {
      const uint64_t off = a.seq_off[r];
      const uint32_t L = (uint32_t)(a.seq_off[r + 1] - off);
      const uint32_t V0 = G.hdr->n_nodes;
      // predecessor entries of this read's DP: every in-edge, plus row 0
      // for each source node; known once the rows are built
      const uint64_t npred_before = V0 ? 1 : 0;
      cells += (unsigned long long)V0 * L * (strand ? 2u : 1u);
      window_read<SUB, CPT, T, SEGS, NT>(S, G, D, sh, ss, a.seqs + off, L,
                                         a.quals ? a.quals + off : nullptr, strand, &s_score,
                                         &s_rev, &s_pairs, &s_np);
      if (ss.status != kOk) {
        status = ss.status;
        break;
      }
      if (npred_before && ss.mode == 1)
        pred_cells += (unsigned long long)D.pred_ptr[V0 + 1] * L * (strand ? 2u : 1u);
      if (threadIdx.x == 0) {
        a.read_scores[r] = s_score;
        a.read_rev[r] = (uint8_t)s_rev;
        if (a.aln_out) {
          const uint64_t cap = a.aln_off[r + 1] - a.aln_off[r];
          const uint32_t np = (uint32_t)min((uint64_t)s_np, cap);
          for (uint32_t k = 0; k < 2 * np; ++k) a.aln_out[2 * a.aln_off[r] + k] = s_pairs[k];
          a.aln_len[r] = s_np;
        }
      }
      __syncthreads();
    }
    if (status == kOk) {
      if (threadIdx.x == 0) {
        const uint64_t cap = a.cons_off[w + 1] - a.cons_off[w];
        write_consensus(G, a.cons + a.cons_off[w], cap, &a.cons_len[w]);
        if (a.cons_len[w] > cap) s_dims[0] = kCapacity;
        else s_dims[0] = kOk;
      }
      __syncthreads();
      if (s_dims[0] != kOk) status = kCapacity;
      __syncthreads();
      if (status == kOk && a.msa_out) {
        int32_t st = window_msa(G, false, a.msa_out + a.msa_off[w], a.msa_off[w + 1] - a.msa_off[w],
                                &a.msa_rows[w], &a.msa_cols[w], s_dims);
        if (st != kOk) status = st;
      }
    }
    if (threadIdx.x == 0) {
      a.win_status[w] = status;
      if (a.cells) atomicAdd(a.cells, cells);
      if (a.pred_cells) atomicAdd(a.pred_cells, pred_cells);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// resident kernel of the served form
// ---------------------------------------------------------------------------
// Windows handed to a running kernel: the host appends one slot per window
// to a ring in host-mapped memory and then raises `tail`; every CTA of the
// resident kernel claims the next published slot (CAS on `head`, device
// memory), runs the window in its own arena (the per-read loop of
// src/main.cpp:275-314, then GenerateConsensus) and writes the consensus
// and status back into host-mapped memory, `seq` last.  A CTA that finds no
// work polls with a back-off and leaves after `idle_ns` nanoseconds without
// any (a bounded wait: the kernel never spins forever; the host launches it
// again when new work arrives and it has ended).
struct ServeSlot {
  const uint8_t* seqs;      // device: the window's reads back to back
  const uint64_t* seq_off;  // device: n_reads + 1 offsets into seqs
  uint8_t* cons;            // host-mapped: consensus output, cons_cap bytes
  uint32_t n_reads, cons_cap;
  int32_t type, strand;
};
struct ServeDone {
  int32_t status;
  uint32_t cons_len;
  unsigned long long cells;
  unsigned long long seq;  // slot index + 1 of the finished window, written last
};
struct ServeArgs {
  Scoring base;
  const ServeSlot* ring;  // host-mapped, `cap` slots
  ServeDone* done;        // host-mapped, `cap` entries
  uint32_t cap;
  const unsigned long long* tail;  // host-mapped: slots published
  unsigned long long* head;        // device: slots claimed
  uint8_t* arena;
  uint64_t arena_stride;
  GraphCaps gcaps;
  DpCaps dcaps;
  unsigned long long idle_ns;
};

__device__ __forceinline__ unsigned long long serve_clock_ns() {
  unsigned long long t = 0;
#ifdef __CUDA_ARCH__
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
#endif
  return t;
}

__device__ __forceinline__ unsigned long long load_acquire_sys(const unsigned long long* p) {
  unsigned long long v = 0;
#ifdef __CUDA_ARCH__
  asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
#endif
  return v;
}

__device__ __forceinline__ void store_release_sys(unsigned long long* p, unsigned long long v) {
#ifdef __CUDA_ARCH__
  asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
#endif
}

template <int SUB, int CPT, typename T, int NT = 0>
__global__ void __maxnreg__(kBatchMaxRegs<T>) k_serve(ServeArgs a) {
  __shared__ BlockScratch sh;
  __shared__ SharedState ss;
  __shared__ unsigned long long s_k;
  __shared__ ServeSlot slot;
  __shared__ const int32_t* s_pairs;
  __shared__ int32_t s_score, s_rev;
  __shared__ uint32_t s_np;
  __shared__ GraphView G;
  __shared__ DpView D;
  if (threadIdx.x == 0) {
    uint8_t* base = a.arena + a.arena_stride * blockIdx.x;
    const uint64_t gbytes = graph_layout(base, a.gcaps, &G);
    dp_layout(base + gbytes, a.dcaps, &D);
  }
  __syncthreads();
  Scoring S = a.base;
  while (true) {
    if (threadIdx.x == 0) {
      // claim the next published slot, waiting at most idle_ns for one
      s_k = ~0ull;
      const unsigned long long t0 = serve_clock_ns();
      unsigned int nap = 256;
      while (true) {
        const unsigned long long t = load_acquire_sys(a.tail);
        const unsigned long long h = *(volatile unsigned long long*)a.head;
        if (h < t) {
          if (atomicCAS(a.head, h, h + 1) == h) {
            s_k = h;
            break;
          }
          continue;
        }
        if (serve_clock_ns() - t0 > a.idle_ns) break;
#ifdef __CUDA_ARCH__
        __nanosleep(nap);
#endif
        if (nap < 65536) nap *= 2;
      }
      if (s_k != ~0ull) {
        const volatile ServeSlot* v = a.ring + (s_k % a.cap);
        slot.seqs = v->seqs;
        slot.seq_off = v->seq_off;
        slot.cons = v->cons;
        slot.n_reads = v->n_reads;
        slot.cons_cap = v->cons_cap;
        slot.type = v->type;
        slot.strand = v->strand;
        g_reset(G);
      }
    }
    __syncthreads();
    const unsigned long long k = s_k;
    if (k == ~0ull) break;
    S.type = slot.type;
    const bool strand = slot.strand != 0;
    int32_t status = kOk;
    unsigned long long cells = 0;
    for (uint32_t r = 0; r < slot.n_reads; ++r) {
      const uint64_t off = slot.seq_off[r];
      const uint32_t L = (uint32_t)(slot.seq_off[r + 1] - off);
      cells += (unsigned long long)G.hdr->n_nodes * L * (strand ? 2u : 1u);
      window_read<SUB, CPT, T, 1, NT>(S, G, D, sh, ss, slot.seqs + off, L, nullptr, strand,
                                      &s_score, &s_rev, &s_pairs, &s_np);
      if (ss.status != kOk) {
        status = ss.status;
        break;
      }
    }
    if (threadIdx.x == 0) {
      uint32_t len = 0;
      if (status == kOk) {
        write_consensus(G, slot.cons, slot.cons_cap, &len);
        if (len > slot.cons_cap) status = kCapacity;
      }
      ServeDone* d = a.done + (k % a.cap);
      d->status = status;
      d->cons_len = len;
      d->cells = cells;
      __threadfence_system();
      store_release_sys(&d->seq, k + 1);
    }
    __syncthreads();
  }
}

// Long windows on thread-block clusters: a cluster of CL CTAs owns one
// window at a time and spreads each row over its CTAs (window_read_cl);
// the lead CTA takes windows from the work queue and runs the serial
// phases.  The arena is per cluster.  Launched with cluster dimensions
// (CL, 1, 1) by launch_batch_cl.
template <int SUB, int CPT, typename T, int CL>
__global__ void __maxnreg__(kBatchMaxRegs<T>) k_batch_cl(BatchArgs a) {
  __shared__ BlockScratch sh;
  __shared__ SharedState ss;
  __shared__ int32_t s_w;
  __shared__ uint32_t s_dims[2];
  __shared__ const int32_t* s_pairs;
  __shared__ int32_t s_score, s_rev;
  __shared__ uint32_t s_np;
  __shared__ GraphView G;
  __shared__ DpView D;
  const bool lead = cl_rank<CL>() == 0;
  if (threadIdx.x == 0) {
    uint8_t* base = a.arena + a.arena_stride * (blockIdx.x / CL);
    const uint64_t gbytes = graph_layout(base, a.gcaps, &G);
    dp_layout(base + gbytes, a.dcaps, &D);
  }
  __syncthreads();
  Scoring S = a.base;
  while (true) {
    if (lead && threadIdx.x == 0) {
      const uint32_t k = atomicAdd(a.queue, 1u);
      s_w = (int32_t)(k < a.n_work ? a.work[k] : kNone);
    }
    cl_sync<CL>();
    const uint32_t w = (uint32_t)cl_peek(&s_w, 0);
    if (w == kNone) break;
    if (lead && threadIdx.x == 0) g_reset(G);
    S.type = a.win_type ? a.win_type[w] : a.base.type;
    const bool strand = a.win_strand ? a.win_strand[w] != 0 : false;
    cl_sync<CL>();
    int32_t status = kOk;
    unsigned long long cells = 0;
    for (uint32_t r = a.win_read_off[w]; r < a.win_read_off[w + 1]; ++r) {
      const uint64_t off = a.seq_off[r];
      const uint32_t L = (uint32_t)(a.seq_off[r + 1] - off);
      cells += (unsigned long long)G.hdr->n_nodes * L * (strand ? 2u : 1u);
      const int32_t st = window_read_cl<SUB, CPT, T, CL>(
          S, G, D, sh, ss, a.seqs + off, L, a.quals ? a.quals + off : nullptr, strand, &s_score,
          &s_rev, &s_pairs, &s_np);
      if (st != kOk) {
        status = st;
        break;
      }
      if (lead && threadIdx.x == 0) {
        a.read_scores[r] = s_score;
        a.read_rev[r] = (uint8_t)s_rev;
        if (a.aln_out) {
          const uint64_t cap = a.aln_off[r + 1] - a.aln_off[r];
          const uint32_t np = (uint32_t)min((uint64_t)s_np, cap);
          for (uint32_t k = 0; k < 2 * np; ++k) a.aln_out[2 * a.aln_off[r] + k] = s_pairs[k];
          a.aln_len[r] = s_np;
        }
      }
    }
    if (lead) {
      if (status == kOk) {
        if (threadIdx.x == 0) {
          const uint64_t cap = a.cons_off[w + 1] - a.cons_off[w];
          write_consensus(G, a.cons + a.cons_off[w], cap, &a.cons_len[w]);
          s_dims[0] = a.cons_len[w] > cap ? kCapacity : kOk;
        }
        __syncthreads();
        if (s_dims[0] != kOk) status = kCapacity;
        __syncthreads();
        if (status == kOk && a.msa_out) {
          const int32_t st = window_msa(G, false, a.msa_out + a.msa_off[w],
                                        a.msa_off[w + 1] - a.msa_off[w], &a.msa_rows[w],
                                        &a.msa_cols[w], s_dims);
          if (st != kOk) status = st;
        }
      }
      if (threadIdx.x == 0) {
        a.win_status[w] = status;
        if (a.cells) atomicAdd(a.cells, cells);
      }
    }
    cl_sync<CL>();
  }
  // no CTA leaves while another may still read its shared memory
  cl_sync<CL>();
}

// W windows per CTA (batch_cta_mw): the serial graph updates of the W
// windows run on W lanes side by side.
template <int SUB, int CPT, typename T, int W>
__global__ void __maxnreg__(kBatchMaxRegs<T>) k_batch_mw(BatchArgs a) {
  __shared__ BlockScratch sh;
  __shared__ SharedState ss;
  __shared__ MwSlot slot[W];
  __shared__ GraphView Gs[W];
  __shared__ DpView D;
  __shared__ int32_t* pairs[W];
  __shared__ uint8_t* reads[W];
  __shared__ uint32_t* pre[W];
  __shared__ MwShared m;
  if (threadIdx.x == 0)
    mw_layout(a.arena + a.arena_stride * blockIdx.x, W, a.gcaps, a.dcaps, &D, Gs, pairs, reads,
              pre);
  __syncthreads();
  batch_cta_mw<SUB, CPT, T, W>(a, sh, ss, slot, Gs, D, pairs, reads, pre, m);
}

}  // namespace spoa_gb300


namespace spoa_gb300 {

// Launch wrappers; each (gap model, width) pair is explicitly instantiated in
// its own translation unit (inst_*.cu).  Columns per thread: 8, 12, 16, 20,
// 24 or 32 for int16 pairs; 8, 12, 16, 24 or 32 for int32 pairs.
template <typename T>
__host__ __device__ constexpr bool cpt_supported(int cpt) {
  return sizeof(T) == 2 ? (cpt == 8 || cpt == 12 || cpt == 16 || cpt == 20 || cpt == 24 || cpt == 32)
                        : (cpt == 8 || cpt == 12 || cpt == 16 || cpt == 24 || cpt == 32);
}

#define SPOA_CPT_SWITCH(T, cpt, LAUNCH)                  \
  if (sizeof(T) == 2) {                                  \
    switch (cpt) {                                       \
      case 8: LAUNCH(8); break;                          \
      case 12: LAUNCH(12); break;                        \
      case 16: LAUNCH(16); break;                        \
      case 20: LAUNCH(20); break;                        \
      case 24: LAUNCH(24); break;                        \
      case 32: LAUNCH(32); break;                        \
      default: return kInvalidArgument;                  \
    }                                                    \
  } else {                                               \
    switch (cpt) {                                       \
      case 8: LAUNCH(8); break;                          \
      case 12: LAUNCH(12); break;                        \
      case 16: LAUNCH(16); break;                        \
      case 24: LAUNCH(24); break;                        \
      case 32: LAUNCH(32); break;                        \
      default: return kInvalidArgument;                  \
    }                                                    \
  }

template <int SUB, typename T>
int32_t launch_align(int cpt, int nt, const Scoring& S, const GraphView& G, const DpView& D,
                     const uint8_t* seq, uint32_t L, ReadOut* out) {
#define L_(C) k_align<SUB, C, T><<<1, nt>>>(S, G, D, seq, L, out)
  SPOA_CPT_SWITCH(T, cpt, L_)
#undef L_
  return cudaGetLastError() == cudaSuccess ? kOk : kCuda;
}

template <int SUB, typename T>
int32_t launch_align_add(int cpt, int nt, const Scoring& S, const GraphView& G,
                         const DpView& D, const uint8_t* seq, uint32_t L, const uint8_t* qual,
                         int32_t strand, ReadOut* out, const ReadOut* prev, cudaStream_t s) {
#define L_(C) k_align_add<SUB, C, T><<<1, nt, 0, s>>>(S, G, D, seq, L, qual, strand, out, prev)
  SPOA_CPT_SWITCH(T, cpt, L_)
#undef L_
  return cudaGetLastError() == cudaSuccess ? kOk : kCuda;
}

// One-warp tiles (every polishing-sized window) run the kernels built for
// exactly 32 threads (NT = 32 in dp_forward); other tiles the general ones.
template <int SUB, typename T>
int32_t launch_batch(int cpt, int nt, int grid, const BatchArgs& a, cudaStream_t s) {
#define L_(C)                                          \
  if (nt == 32)                                        \
    k_batch<SUB, C, T, 1, 32><<<grid, nt, 0, s>>>(a);  \
  else                                                 \
    k_batch<SUB, C, T><<<grid, nt, 0, s>>>(a)
  SPOA_CPT_SWITCH(T, cpt, L_)
#undef L_
  return cudaGetLastError() == cudaSuccess ? kOk : kCuda;
}

// Segmented kernels (dp_forward_seg) for rows wider than one strip per
// thread can hold in registers: 12 columns per strip, 2, 4 or 8 strips per
// thread.  Instantiated for int32 pairs only: the scores of such long rows
// pass the int16 width rule only under the smallest penalties, and those
// windows keep the single-strip int16 kernels (up to 32 x 512 columns).
constexpr int kSegCpt = 12;
template <int SUB, typename T>
int32_t launch_batch_seg(int segs, int nt, int grid, const BatchArgs& a, cudaStream_t s) {
  switch (segs) {
    case 2: k_batch<SUB, kSegCpt, T, 2><<<grid, nt, 0, s>>>(a); break;
    case 4: k_batch<SUB, kSegCpt, T, 4><<<grid, nt, 0, s>>>(a); break;
    case 8: k_batch<SUB, kSegCpt, T, 8><<<grid, nt, 0, s>>>(a); break;
    default: return kInvalidArgument;
  }
  return cudaGetLastError() == cudaSuccess ? kOk : kCuda;
}

template <int SUB, typename T>
int32_t occupancy_batch_seg(int segs, int nt, int* blocks) {
  cudaError_t err = cudaSuccess;
  switch (segs) {
    case 2: err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_batch<SUB, kSegCpt, T, 2>, nt, 0); break;
    case 4: err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_batch<SUB, kSegCpt, T, 4>, nt, 0); break;
    case 8: err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_batch<SUB, kSegCpt, T, 8>, nt, 0); break;
    default: return kInvalidArgument;
  }
  if (err != cudaSuccess) {
    cudaGetLastError();
    return kCuda;
  }
  return kOk;
}

template <int SUB, typename T>
int32_t occupancy_batch(int cpt, int nt, int* blocks) {
  cudaError_t err = cudaSuccess;
#define L_(C)                                                                                 \
  err = nt == 32 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_batch<SUB, C, T, 1, 32>, \
                                                                 nt, 0)                       \
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_batch<SUB, C, T>, nt, 0)
  SPOA_CPT_SWITCH(T, cpt, L_)
#undef L_
  if (err != cudaSuccess) {
    cudaGetLastError();
    return kCuda;
  }
  return kOk;
}

// One-warp 16-bit tiles with 128 registers per thread (a tuner candidate)
template <int SUB>
int32_t launch_batch_r128(int cpt, int grid, const BatchArgs& a, cudaStream_t s) {
  using T = int16_t;
#define L_(C) k_batch<SUB, C, T, 1, 32, 128><<<grid, 32, 0, s>>>(a)
  SPOA_CPT_SWITCH(T, cpt, L_)
#undef L_
  return cudaGetLastError() == cudaSuccess ? kOk : kCuda;
}

template <int SUB>
int32_t occupancy_batch_r128(int cpt, int* blocks) {
  using T = int16_t;
  cudaError_t err = cudaSuccess;
#define L_(C) \
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_batch<SUB, C, T, 1, 32, 128>, 32, 0)
  SPOA_CPT_SWITCH(T, cpt, L_)
#undef L_
  if (err != cudaSuccess) {
    cudaGetLastError();
    return kCuda;
  }
  return kOk;
}

// W windows per CTA (2 or 4), 16-bit lanes
template <int SUB>
int32_t launch_batch_mw(int cpt, int nt, int W, int grid, const BatchArgs& a, cudaStream_t s) {
  using T = int16_t;
#define L_(C)                                                      \
  if (W == 2)                                                      \
    k_batch_mw<SUB, C, T, 2><<<grid, nt, 0, s>>>(a);              \
  else                                                             \
    k_batch_mw<SUB, C, T, 4><<<grid, nt, 0, s>>>(a)
  SPOA_CPT_SWITCH(T, cpt, L_)
#undef L_
  return cudaGetLastError() == cudaSuccess ? kOk : kCuda;
}

template <int SUB>
int32_t occupancy_batch_mw(int cpt, int nt, int W, int* blocks) {
  using T = int16_t;
  cudaError_t err = cudaSuccess;
#define L_(C)                                                                           \
  err = W == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(                       \
                     blocks, k_batch_mw<SUB, C, T, 2>, nt, 0)                          \
               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(                       \
                     blocks, k_batch_mw<SUB, C, T, 4>, nt, 0)
  SPOA_CPT_SWITCH(T, cpt, L_)
#undef L_
  if (err != cudaSuccess) {
    cudaGetLastError();
    return kCuda;
  }
  return kOk;
}

template <int SUB, typename T>
int32_t launch_serve(int cpt, int nt, int grid, const ServeArgs& a, cudaStream_t s) {
#define L_(C)                                          \
  if (nt == 32)                                        \
    k_serve<SUB, C, T, 32><<<grid, nt, 0, s>>>(a);     \
  else                                                 \
    k_serve<SUB, C, T><<<grid, nt, 0, s>>>(a)
  SPOA_CPT_SWITCH(T, cpt, L_)
#undef L_
  return cudaGetLastError() == cudaSuccess ? kOk : kCuda;
}

template <int SUB, typename T>
int32_t occupancy_serve(int cpt, int nt, int* blocks) {
  cudaError_t err = cudaSuccess;
#define L_(C)                                                                                  \
  err = nt == 32 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_serve<SUB, C, T, 32>, nt, 0) \
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_serve<SUB, C, T>, nt, 0)
  SPOA_CPT_SWITCH(T, cpt, L_)
#undef L_
  if (err != cudaSuccess) {
    cudaGetLastError();
    return kCuda;
  }
  return kOk;
}

// Clusters of CL CTAs of nt threads (12 columns per thread, 32-bit
// lanes), `clusters` of them.
constexpr int kClCpt = 12;
template <int SUB, int CL>
int32_t launch_batch_cl_n(int nt, int clusters, const BatchArgs& a, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(clusters * CL), 1, 1);
  cfg.blockDim = dim3((unsigned)nt, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, k_batch_cl<SUB, kClCpt, int32_t, CL>, a) != cudaSuccess) {
    cudaGetLastError();
    return kCuda;
  }
  return kOk;
}

template <int SUB>
int32_t launch_batch_cl(int cl, int nt, int clusters, const BatchArgs& a, cudaStream_t s) {
  switch (cl) {
    case 2: return launch_batch_cl_n<SUB, 2>(nt, clusters, a, s);
    case 4: return launch_batch_cl_n<SUB, 4>(nt, clusters, a, s);
    case 8: return launch_batch_cl_n<SUB, 8>(nt, clusters, a, s);
    default: return kInvalidArgument;
  }
}

// Clusters of the kernel that can be resident at once.
template <int SUB, int CL>
int32_t occupancy_batch_cl_n(int nt, int* clusters) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(CL * 64), 1, 1);
  cfg.blockDim = dim3((unsigned)nt, 1, 1);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaOccupancyMaxActiveClusters(clusters, k_batch_cl<SUB, kClCpt, int32_t, CL>, &cfg) !=
      cudaSuccess) {
    cudaGetLastError();
    return kCuda;
  }
  return kOk;
}

template <int SUB>
int32_t occupancy_batch_cl(int cl, int nt, int* clusters) {
  switch (cl) {
    case 2: return occupancy_batch_cl_n<SUB, 2>(nt, clusters);
    case 4: return occupancy_batch_cl_n<SUB, 4>(nt, clusters);
    case 8: return occupancy_batch_cl_n<SUB, 8>(nt, clusters);
    default: return kInvalidArgument;
  }
}

#define SPOA_GB300_INSTANTIATE(SUB, T)                                                          \
  template int32_t launch_align<SUB, T>(int, int, const Scoring&, const GraphView&,             \
                                        const DpView&, const uint8_t*, uint32_t, ReadOut*);     \
  template int32_t launch_align_add<SUB, T>(int, int, const Scoring&, const GraphView&,         \
                                            const DpView&, const uint8_t*, uint32_t,            \
                                            const uint8_t*, int32_t, ReadOut*, const ReadOut*,  \
                                            cudaStream_t);                                      \
  template int32_t launch_batch<SUB, T>(int, int, int, const BatchArgs&, cudaStream_t);         \
  template int32_t occupancy_batch<SUB, T>(int, int, int*);                                      \
  template int32_t launch_serve<SUB, T>(int, int, int, const ServeArgs&, cudaStream_t);         \
  template int32_t occupancy_serve<SUB, T>(int, int, int*);

#define SPOA_GB300_INSTANTIATE_MW(SUB)                                                          \
  template int32_t launch_batch_mw<SUB>(int, int, int, int, const BatchArgs&, cudaStream_t);    \
  template int32_t occupancy_batch_mw<SUB>(int, int, int, int*);                                \
  template int32_t launch_batch_r128<SUB>(int, int, const BatchArgs&, cudaStream_t);            \
  template int32_t occupancy_batch_r128<SUB>(int, int*);

#define SPOA_GB300_INSTANTIATE_SEG(SUB)                                                         \
  template int32_t launch_batch_seg<SUB, int32_t>(int, int, int, const BatchArgs&, cudaStream_t); \
  template int32_t occupancy_batch_seg<SUB, int32_t>(int, int, int*);                             \
  template int32_t launch_batch_cl<SUB>(int, int, int, const BatchArgs&, cudaStream_t);           \
  template int32_t occupancy_batch_cl<SUB>(int, int, int*);

}  // namespace spoa_gb300
