// poa_dp.cuh - graph-to-sequence DP of one read against one window's graph,
// run by one CTA, and its traceback.
//
// Layout: row i (1-based rank + 1, row 0 is the initial row) x column j
// (read position).  Thread t owns the strip of CPT consecutive columns
// [t*CPT, (t+1)*CPT).  Rows are processed in rank order; the predecessor
// rows of row i are read back from the H/F/O matrices in HBM (they can be
// any earlier row).  The in-row gap recurrences are max-plus linear scans
//     X[j] = max(a[j], X[j-1] + pen)
// computed as a per-thread strip scan, a CTA-wide exclusive prefix-max of
// the strip aggregates (warp shuffles + shared memory) and a fix-up pass.
//
// Semantics follow the AVX2 SimdAlignmentEngine cell by cell
// (src/simd_alignment_engine_implementation.hpp):
//   F = max_p(max(H_p + (g-e), F_p) + e)          (1199-1203, 1226-1232)
//   O = max_p(max(H_p + (q-c), O_p) + c)          (1667-1671, 1704-1710)
//   Hd = max_p(H_p[j-1] + profile)                 (1206-1210)
//   H1 = max(Hd, F, O)                             (1734-1736)
//   Q[j] = max(H1[j-1] + q, Q[j-1] + c), Q[0] = fc + q     (1748-1756)
//   E[j] = max(H1[j-1] + g, E[j-1] + e), E[0] = fc + g     (1738-1746)
//          and, in convex mode only, at vector starts (j % lanes == 0)
//          also Q[j-1] + g: the carried lane is the previous vector's
//          final H, which includes Q (1762-1764)
//   H = max(H1, E, Q); SW stores max(H, 0) but E/Q carry the unclamped H
// In the scans the recurrences are shifted by one column (E'[k] = E[k+1])
// so that every input of a strip is owned by the strip's thread.
#pragma once

#include "poa_device.cuh"

namespace spoa_gb300 {

__device__ __forceinline__ int32_t imax(int32_t a, int32_t b) { return a > b ? a : b; }
__device__ __forceinline__ int32_t imax3(int32_t a, int32_t b, int32_t c) {
  return __vimax3_s32(a, b, c);
}
// max(a + b, c) on the DPX path
__device__ __forceinline__ int32_t addmax(int32_t a, int32_t b, int32_t c) {
  return __viaddmax_s32(a, b, c);
}

struct BlockScratch {
  int32_t wv[32];
  int32_t wv2[32];
  int32_t bcast[8];
};

// Exclusive prefix-max of v over the CTA's threads (kNegBig for thread 0).
__device__ __forceinline__ int32_t block_excl_max(int32_t v, BlockScratch& sh) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nw = blockDim.x >> 5;
  int32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x = imax(x, y);
  }
  int32_t ex = __shfl_up_sync(0xffffffffu, x, 1);
  if (lane == 0) ex = kNegBig;
  if (nw > 1) {
    if (lane == 31) sh.wv[warp] = x;
    __syncthreads();
    int32_t wp = kNegBig;
    for (uint32_t w = 0; w < warp; ++w) wp = imax(wp, sh.wv[w]);
    __syncthreads();
    ex = imax(ex, wp);
  }
  return ex;
}

__device__ __forceinline__ int32_t block_max(int32_t v, BlockScratch& sh) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = imax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (nw > 1) {
    __syncthreads();
    if (lane == 0) sh.wv2[warp] = v;
    __syncthreads();
    v = kNegBig;
    for (uint32_t w = 0; w < nw; ++w) v = imax(v, sh.wv2[w]);
    __syncthreads();
  }
  return v;
}

__device__ __forceinline__ int32_t block_min(int32_t v, BlockScratch& sh) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (nw > 1) {
    __syncthreads();
    if (lane == 0) sh.wv2[warp] = v;
    __syncthreads();
    v = 0x7fffffff;
    for (uint32_t w = 0; w < nw; ++w) v = min(v, sh.wv2[w]);
    __syncthreads();
  }
  return v;
}

// Carry X[s-1] into strip t (s = t*CPT) of the scan
//   X[j] = max(a[j], X[j-1] + pen),  X[-1] = init,
// given the strip aggregate agg = max_k a[s+k] + (CPT-1-k)*pen.
//   X[s-1] = max(init + s*pen, max_{t'<t} agg_t' + (t-1-t')*CPT*pen)
// With b_t = agg_t - t*CPT*pen this is a plain prefix-max.  Only thread 0
// knows `init`; it folds it into its own aggregate (its strip end is then
// exactly X[CPT-1]), so the other threads never need it.
template <int CPT>
__device__ __forceinline__ int32_t scan_carry(int32_t agg, int32_t init, int32_t pen,
                                              BlockScratch& sh) {
  const int32_t t = (int32_t)threadIdx.x;
  const int32_t D = CPT * pen;
  int32_t v = t == 0 ? imax(agg, init + D) : agg;
  int32_t ex = block_excl_max(v - t * D, sh);
  return t == 0 ? init : ex + (t - 1) * D;
}

// Builds the rank-ordered predecessor lists of the graph into the DP arena:
// row i = rank + 1; preds of a source row = {0}.
__device__ inline void dp_build_rows(const GraphView& G, DpView& D, BlockScratch& sh) {
  const uint32_t V = G.hdr->n_nodes;
  const uint32_t nt = blockDim.x, t = threadIdx.x;
  const uint32_t chunk = (V + nt - 1) / nt;
  const uint32_t r0 = min(V, t * chunk), r1 = min(V, r0 + chunk);
  uint32_t cnt = 0;
  for (uint32_t r = r0; r < r1; ++r) {
    uint32_t d = G.in_deg[G.rank_to_node[r]];
    cnt += d ? d : 1;
  }
  // exclusive sum of cnt over threads
  __syncthreads();
  uint32_t x = cnt;
  const uint32_t lane = t & 31, warp = t >> 5, nw = nt >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  uint32_t ex = x - cnt;
  if (lane == 31) sh.wv[warp] = (int32_t)x;
  __syncthreads();
  for (uint32_t w = 0; w < warp && w < nw; ++w) ex += (uint32_t)sh.wv[w];
  __syncthreads();
  uint32_t off = ex;
  for (uint32_t r = r0; r < r1; ++r) {
    const uint32_t node = G.rank_to_node[r];
    const uint32_t i = r + 1;
    D.pred_ptr[i] = off;
    const uint32_t d = G.in_deg[node];
    D.row_indeg[i] = d;
    D.row_char[i] = (uint8_t)G.hdr->decoder[G.code[node]];
    D.row_sink[i] = G.out_first[node] == kNone;
    if (d == 0) {
      D.preds[off++] = 0;
    } else {
      for (uint32_t e = G.in_first[node]; e != kNone; e = G.e_next_in[e])
        D.preds[off++] = G.node_to_rank[G.e_tail[e]] + 1;
    }
  }
  if (t == nt - 1) D.pred_ptr[V + 1] = off;
  __syncthreads();
}

struct AlignResult {
  int32_t status;
  int32_t has_score;  // 0: score not written (reference returns early)
  int32_t score;
  uint32_t n_pairs;
  int32_t lanes;
};

// Forward pass + row selection + max_j.  Returns (in smem-broadcast values)
// max_i, max_j and the score; traceback is run by the caller on thread 0.
template <int SUB, int CPT>
__device__ void dp_forward(const Scoring& S, DpView& D, const uint8_t* __restrict__ seq,
                           uint32_t L, uint32_t V, int32_t lanes, BlockScratch& sh,
                           int64_t* out_max_i, int64_t* out_max_j, int32_t* out_score) {
  const uint32_t t = threadIdx.x;
  const uint32_t s0 = t * CPT;
  const uint64_t ld = D.caps.ld;
  const int32_t type = S.type;
  const int32_t m = S.m, n = S.n, g = S.g, e = S.e, q = S.q, c = S.c;
  const int32_t NEGW = lanes == 8 ? (INT32_MIN + 1024) : (INT16_MIN + 1024);
  int32_t* __restrict__ H = D.H;
  int32_t* __restrict__ F = D.F;
  int32_t* __restrict__ E = D.E;
  int32_t* __restrict__ O = D.O;
  int32_t* __restrict__ Q = D.Q;

  uint8_t sc[CPT];
#pragma unroll
  for (int k = 0; k < CPT; ++k) {
    uint32_t j = s0 + k;
    sc[k] = j < L ? seq[j] : 0;
  }

  // row 0 and first column (implementation.hpp:555-694)
#pragma unroll
  for (int k = 0; k < CPT; ++k) {
    int32_t j = (int32_t)(s0 + k);
    int32_t h0;
    if (type == kSW) {
      h0 = 0;
    } else if (SUB == kConvex) {
      h0 = imax(g + j * e, q + j * c);
    } else if (SUB == kAffine) {
      h0 = g + j * e;
    } else {
      h0 = g + j * g;
    }
    H[s0 + k] = h0;
    if (SUB >= kAffine) F[s0 + k] = kNegBig;
    if (SUB == kConvex) O[s0 + k] = kNegBig;
  }
  if (t == 0) {
    D.fc[0] = 0;
    D.fcF[0] = 0;
    D.fcO[0] = 0;
  }
  // selection state (strict <: the earliest row wins a tie)
  int32_t bval = type == kSW ? 0 : (type == kOV ? kNegBig : NEGW);
  int32_t brow = -1;
  int32_t first_sink = -1;
  __syncthreads();

  for (uint32_t i = 1; i <= V; ++i) {
    const uint32_t pb = D.pred_ptr[i], pe = D.pred_ptr[i + 1];
    const uint8_t rc = D.row_char[i];
    int32_t h[CPT], f[CPT], o[CPT];
    // fc of this row (thread 0 only): NW first column
    int32_t fci = 0;
    int32_t fl = kNegBig, fa = kNegBig, fo = kNegBig;
    for (uint32_t pi = pb; pi < pe; ++pi) {
      const uint32_t p = D.preds[pi];
      const int32_t* __restrict__ Hp = H + (uint64_t)p * ld + s0;
      int32_t hleft;
      if (t == 0) {
        hleft = D.fc[p];
        fl = imax(fl, D.fc[p]);
        if (SUB >= kAffine) fa = imax(fa, D.fcF[p]);
        if (SUB == kConvex) fo = imax(fo, D.fcO[p]);
      } else {
        hleft = Hp[-1];
      }
      int32_t hp[CPT];
#pragma unroll
      for (int k = 0; k < CPT; k += 4) {
        int4 v = *reinterpret_cast<const int4*>(Hp + k);
        hp[k] = v.x; hp[k + 1] = v.y; hp[k + 2] = v.z; hp[k + 3] = v.w;
      }
#pragma unroll
      for (int k = 0; k < CPT; ++k) {
        int32_t dg = (k == 0 ? hleft : hp[k - 1]) + (sc[k] == rc ? m : n);
        int32_t cand;
        if (SUB == kLinear) {
          cand = addmax(hp[k], g, dg);
        } else {
          cand = dg;
        }
        h[k] = pi == pb ? cand : imax(h[k], cand);
      }
      if (SUB >= kAffine) {
        const int32_t* __restrict__ Fp = F + (uint64_t)p * ld + s0;
#pragma unroll
        for (int k = 0; k < CPT; k += 4) {
          int4 v = *reinterpret_cast<const int4*>(Fp + k);
          int32_t fv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            int32_t cand = addmax(hp[k + u], g - e, fv[u]) + e;
            f[k + u] = pi == pb ? cand : imax(f[k + u], cand);
          }
        }
      }
      if (SUB == kConvex) {
        const int32_t* __restrict__ Op = O + (uint64_t)p * ld + s0;
#pragma unroll
        for (int k = 0; k < CPT; k += 4) {
          int4 v = *reinterpret_cast<const int4*>(Op + k);
          int32_t ov[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            int32_t cand = addmax(hp[k + u], q - c, ov[u]) + c;
            o[k + u] = pi == pb ? cand : imax(o[k + u], cand);
          }
        }
      }
    }
    if (t == 0) {
      const bool source = D.row_indeg[i] == 0;
      if (type == kNW) {
        if (SUB == kLinear) {
          fci = (source ? 0 : fl) + g;
        } else {
          int32_t vF = (source ? g - e : fa) + e;
          D.fcF[i] = vF;
          if (SUB == kConvex) {
            int32_t vO = (source ? q - c : fo) + c;
            D.fcO[i] = vO;
            fci = imax(vF, vO);
          } else {
            fci = vF;
          }
        }
      }
      D.fc[i] = fci;
    }
    int32_t* __restrict__ Hi = H + (uint64_t)i * ld + s0;
    // H1 and the stored F/O rows
    if (SUB >= kAffine) {
      int32_t* __restrict__ Fi = F + (uint64_t)i * ld + s0;
#pragma unroll
      for (int k = 0; k < CPT; k += 4)
        *reinterpret_cast<int4*>(Fi + k) = make_int4(f[k], f[k + 1], f[k + 2], f[k + 3]);
      if (SUB == kConvex) {
        int32_t* __restrict__ Oi = O + (uint64_t)i * ld + s0;
#pragma unroll
        for (int k = 0; k < CPT; k += 4)
          *reinterpret_cast<int4*>(Oi + k) = make_int4(o[k], o[k + 1], o[k + 2], o[k + 3]);
#pragma unroll
        for (int k = 0; k < CPT; ++k) h[k] = imax3(h[k], f[k], o[k]);
      } else {
#pragma unroll
        for (int k = 0; k < CPT; ++k) h[k] = imax(h[k], f[k]);
      }
    }
    // columns past the read never feed real columns (scans run rightwards)
#pragma unroll
    for (int k = 0; k < CPT; ++k)
      if (s0 + k >= L) h[k] = kNegBig;

    int32_t hs[CPT];
    if (SUB == kLinear) {
      int32_t loc[CPT];
      loc[0] = h[0];
#pragma unroll
      for (int k = 1; k < CPT; ++k) loc[k] = addmax(loc[k - 1], g, h[k]);
      int32_t carry = scan_carry<CPT>(loc[CPT - 1], fci, g, sh);
#pragma unroll
      for (int k = 0; k < CPT; ++k) {
        int32_t hf = addmax(carry, (k + 1) * g, loc[k]);
        hs[k] = type == kSW ? imax(hf, 0) : hf;
      }
    } else {
      int32_t qq[CPT];  // Q[s0 + k]
      if (SUB == kConvex) {
        int32_t loc[CPT];
        loc[0] = h[0] + q;
#pragma unroll
        for (int k = 1; k < CPT; ++k) loc[k] = addmax(loc[k - 1], c, h[k] + q);
        int32_t carry = scan_carry<CPT>(loc[CPT - 1], fci + q, c, sh);
        qq[0] = carry;
#pragma unroll
        for (int k = 1; k < CPT; ++k) qq[k] = addmax(carry, k * c, loc[k - 1]);
        int32_t* __restrict__ Qi = Q + (uint64_t)i * ld + s0;
#pragma unroll
        for (int k = 0; k < CPT; k += 4)
          *reinterpret_cast<int4*>(Qi + k) = make_int4(qq[k], qq[k + 1], qq[k + 2], qq[k + 3]);
      }
      int32_t ee[CPT];  // E[s0 + k]
      {
        int32_t loc[CPT];
#pragma unroll
        for (int k = 0; k < CPT; ++k) {
          int32_t a = h[k] + g;
          if (SUB == kConvex && ((s0 + k + 1) % (uint32_t)lanes) == 0) a = imax(a, qq[k] + g);
          loc[k] = k == 0 ? a : addmax(loc[k - 1], e, a);
        }
        int32_t carry = scan_carry<CPT>(loc[CPT - 1], fci + g, e, sh);
        ee[0] = carry;
#pragma unroll
        for (int k = 1; k < CPT; ++k) ee[k] = addmax(carry, k * e, loc[k - 1]);
        int32_t* __restrict__ Ei = E + (uint64_t)i * ld + s0;
#pragma unroll
        for (int k = 0; k < CPT; k += 4)
          *reinterpret_cast<int4*>(Ei + k) = make_int4(ee[k], ee[k + 1], ee[k + 2], ee[k + 3]);
      }
#pragma unroll
      for (int k = 0; k < CPT; ++k) {
        int32_t hf = SUB == kConvex ? imax3(h[k], ee[k], qq[k]) : imax(h[k], ee[k]);
        hs[k] = type == kSW ? imax(hf, 0) : hf;
      }
    }
#pragma unroll
    for (int k = 0; k < CPT; k += 4)
      *reinterpret_cast<int4*>(Hi + k) = make_int4(hs[k], hs[k + 1], hs[k + 2], hs[k + 3]);

    // row selection
    if (type == kNW) {
      if (D.row_sink[i] && L - 1 >= s0 && L - 1 < s0 + CPT) {
        int32_t v = kNegBig;
#pragma unroll
        for (int k = 0; k < CPT; ++k)
          if (s0 + k == L - 1) v = hs[k];
        if (v > bval) {
          bval = v;
          brow = (int32_t)i;
        }
      }
    } else if (type == kSW || D.row_sink[i]) {
      int32_t tm = kNegBig;
#pragma unroll
      for (int k = 0; k < CPT; ++k)
        if (s0 + k < L) tm = imax(tm, hs[k]);
      if (tm > bval) {
        bval = tm;
        brow = (int32_t)i;
      }
      if (type == kOV && first_sink < 0) first_sink = (int32_t)i;
    }
    __syncthreads();
  }

  // global selection: best value, then the earliest row reaching it
  int32_t B = block_max(bval, sh);
  int32_t R = block_min(bval == B && brow >= 0 ? brow : 0x7fffffff, sh);
  int64_t max_i = -1;
  int32_t score = 0;
  if (type == kSW) {
    if (B > 0 && R != 0x7fffffff) {
      max_i = R;
      score = B;
    }
  } else if (type == kOV) {
    // _mmxxx_max_value starts from 0: a sink row never scores below 0, and
    // when no sink row is positive the first sink row wins with score 0.
    if (B > 0) {
      max_i = R;
      score = B;
    } else {
      max_i = first_sink;  // identical in every thread
      score = 0;
    }
  } else {
    if (R != 0x7fffffff && B > NEGW) {
      max_i = R;
      score = B;
    }
  }
  int64_t max_j = -1;
  if (max_i >= 0) {
    if (type == kNW) {
      max_j = (int64_t)L - 1;
    } else {
      const int32_t* Hm = H + (uint64_t)max_i * ld + s0;
      int32_t jj = 0x7fffffff;
#pragma unroll
      for (int k = 0; k < CPT; ++k)
        if (s0 + k < L && Hm[k] == score && jj == 0x7fffffff) jj = (int32_t)(s0 + k);
      jj = block_min(jj, sh);
      max_j = jj == 0x7fffffff ? -1 : jj;
    }
  }
  *out_max_i = max_i;
  *out_max_j = max_j;
  *out_score = score;
}

// Traceback from (max_i, max_j) (implementation.hpp:955-1124, 1324-1574,
// 1826-2121), thread 0.  Pairs are written to `out` in forward order.
template <int SUB>
__device__ int32_t dp_traceback(const Scoring& S, const DpView& D, const GraphView& G,
                                const uint8_t* seq, uint32_t L, uint32_t V, int64_t max_i,
                                int64_t max_j, int32_t* out, uint32_t* n_out) {
  const uint64_t ld = D.caps.ld;
  const int32_t type = S.type;
  const int32_t m = S.m, n = S.n, g = S.g, e = S.e, q = S.q, c = S.c;
  const int32_t* H = D.H;
  const int32_t* F = D.F;
  const int32_t* E = D.E;
  const int32_t* O = D.O;
  const int32_t* Q = D.Q;
  int32_t* tb = out;  // written back to front, reversed at the end
  uint64_t np = 0;
  const uint64_t cap = D.aln_cap;
  int64_t i = max_i, j = max_j, prev_i = 0, prev_j = 0;
  uint64_t guard = 0;
  const uint64_t guard_max = 4 * ((uint64_t)V + L) + 64;
#define EMIT(a, b)                      \
  do {                                  \
    if (np >= cap) return kTraceback;   \
    tb[2 * np] = (a);                   \
    tb[2 * np + 1] = (b);               \
    ++np;                               \
  } while (0)
  while (true) {
    if (++guard > guard_max) return kTraceback;
    if (j == -1 || i == 0) break;
    const uint32_t node = G.rank_to_node[i - 1];
    const int32_t h = H[(uint64_t)i * ld + j];
    if (type == kSW && h == 0) break;
    const uint32_t pb = D.pred_ptr[i], pe = D.pred_ptr[i + 1];
    const int32_t prf = D.row_char[i] == seq[j] ? m : n;
    bool found = false, ext_left = false, ext_up = false;
    for (uint32_t pi = pb; pi < pe; ++pi) {
      const uint64_t p = D.preds[pi];
      const int32_t hd = j ? H[p * ld + j - 1] : D.fc[p];
      if (h == hd + prf) {
        prev_i = (int64_t)p;
        prev_j = j - 1;
        found = true;
        break;
      }
    }
    if (!found) {
      for (uint32_t pi = pb; pi < pe; ++pi) {
        const uint64_t p = D.preds[pi];
        const int32_t hp = H[p * ld + j];
        bool take;
        if (SUB == kLinear) {
          take = h == hp + g;
        } else if (SUB == kAffine) {
          ext_up = h == F[p * ld + j] + e;
          take = ext_up || h == hp + g;
        } else {
          ext_up = h == F[p * ld + j] + e;
          if (ext_up) {
            take = true;
          } else if (h == hp + g) {
            take = true;
          } else {
            ext_up = h == O[p * ld + j] + c;
            take = ext_up || h == hp + q;
          }
        }
        if (take) {
          prev_i = (int64_t)p;
          prev_j = j;
          found = true;
          break;
        }
      }
    }
    if (!found) {
      const uint64_t row = (uint64_t)i * ld;
      const int32_t hl = j ? H[row + j - 1] : D.fc[i];
      bool take;
      if (SUB == kLinear) {
        take = h == hl + g;
      } else if (SUB == kAffine) {
        const int32_t el = j ? E[row + j - 1] : D.fc[i];
        ext_left = h == el + e;
        take = ext_left || h == hl + g;
      } else {
        const int32_t el = j ? E[row + j - 1] : D.fc[i];
        const int32_t ql = j ? Q[row + j - 1] : D.fc[i];
        ext_left = h == el + e;
        if (ext_left) {
          take = true;
        } else if (h == hl + g) {
          take = true;
        } else {
          ext_left = h == ql + c;
          take = ext_left || h == hl + q;
        }
      }
      if (take) {
        prev_i = i;
        prev_j = j - 1;
        found = true;
      }
    }
    EMIT(i == prev_i ? -1 : (int32_t)node, j == prev_j ? -1 : (int32_t)j);
    i = prev_i;
    j = prev_j;
    if (SUB >= kAffine && ext_left) {
      const uint64_t row = (uint64_t)i * ld;
      while (true) {
        if (++guard > guard_max) return kTraceback;
        EMIT(-1, (int32_t)j);
        --j;
        if (j == -1) break;
        if (E[row + j] + e != E[row + j + 1]) break;
        if (SUB == kConvex && Q[row + j] + c != Q[row + j + 1]) break;
      }
    } else if (SUB >= kAffine && ext_up) {
      while (true) {
        if (++guard > guard_max) return kTraceback;
        const uint32_t un = G.rank_to_node[i - 1];
        const uint64_t row = (uint64_t)i * ld;
        const int32_t fv = F[row + j];
        const uint32_t pb2 = D.pred_ptr[i];
        const uint32_t pe2 = D.row_indeg[i] ? D.pred_ptr[i + 1] : pb2;  // sources: none
        bool stop;
        prev_i = 0;
        if (SUB == kAffine) {
          stop = false;
          for (uint32_t pi = pb2; pi < pe2; ++pi) {
            const uint64_t p = D.preds[pi];
            stop = fv == H[p * ld + j] + g;
            if (stop || fv == F[p * ld + j] + e) {
              prev_i = (int64_t)p;
              break;
            }
          }
        } else {
          const int32_t ov = O[row + j];
          stop = true;
          for (uint32_t pi = pb2; pi < pe2; ++pi) {
            const uint64_t p = D.preds[pi];
            if (fv == F[p * ld + j] + e || ov == O[p * ld + j] + c) {
              prev_i = (int64_t)p;
              stop = false;
              break;
            }
          }
          if (stop) {
            for (uint32_t pi = pb2; pi < pe2; ++pi) {
              const uint64_t p = D.preds[pi];
              if (fv == H[p * ld + j] + g || ov == H[p * ld + j] + q) {
                prev_i = (int64_t)p;
                break;
              }
            }
          }
        }
        EMIT((int32_t)un, -1);
        i = prev_i;
        if (stop || i == 0) break;
      }
    }
  }
  if (type == kNW) {
    while (i == 0 && j != -1) {
      EMIT(-1, (int32_t)j);
      --j;
    }
    while (i != 0 && j == -1) {
      if (++guard > guard_max) return kTraceback;
      const uint32_t un = G.rank_to_node[i - 1];
      EMIT((int32_t)un, -1);
      if (D.row_indeg[i] == 0) {
        i = 0;
      } else {
        for (uint32_t pi = D.pred_ptr[i]; pi < D.pred_ptr[i + 1]; ++pi) {
          const uint64_t p = D.preds[pi];
          bool hit;
          if (SUB == kLinear) {
            hit = D.fc[i] == D.fc[p] + g;
          } else if (SUB == kAffine) {
            hit = D.fcF[i] == D.fcF[p] + e;
          } else {
            hit = D.fcF[i] == D.fcF[p] + e || D.fcO[i] == D.fcO[p] + c;
          }
          if (hit) {
            i = (int64_t)p;
            break;
          }
        }
      }
    }
  }
#undef EMIT
  for (uint64_t a = 0, b = np ? np - 1 : 0; a < b; ++a, --b) {
    int32_t x0 = tb[2 * a], x1 = tb[2 * a + 1];
    tb[2 * a] = tb[2 * b];
    tb[2 * a + 1] = tb[2 * b + 1];
    tb[2 * b] = x0;
    tb[2 * b + 1] = x1;
  }
  *n_out = (uint32_t)np;
  return kOk;
}

}  // namespace spoa_gb300
