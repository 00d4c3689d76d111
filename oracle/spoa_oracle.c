/*
 * spoa_oracle.c - CPU restatement of spoa's partial-order-alignment path.
 *
 * TEST INFRASTRUCTURE ONLY (parity oracle and CPU baseline).  The product
 * library never links or calls this file.
 *
 * What it restates, cell by cell, is the AVX2 build of the reference:
 *   - AlignmentEngine::Create / WorstCaseAlignmentScore
 *       (src/alignment_engine.cpp:32-73, 101-110)
 *   - SimdAlignmentEngine::Align width rule and Initialize
 *       (src/simd_alignment_engine_implementation.hpp:703-780, 518-701)
 *   - Linear / Affine / Convex forward passes and tracebacks
 *       (same file 782-1134, 1136-1584, 1586-2131)
 *   - Graph::AddAlignment, AddSequence, AddEdge, TopologicalSort,
 *     TraverseHeaviestBundle, BranchCompletion, MSA (src/graph.cpp)
 *
 * The SIMD code works on vectors of `lanes` scores (16 int16 or 8 int32 on
 * AVX2).  Scores are exact integers in both widths (the width rule keeps
 * every reachable value inside the type), so the restatement computes in
 * int32.  Two lane effects are observable and are reproduced:
 *   (1) in convex mode the horizontal E recurrence sees the Q matrix only at
 *       vector starts (j % lanes == 0), through the carried H of the
 *       previous vector (implementation.hpp:1738-1768);
 *   (2) -infinity is INT16_MIN+1024 or INT32_MIN+1024 depending on width.
 * Padding lanes beyond the sequence never exceed the row's last real cell
 * (padding score <= every gap-open penalty), so they change neither row
 * maxima nor first-index searches and are not materialised.
 */
#define _POSIX_C_SOURCE 199309L  /* clock_gettime */
#include "spoa_oracle.h"

#include <limits.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ------------------------------------------------------------------ */
/* small growable vector                                               */
/* ------------------------------------------------------------------ */
typedef struct {
  uint32_t* a;
  uint32_t n, cap;
} vec_u32;

static int vu_push(vec_u32* v, uint32_t x) {
  if (v->n == v->cap) {
    uint32_t nc = v->cap ? v->cap * 2 : 4;
    uint32_t* na = (uint32_t*)realloc(v->a, (size_t)nc * sizeof(uint32_t));
    if (!na) return -1;
    v->a = na;
    v->cap = nc;
  }
  v->a[v->n++] = x;
  return 0;
}
static void vu_free(vec_u32* v) {
  free(v->a);
  v->a = NULL;
  v->n = v->cap = 0;
}

/* ------------------------------------------------------------------ */
/* graph (include/spoa/graph.hpp:40-100, 305-318)                      */
/* ------------------------------------------------------------------ */
typedef struct {
  uint32_t code;
  vec_u32 in;      /* edge ids, insertion order */
  vec_u32 out;     /* edge ids, insertion order */
  vec_u32 aligned; /* node ids, insertion order */
} onode;

typedef struct {
  uint32_t tail, head;
  vec_u32 labels;
  int64_t weight;
} oedge;

struct oracle_graph {
  uint32_t num_codes;
  int32_t coder[256];
  int32_t decoder[256];
  onode* nodes;
  uint32_t n_nodes, cap_nodes;
  oedge* edges;
  uint32_t n_edges, cap_edges;
  vec_u32 sequences;
  vec_u32 rank_to_node;
  vec_u32 consensus;
};

struct oracle_engine {
  int32_t type;    /* 0 SW, 1 NW, 2 OV */
  int32_t subtype; /* 0 linear, 1 affine, 2 convex */
  int32_t m, n, g, e, q, c;
};

#define T_SW 0
#define T_NW 1
#define T_OV 2
#define S_LIN 0
#define S_AFF 1
#define S_CVX 2

oracle_graph* oracle_graph_create(void) {
  oracle_graph* g = (oracle_graph*)calloc(1, sizeof(oracle_graph));
  if (!g) return NULL;
  for (int i = 0; i < 256; ++i) g->coder[i] = g->decoder[i] = -1;
  return g;
}

void oracle_graph_clear(oracle_graph* g) {
  for (uint32_t i = 0; i < g->n_nodes; ++i) {
    vu_free(&g->nodes[i].in);
    vu_free(&g->nodes[i].out);
    vu_free(&g->nodes[i].aligned);
  }
  for (uint32_t i = 0; i < g->n_edges; ++i) vu_free(&g->edges[i].labels);
  g->n_nodes = 0;
  g->n_edges = 0;
  g->num_codes = 0;
  for (int i = 0; i < 256; ++i) g->coder[i] = g->decoder[i] = -1;
  g->sequences.n = 0;
  g->rank_to_node.n = 0;
  g->consensus.n = 0;
}

void oracle_graph_destroy(oracle_graph* g) {
  if (!g) return;
  oracle_graph_clear(g);
  free(g->nodes);
  free(g->edges);
  vu_free(&g->sequences);
  vu_free(&g->rank_to_node);
  vu_free(&g->consensus);
  free(g);
}

/* Graph::AddNode (graph.cpp:76-79) */
static int64_t add_node(oracle_graph* g, uint32_t code) {
  if (g->n_nodes == g->cap_nodes) {
    uint32_t nc = g->cap_nodes ? g->cap_nodes * 2 : 64;
    onode* nn = (onode*)realloc(g->nodes, (size_t)nc * sizeof(onode));
    if (!nn) return -1;
    g->nodes = nn;
    g->cap_nodes = nc;
  }
  onode* nd = &g->nodes[g->n_nodes];
  memset(nd, 0, sizeof(*nd));
  nd->code = code;
  return g->n_nodes++;
}

/* Graph::AddEdge (graph.cpp:81-91): an existing tail->head edge gains the
 * label and the weight, otherwise a new edge is appended to both lists. */
static int add_edge(oracle_graph* g, uint32_t tail, uint32_t head,
                    uint32_t weight) {
  onode* t = &g->nodes[tail];
  for (uint32_t k = 0; k < t->out.n; ++k) {
    oedge* ed = &g->edges[t->out.a[k]];
    if (ed->head == head) {
      if (vu_push(&ed->labels, g->sequences.n)) return -1;
      ed->weight += weight;
      return 0;
    }
  }
  if (g->n_edges == g->cap_edges) {
    uint32_t nc = g->cap_edges ? g->cap_edges * 2 : 64;
    oedge* ne = (oedge*)realloc(g->edges, (size_t)nc * sizeof(oedge));
    if (!ne) return -1;
    g->edges = ne;
    g->cap_edges = nc;
  }
  uint32_t id = g->n_edges++;
  oedge* ed = &g->edges[id];
  memset(ed, 0, sizeof(*ed));
  ed->tail = tail;
  ed->head = head;
  ed->weight = weight;
  if (vu_push(&ed->labels, g->sequences.n)) return -1;
  if (vu_push(&g->nodes[tail].out, id)) return -1;
  if (vu_push(&g->nodes[head].in, id)) return -1;
  return 0;
}

/* Graph::AddSequence (graph.cpp:93-110).  Returns the first node or -1
 * (nullptr) for an empty range; -2 on allocation failure. */
static int64_t add_sequence(oracle_graph* g, const char* seq,
                            const uint32_t* w, uint32_t begin, uint32_t end) {
  if (begin == end) return -1;
  int64_t prev = -1;
  for (uint32_t i = begin; i < end; ++i) {
    int64_t curr = add_node(g, (uint32_t)g->coder[(uint8_t)seq[i]]);
    if (curr < 0) return -2;
    if (prev >= 0) {
      if (add_edge(g, (uint32_t)prev, (uint32_t)curr, w[i - 1] + w[i]))
        return -2;
    }
    prev = curr;
  }
  return (int64_t)g->n_nodes - (end - begin);
}

/* Graph::TopologicalSort (graph.cpp:249-303): iterative DFS over node ids;
 * in-edge tails and (for non-ignored nodes) aligned nodes are pushed in
 * list order; an aligned group is emitted contiguously after its first
 * finished member. */
static int topological_sort(oracle_graph* g) {
  uint32_t nn = g->n_nodes;
  g->rank_to_node.n = 0;
  uint8_t* marks = (uint8_t*)calloc(nn ? nn : 1, 1);
  uint8_t* ignored = (uint8_t*)calloc(nn ? nn : 1, 1);
  vec_u32 stack = {0};
  if (!marks || !ignored) {
    free(marks);
    free(ignored);
    return -1;
  }
  int rc = 0;
  for (uint32_t s = 0; s < nn && rc == 0; ++s) {
    if (marks[s] != 0) continue;
    if (vu_push(&stack, s)) { rc = -1; break; }
    while (stack.n) {
      uint32_t curr = stack.a[stack.n - 1];
      int is_valid = 1;
      if (marks[curr] != 2) {
        onode* nd = &g->nodes[curr];
        for (uint32_t k = 0; k < nd->in.n; ++k) {
          uint32_t t = g->edges[nd->in.a[k]].tail;
          if (marks[t] != 2) {
            if (vu_push(&stack, t)) { rc = -1; break; }
            is_valid = 0;
          }
        }
        if (rc) break;
        if (!ignored[curr]) {
          for (uint32_t k = 0; k < nd->aligned.n; ++k) {
            uint32_t a = nd->aligned.a[k];
            if (marks[a] != 2) {
              if (vu_push(&stack, a)) { rc = -1; break; }
              ignored[a] = 1;
              is_valid = 0;
            }
          }
          if (rc) break;
        }
        if (is_valid) {
          marks[curr] = 2;
          if (!ignored[curr]) {
            if (vu_push(&g->rank_to_node, curr)) { rc = -1; break; }
            for (uint32_t k = 0; k < nd->aligned.n; ++k)
              if (vu_push(&g->rank_to_node, nd->aligned.a[k])) { rc = -1; break; }
            if (rc) break;
          }
        } else {
          marks[curr] = 1;
        }
      }
      if (is_valid) stack.n--;
    }
  }
  vu_free(&stack);
  free(marks);
  free(ignored);
  return rc;
}

/* Graph::AddAlignment (graph.cpp:155-247). */
int32_t oracle_add_alignment(oracle_graph* g, const int32_t* pairs,
                             uint32_t n_pairs, const char* seq, uint32_t len,
                             const uint32_t* w, uint32_t n_weights) {
  if (len == 0) return ORACLE_OK;
  if (len != n_weights) return ORACLE_ERR_UNEQUAL_WEIGHTS;
  for (uint32_t i = 0; i < len; ++i) {
    uint8_t ch = (uint8_t)seq[i];
    if (g->coder[ch] == -1) {
      g->coder[ch] = (int32_t)g->num_codes;
      g->decoder[g->num_codes++] = ch;
    }
  }
  if (n_pairs == 0) {
    int64_t b = add_sequence(g, seq, w, 0, len);
    if (b < -1) return ORACLE_ERR_NO_MEMORY;
    if (vu_push(&g->sequences, (uint32_t)b)) return ORACLE_ERR_NO_MEMORY;
    return topological_sort(g) ? ORACLE_ERR_NO_MEMORY : ORACLE_OK;
  }
  int32_t first_valid = -1, last_valid = -1;
  for (uint32_t k = 0; k < n_pairs; ++k) {
    int32_t pos = pairs[2 * k + 1];
    if (pos != -1) {
      if (pos < 0 || pos >= (int32_t)len) return ORACLE_ERR_INVALID_ALIGNMENT;
      if (first_valid == -1) first_valid = pos;
      last_valid = pos;
    }
  }
  if (first_valid == -1) return ORACLE_ERR_MISSING_SEQUENCE;

  int64_t begin = add_sequence(g, seq, w, 0, (uint32_t)first_valid);
  if (begin < -1) return ORACLE_ERR_NO_MEMORY;
  int64_t prev = begin >= 0 ? (int64_t)g->n_nodes - 1 : -1;
  int64_t last = add_sequence(g, seq, w, (uint32_t)last_valid + 1, len);
  if (last < -1) return ORACLE_ERR_NO_MEMORY;

  for (uint32_t k = 0; k < n_pairs; ++k) {
    int32_t nid = pairs[2 * k], pos = pairs[2 * k + 1];
    if (pos == -1) continue;
    uint32_t code = (uint32_t)g->coder[(uint8_t)seq[pos]];
    int64_t curr = -1;
    if (nid == -1) {
      curr = add_node(g, code);
      if (curr < 0) return ORACLE_ERR_NO_MEMORY;
    } else {
      onode* jt = &g->nodes[nid];
      if (jt->code == code) {
        curr = nid;
      } else {
        for (uint32_t a = 0; a < jt->aligned.n; ++a) {
          if (g->nodes[jt->aligned.a[a]].code == code) {
            curr = jt->aligned.a[a];
            break;
          }
        }
        if (curr < 0) {
          curr = add_node(g, code);
          if (curr < 0) return ORACLE_ERR_NO_MEMORY;
          jt = &g->nodes[nid]; /* realloc may have moved nodes */
          for (uint32_t a = 0; a < jt->aligned.n; ++a) {
            uint32_t kt = jt->aligned.a[a];
            if (vu_push(&g->nodes[kt].aligned, (uint32_t)curr) ||
                vu_push(&g->nodes[curr].aligned, kt))
              return ORACLE_ERR_NO_MEMORY;
          }
          if (vu_push(&jt->aligned, (uint32_t)curr) ||
              vu_push(&g->nodes[curr].aligned, (uint32_t)nid))
            return ORACLE_ERR_NO_MEMORY;
        }
      }
    }
    if (begin < 0) begin = curr;
    if (prev >= 0) {
      if (add_edge(g, (uint32_t)prev, (uint32_t)curr, w[pos - 1] + w[pos]))
        return ORACLE_ERR_NO_MEMORY;
    }
    prev = curr;
  }
  if (last >= 0) {
    if (add_edge(g, (uint32_t)prev, (uint32_t)last,
                 w[last_valid] + w[last_valid + 1]))
      return ORACLE_ERR_NO_MEMORY;
  }
  if (vu_push(&g->sequences, (uint32_t)begin)) return ORACLE_ERR_NO_MEMORY;
  return topological_sort(g) ? ORACLE_ERR_NO_MEMORY : ORACLE_OK;
}

/* ------------------------------------------------------------------ */
/* consensus (graph.cpp:433-516)                                       */
/* ------------------------------------------------------------------ */
static int64_t branch_completion(oracle_graph* g, uint32_t rank,
                                 int64_t* scores, int64_t* preds) {
  uint32_t start = g->rank_to_node.a[rank];
  onode* sn = &g->nodes[start];
  for (uint32_t k = 0; k < sn->out.n; ++k) {
    onode* hn = &g->nodes[g->edges[sn->out.a[k]].head];
    for (uint32_t l = 0; l < hn->in.n; ++l) {
      uint32_t t = g->edges[hn->in.a[l]].tail;
      if (t != start) scores[t] = -1;
    }
  }
  int64_t max = -1;
  for (uint32_t r = rank + 1; r < g->rank_to_node.n; ++r) {
    uint32_t it = g->rank_to_node.a[r];
    scores[it] = -1;
    preds[it] = -1;
    onode* nd = &g->nodes[it];
    for (uint32_t l = 0; l < nd->in.n; ++l) {
      oedge* ed = &g->edges[nd->in.a[l]];
      if (scores[ed->tail] == -1) continue;
      if (scores[it] < ed->weight ||
          (scores[it] == ed->weight && scores[preds[it]] <= scores[ed->tail])) {
        scores[it] = ed->weight;
        preds[it] = ed->tail;
      }
    }
    if (preds[it] != -1) scores[it] += scores[preds[it]];
    if (max == -1 || scores[max] < scores[it]) max = it;
  }
  return max;
}

static int traverse_heaviest_bundle(oracle_graph* g) {
  if (g->rank_to_node.n == 0) return 0;
  uint32_t nn = g->n_nodes;
  int64_t* scores = (int64_t*)malloc((size_t)nn * sizeof(int64_t));
  int64_t* preds = (int64_t*)malloc((size_t)nn * sizeof(int64_t));
  uint32_t* n2r = (uint32_t*)calloc(nn, sizeof(uint32_t));
  if (!scores || !preds || !n2r) {
    free(scores); free(preds); free(n2r);
    return -1;
  }
  for (uint32_t i = 0; i < nn; ++i) {
    scores[i] = -1;
    preds[i] = -1;
  }
  int64_t max = -1;
  for (uint32_t r = 0; r < g->rank_to_node.n; ++r) {
    uint32_t it = g->rank_to_node.a[r];
    onode* nd = &g->nodes[it];
    for (uint32_t l = 0; l < nd->in.n; ++l) {
      oedge* ed = &g->edges[nd->in.a[l]];
      if (scores[it] < ed->weight ||
          (scores[it] == ed->weight && scores[preds[it]] <= scores[ed->tail])) {
        scores[it] = ed->weight;
        preds[it] = ed->tail;
      }
    }
    if (preds[it] != -1) scores[it] += scores[preds[it]];
    if (max == -1 || scores[max] < scores[it]) max = it;
  }
  if (g->nodes[max].out.n) {
    for (uint32_t r = 0; r < g->rank_to_node.n; ++r) n2r[g->rank_to_node.a[r]] = r;
    while (g->nodes[max].out.n)
      max = branch_completion(g, n2r[max], scores, preds);
  }
  g->consensus.n = 0;
  while (preds[max] != -1) {
    if (vu_push(&g->consensus, (uint32_t)max)) goto oom;
    max = preds[max];
  }
  if (vu_push(&g->consensus, (uint32_t)max)) goto oom;
  for (uint32_t a = 0, b = g->consensus.n - 1; a < b; ++a, --b) {
    uint32_t t = g->consensus.a[a];
    g->consensus.a[a] = g->consensus.a[b];
    g->consensus.a[b] = t;
  }
  free(scores); free(preds); free(n2r);
  return 0;
oom:
  free(scores); free(preds); free(n2r);
  return -1;
}

uint32_t oracle_consensus(oracle_graph* g, char* out, uint32_t cap) {
  if (traverse_heaviest_bundle(g)) return 0;
  uint32_t n = g->consensus.n;
  for (uint32_t i = 0; i < n && i < cap; ++i)
    out[i] = (char)g->decoder[g->nodes[g->consensus.a[i]].code];
  return n;
}

/* Node::Successor (graph.cpp:22-30) */
static int64_t successor(const oracle_graph* g, uint32_t node, uint32_t label) {
  const onode* nd = &g->nodes[node];
  for (uint32_t k = 0; k < nd->out.n; ++k) {
    const oedge* ed = &g->edges[nd->out.a[k]];
    for (uint32_t l = 0; l < ed->labels.n; ++l)
      if (ed->labels.a[l] == label) return ed->head;
  }
  return -1;
}

/* InitializeMultipleSequenceAlignment + GenerateMultipleSequenceAlignment
 * (graph.cpp:321-366). */
int32_t oracle_msa(oracle_graph* g, int32_t include_consensus, char* out,
                   uint64_t cap, uint32_t* n_rows, uint32_t* row_len) {
  uint32_t nn = g->n_nodes;
  uint32_t* col = (uint32_t*)calloc(nn ? nn : 1, sizeof(uint32_t));
  if (!col) return ORACLE_ERR_NO_MEMORY;
  uint32_t j = 0;
  for (uint32_t i = 0; i < g->rank_to_node.n; ++i, ++j) {
    uint32_t it = g->rank_to_node.a[i];
    col[it] = j;
    onode* nd = &g->nodes[it];
    for (uint32_t k = 0; k < nd->aligned.n; ++k) {
      col[nd->aligned.a[k]] = j;
      ++i;
    }
  }
  uint32_t rows = g->sequences.n + (include_consensus ? 1 : 0);
  *n_rows = rows;
  *row_len = j;
  if ((uint64_t)rows * j > cap) {
    free(col);
    return ORACLE_ERR_CAPACITY;
  }
  for (uint32_t s = 0; s < g->sequences.n; ++s) {
    char* row = out + (uint64_t)s * j;
    memset(row, '-', j);
    int64_t it = g->sequences.a[s];
    while (it >= 0) {
      row[col[it]] = (char)g->decoder[g->nodes[it].code];
      it = successor(g, (uint32_t)it, s);
    }
  }
  if (include_consensus) {
    if (traverse_heaviest_bundle(g)) {
      free(col);
      return ORACLE_ERR_NO_MEMORY;
    }
    char* row = out + (uint64_t)g->sequences.n * j;
    memset(row, '-', j);
    for (uint32_t k = 0; k < g->consensus.n; ++k) {
      uint32_t it = g->consensus.a[k];
      row[col[it]] = (char)g->decoder[g->nodes[it].code];
    }
  }
  free(col);
  return ORACLE_OK;
}

uint32_t oracle_graph_num_nodes(const oracle_graph* g) { return g->n_nodes; }
uint32_t oracle_graph_num_edges(const oracle_graph* g) { return g->n_edges; }
uint32_t oracle_graph_num_sequences(const oracle_graph* g) {
  return g->sequences.n;
}
uint32_t oracle_graph_consensus_len(const oracle_graph* g) {
  return g->consensus.n;
}

void oracle_graph_export(const oracle_graph* g, uint8_t* chars,
                         uint32_t* rank_to_node, uint32_t* edge_tail,
                         uint32_t* edge_head, int64_t* edge_weight,
                         uint32_t* seq_begin, uint32_t* consensus) {
  uint32_t e = 0;
  for (uint32_t i = 0; i < g->n_nodes; ++i) {
    const onode* nd = &g->nodes[i];
    if (chars) chars[i] = (uint8_t)g->decoder[nd->code];
    for (uint32_t k = 0; k < nd->out.n; ++k, ++e) {
      const oedge* ed = &g->edges[nd->out.a[k]];
      if (edge_tail) edge_tail[e] = ed->tail;
      if (edge_head) edge_head[e] = ed->head;
      if (edge_weight) edge_weight[e] = ed->weight;
    }
  }
  /* memcpy wants valid pointers even for 0 bytes: empty lists copy nothing */
  if (rank_to_node && g->rank_to_node.n)
    memcpy(rank_to_node, g->rank_to_node.a,
           (size_t)g->rank_to_node.n * sizeof(uint32_t));
  if (seq_begin && g->sequences.n)
    memcpy(seq_begin, g->sequences.a, (size_t)g->sequences.n * sizeof(uint32_t));
  if (consensus && g->consensus.n)
    memcpy(consensus, g->consensus.a, (size_t)g->consensus.n * sizeof(uint32_t));
}

/* Edges in id order (Graph::edges()) and the aligned-node lists as CSR
 * (aligned_off has n_nodes + 1 entries); any pointer may be NULL.
 * Returns the total length of the aligned lists. */
uint32_t oracle_graph_export_ids(const oracle_graph* g, uint32_t* edge_tail,
                                 uint32_t* edge_head, int64_t* edge_weight,
                                 uint32_t* aligned_off, uint32_t* aligned) {
  for (uint32_t e = 0; e < g->n_edges; ++e) {
    if (edge_tail) edge_tail[e] = g->edges[e].tail;
    if (edge_head) edge_head[e] = g->edges[e].head;
    if (edge_weight) edge_weight[e] = g->edges[e].weight;
  }
  uint32_t n = 0;
  for (uint32_t v = 0; v < g->n_nodes; ++v) {
    if (aligned_off) aligned_off[v] = n;
    for (uint32_t k = 0; k < g->nodes[v].aligned.n; ++k, ++n)
      if (aligned) aligned[n] = g->nodes[v].aligned.a[k];
  }
  if (aligned_off) aligned_off[g->n_nodes] = n;
  return n;
}

/* Labels of every edge in id order as CSR (label_off: n_edges + 1
 * entries); NULL skips an array.  Returns the total number of labels. */
uint32_t oracle_graph_edge_labels(const oracle_graph* g, uint32_t* label_off,
                                  uint32_t* labels) {
  uint32_t n = 0;
  for (uint32_t e = 0; e < g->n_edges; ++e) {
    if (label_off) label_off[e] = n;
    for (uint32_t k = 0; k < g->edges[e].labels.n; ++k, ++n)
      if (labels) labels[n] = g->edges[e].labels.a[k];
  }
  if (label_off) label_off[g->n_edges] = n;
  return n;
}

/* Graph::save followed by Graph::load (include/spoa/graph.hpp:187-276):
 * `out` becomes what the reference's load rebuilds from what its save
 * archives of g.  Nodes (id, code), edges (labels, weight) and the coder
 * tables are copied; each edge, in id order, is appended to its tail's
 * out-edges and its head's in-edges; the aligned pairs (a, b), a < b, taken
 * in node order and then list order, are appended to both lists in that
 * order; sequence starts, rank order and consensus are copied. */
int32_t oracle_graph_reload(const oracle_graph* g, oracle_graph* out) {
  if (out == g) return ORACLE_ERR_INVALID_ARGUMENT;
  oracle_graph_clear(out);
  out->num_codes = g->num_codes;
  memcpy(out->coder, g->coder, sizeof(g->coder));
  memcpy(out->decoder, g->decoder, sizeof(g->decoder));
  for (uint32_t v = 0; v < g->n_nodes; ++v)
    if (add_node(out, g->nodes[v].code) < 0) return ORACLE_ERR_NO_MEMORY;
  for (uint32_t e = 0; e < g->n_edges; ++e) {
    if (out->n_edges == out->cap_edges) {
      uint32_t nc = out->cap_edges ? out->cap_edges * 2 : 64;
      oedge* ne = (oedge*)realloc(out->edges, (size_t)nc * sizeof(oedge));
      if (!ne) return ORACLE_ERR_NO_MEMORY;
      out->edges = ne;
      out->cap_edges = nc;
    }
    const oedge* src = &g->edges[e];
    oedge* ed = &out->edges[out->n_edges++];
    memset(ed, 0, sizeof(*ed));
    ed->tail = src->tail;
    ed->head = src->head;
    ed->weight = src->weight;
    for (uint32_t k = 0; k < src->labels.n; ++k)
      if (vu_push(&ed->labels, src->labels.a[k])) return ORACLE_ERR_NO_MEMORY;
    if (vu_push(&out->nodes[src->tail].out, e) || vu_push(&out->nodes[src->head].in, e))
      return ORACLE_ERR_NO_MEMORY;
  }
  for (uint32_t v = 0; v < g->n_nodes; ++v) {
    const onode* nd = &g->nodes[v];
    for (uint32_t k = 0; k < nd->aligned.n; ++k) {
      const uint32_t b = nd->aligned.a[k];
      if (v < b && (vu_push(&out->nodes[v].aligned, b) || vu_push(&out->nodes[b].aligned, v)))
        return ORACLE_ERR_NO_MEMORY;
    }
  }
  for (uint32_t k = 0; k < g->sequences.n; ++k)
    if (vu_push(&out->sequences, g->sequences.a[k])) return ORACLE_ERR_NO_MEMORY;
  for (uint32_t k = 0; k < g->rank_to_node.n; ++k)
    if (vu_push(&out->rank_to_node, g->rank_to_node.a[k])) return ORACLE_ERR_NO_MEMORY;
  for (uint32_t k = 0; k < g->consensus.n; ++k)
    if (vu_push(&out->consensus, g->consensus.a[k])) return ORACLE_ERR_NO_MEMORY;
  return ORACLE_OK;
}

/* Graph::Subgraph (graph.cpp:518-595).  ExtractSubgraph's depth-first
 * walk from `end` over in-edge tails and aligned nodes, a node entering the
 * set when its id is at least `begin`; the set's nodes are added to `out`
 * in id order, then per node its in-edges from inside the set
 * (AddEdge with the 32-bit weight, label = number of sequences = 0) and its
 * aligned nodes inside the set, in list order; then TopologicalSort.
 * sub_to_graph gets n_nodes(g) entries: graph id per subgraph node, then
 * UINT32_MAX. */
int32_t oracle_subgraph(const oracle_graph* g, uint32_t begin, uint32_t end,
                        oracle_graph* out, uint32_t* sub_to_graph) {
  const uint32_t nn = g->n_nodes;
  if (begin >= nn || end >= nn || out == g) return ORACLE_ERR_INVALID_ARGUMENT;
  oracle_graph_clear(out);
  out->num_codes = g->num_codes;
  memcpy(out->coder, g->coder, sizeof(g->coder));
  memcpy(out->decoder, g->decoder, sizeof(g->decoder));
  uint8_t* in_set = (uint8_t*)calloc(nn, 1);
  uint32_t* to_sub = (uint32_t*)malloc((size_t)nn * sizeof(uint32_t));
  vec_u32 stack = {0};
  int32_t rc = ORACLE_OK;
  if (!in_set || !to_sub || vu_push(&stack, end)) rc = ORACLE_ERR_NO_MEMORY;
  while (rc == ORACLE_OK && stack.n) {
    uint32_t curr = stack.a[--stack.n];
    if (in_set[curr] || curr < begin) continue;
    const onode* nd = &g->nodes[curr];
    for (uint32_t k = 0; k < nd->in.n && rc == ORACLE_OK; ++k)
      if (vu_push(&stack, g->edges[nd->in.a[k]].tail)) rc = ORACLE_ERR_NO_MEMORY;
    for (uint32_t k = 0; k < nd->aligned.n && rc == ORACLE_OK; ++k)
      if (vu_push(&stack, nd->aligned.a[k])) rc = ORACLE_ERR_NO_MEMORY;
    in_set[curr] = 1;
  }
  for (uint32_t v = 0; v < nn && rc == ORACLE_OK; ++v) {
    to_sub[v] = UINT32_MAX;
    sub_to_graph[v] = UINT32_MAX;
  }
  for (uint32_t v = 0; v < nn && rc == ORACLE_OK; ++v) {
    if (!in_set[v]) continue;
    int64_t id = add_node(out, g->nodes[v].code);
    if (id < 0) { rc = ORACLE_ERR_NO_MEMORY; break; }
    to_sub[v] = (uint32_t)id;
    sub_to_graph[id] = v;
  }
  for (uint32_t v = 0; v < nn && rc == ORACLE_OK; ++v) {
    if (!in_set[v]) continue;
    const onode* nd = &g->nodes[v];
    for (uint32_t k = 0; k < nd->in.n && rc == ORACLE_OK; ++k) {
      const oedge* ed = &g->edges[nd->in.a[k]];
      if (to_sub[ed->tail] != UINT32_MAX &&
          add_edge(out, to_sub[ed->tail], to_sub[v], (uint32_t)ed->weight))
        rc = ORACLE_ERR_NO_MEMORY;
    }
    for (uint32_t k = 0; k < nd->aligned.n && rc == ORACLE_OK; ++k) {
      uint32_t a = to_sub[nd->aligned.a[k]];
      if (a != UINT32_MAX && vu_push(&out->nodes[to_sub[v]].aligned, a)) rc = ORACLE_ERR_NO_MEMORY;
    }
  }
  if (rc == ORACLE_OK && topological_sort(out)) rc = ORACLE_ERR_NO_MEMORY;
  vu_free(&stack);
  free(in_set);
  free(to_sub);
  return rc;
}

uint32_t oracle_graph_path(const oracle_graph* g, uint32_t label,
                           uint32_t* out, uint32_t cap) {
  if (label >= g->sequences.n) return 0;
  uint32_t n = 0;
  int64_t it = g->sequences.a[label];
  while (it >= 0) {
    if (n < cap) out[n] = (uint32_t)it;
    ++n;
    it = successor(g, (uint32_t)it, label);
  }
  return n;
}

/* ------------------------------------------------------------------ */
/* engine                                                              */
/* ------------------------------------------------------------------ */
oracle_engine* oracle_engine_create(int32_t type, int8_t m, int8_t n, int8_t g,
                                    int8_t e, int8_t q, int8_t c,
                                    int32_t* status) {
  *status = ORACLE_OK;
  if (type != T_SW && type != T_NW && type != T_OV) {
    *status = ORACLE_ERR_INVALID_ARGUMENT;
    return NULL;
  }
  if (g > 0 || q > 0 || e > 0 || c > 0) {
    *status = ORACLE_ERR_INVALID_ARGUMENT;
    return NULL;
  }
  oracle_engine* en = (oracle_engine*)calloc(1, sizeof(oracle_engine));
  if (!en) {
    *status = ORACLE_ERR_NO_MEMORY;
    return NULL;
  }
  /* subtype resolution and canonical penalties (alignment_engine.cpp:57-66) */
  int32_t sub = g >= e ? S_LIN : ((g <= q || e >= c) ? S_AFF : S_CVX);
  if (sub == S_LIN) {
    e = g;
  } else if (sub == S_AFF) {
    q = g;
    c = e;
  }
  en->type = type;
  en->subtype = sub;
  en->m = m; en->n = n; en->g = g; en->e = e; en->q = q; en->c = c;
  return en;
}

void oracle_engine_destroy(oracle_engine* en) { free(en); }
int32_t oracle_engine_subtype(const oracle_engine* en) { return en->subtype; }

/* AlignmentEngine::WorstCaseAlignmentScore (alignment_engine.cpp:101-110) */
static int64_t gap_score(const oracle_engine* en, int64_t len) {
  if (len == 0) return 0;
  int64_t a = en->g + (len - 1) * en->e;
  int64_t b = en->q + (len - 1) * en->c;
  return a < b ? a : b;
}
static int64_t worst_case(const oracle_engine* en, int64_t i, int64_t j) {
  int64_t d = i > j ? i - j : j - i;
  int64_t mn = i < j ? i : j;
  int64_t a = -1 * (en->m * mn + gap_score(en, d));
  int64_t b = gap_score(en, i) + gap_score(en, j);
  return a < b ? a : b;
}

static inline int32_t imax(int32_t a, int32_t b) { return a > b ? a : b; }

typedef struct {
  int32_t* p;
  uint64_t n, cap;
} vec_i32;
static int vi_push2(vec_i32* v, int32_t a, int32_t b) {
  if (v->n + 2 > v->cap) {
    uint64_t nc = v->cap ? v->cap * 2 : 256;
    int32_t* np = (int32_t*)realloc(v->p, nc * sizeof(int32_t));
    if (!np) return -1;
    v->p = np;
    v->cap = nc;
  }
  v->p[v->n++] = a;
  v->p[v->n++] = b;
  return 0;
}

int32_t oracle_align(oracle_engine* en, const char* seq, uint32_t len,
                     const oracle_graph* gr, int32_t* score, int32_t* pairs,
                     uint32_t pairs_cap, uint32_t* n_pairs) {
  *n_pairs = 0;
  if (len > (uint32_t)INT32_MAX) return ORACLE_ERR_TOO_LARGE;
  if (gr->n_nodes == 0 || len == 0) return ORACLE_OK;

  /* width rule (implementation.hpp:719-726) */
  int64_t wc = worst_case(en, (int64_t)len + 8, gr->n_nodes);
  if (wc < (int64_t)INT32_MIN + 1024) return ORACLE_ERR_OVERFLOW;
  const int32_t lanes = wc < (int64_t)INT16_MIN + 1024 ? 8 : 16;
  const int32_t NEG = lanes == 8 ? INT32_MIN + 1024 : INT16_MIN + 1024;

  const int32_t type = en->type, sub = en->subtype;
  const int32_t m = en->m, n = en->n, g = en->g, e = en->e, q = en->q,
                c = en->c;
  const uint32_t V = gr->n_nodes;
  const uint64_t L = len;
  const uint64_t rows = (uint64_t)V + 1;
  const int nmat = sub == S_LIN ? 1 : (sub == S_AFF ? 3 : 5);

  int32_t* M = (int32_t*)malloc(rows * L * nmat * sizeof(int32_t));
  int32_t* prof = (int32_t*)malloc((size_t)(gr->num_codes ? gr->num_codes : 1) * L * sizeof(int32_t));
  int32_t* fc = (int32_t*)malloc(rows * 3 * sizeof(int32_t));
  uint32_t* n2r = (uint32_t*)malloc((size_t)V * sizeof(uint32_t));
  uint32_t* predbuf = NULL;
  uint32_t predcap = 0;
  vec_i32 aln = {0};
  int32_t rc = ORACLE_OK;
  if (!M || !prof || !fc || !n2r) {
    rc = ORACLE_ERR_NO_MEMORY;
    goto done;
  }
  int32_t* H = M;
  int32_t* F = sub != S_LIN ? M + rows * L : NULL;
  int32_t* E = sub != S_LIN ? M + 2 * rows * L : NULL;
  int32_t* O = sub == S_CVX ? M + 3 * rows * L : NULL;
  int32_t* Q = sub == S_CVX ? M + 4 * rows * L : NULL;
  int32_t* fcF = fc + rows;
  int32_t* fcO = fc + 2 * rows;

  /* query profile (implementation.hpp:526-542): node character vs base */
  for (uint32_t k = 0; k < gr->num_codes; ++k) {
    char ch = (char)gr->decoder[k];
    for (uint64_t j = 0; j < L; ++j) prof[k * L + j] = ch == seq[j] ? m : n;
  }
  for (uint32_t r = 0; r < V; ++r) n2r[gr->rank_to_node.a[r]] = r;

  /* first column and first row (implementation.hpp:555-694) */
  if (sub == S_CVX) {
    for (uint64_t j = 0; j < L; ++j) {
      O[j] = NEG;
      Q[j] = q + (int32_t)j * c;
    }
    fcO[0] = 0;
    for (uint32_t i = 1; i <= V; ++i) {
      const onode* nd = &gr->nodes[gr->rank_to_node.a[i - 1]];
      int32_t pen = nd->in.n == 0 ? q - c : NEG;
      for (uint32_t k = 0; k < nd->in.n; ++k)
        pen = imax(pen, fcO[n2r[gr->edges[nd->in.a[k]].tail] + 1]);
      fcO[i] = pen + c;
    }
  }
  if (sub != S_LIN) {
    for (uint64_t j = 0; j < L; ++j) {
      F[j] = NEG;
      E[j] = g + (int32_t)j * e;
    }
    fcF[0] = 0;
    for (uint32_t i = 1; i <= V; ++i) {
      const onode* nd = &gr->nodes[gr->rank_to_node.a[i - 1]];
      int32_t pen = nd->in.n == 0 ? g - e : NEG;
      for (uint32_t k = 0; k < nd->in.n; ++k)
        pen = imax(pen, fcF[n2r[gr->edges[nd->in.a[k]].tail] + 1]);
      fcF[i] = pen + e;
    }
  }
  if (type == T_SW) {
    for (uint64_t j = 0; j < L; ++j) H[j] = 0;
    for (uint64_t i = 0; i < rows; ++i) fc[i] = 0;
  } else {
    if (sub == S_CVX) {
      for (uint64_t j = 0; j < L; ++j) H[j] = imax(E[j], Q[j]);
    } else if (sub == S_AFF) {
      for (uint64_t j = 0; j < L; ++j) H[j] = E[j];
    } else {
      for (uint64_t j = 0; j < L; ++j) H[j] = g + (int32_t)j * g;
    }
    if (type == T_NW) {
      if (sub == S_CVX) {
        for (uint64_t i = 0; i < rows; ++i) fc[i] = imax(fcF[i], fcO[i]);
      } else if (sub == S_AFF) {
        for (uint64_t i = 0; i < rows; ++i) fc[i] = fcF[i];
      } else {
        fc[0] = 0;
        for (uint32_t i = 1; i <= V; ++i) {
          const onode* nd = &gr->nodes[gr->rank_to_node.a[i - 1]];
          int32_t pen = nd->in.n == 0 ? 0 : NEG;
          for (uint32_t k = 0; k < nd->in.n; ++k)
            pen = imax(pen, fc[n2r[gr->edges[nd->in.a[k]].tail] + 1]);
          fc[i] = pen + g;
        }
      }
    } else {
      for (uint64_t i = 0; i < rows; ++i) fc[i] = 0;
    }
  }

  /* forward pass over rows in rank order */
  int32_t max_score = type == T_SW ? 0 : NEG;
  int64_t max_i = -1, max_j = -1;
  for (uint32_t r = 0; r < V; ++r) {
    const onode* nd = &gr->nodes[gr->rank_to_node.a[r]];
    const uint64_t i = (uint64_t)r + 1;
    const int32_t* pr = prof + (uint64_t)nd->code * L;
    uint32_t np = nd->in.n ? nd->in.n : 1;
    if (np > predcap) {
      free(predbuf);
      predcap = np * 2;
      predbuf = (uint32_t*)malloc(predcap * sizeof(uint32_t));
      if (!predbuf) { rc = ORACLE_ERR_NO_MEMORY; goto done; }
    }
    if (nd->in.n == 0) {
      predbuf[0] = 0;
    } else {
      for (uint32_t k = 0; k < nd->in.n; ++k)
        predbuf[k] = n2r[gr->edges[nd->in.a[k]].tail] + 1;
    }
    int32_t* Hi = H + i * L;
    int32_t* Fi = F ? F + i * L : NULL;
    int32_t* Oi = O ? O + i * L : NULL;
    for (uint32_t k = 0; k < np; ++k) {
      const uint64_t p = predbuf[k];
      const int32_t* Hp = H + p * L;
      const int32_t hm1 = fc[p];
      if (sub == S_LIN) {
        for (uint64_t j = 0; j < L; ++j) {
          int32_t v = imax((j ? Hp[j - 1] : hm1) + pr[j], Hp[j] + g);
          Hi[j] = k ? imax(Hi[j], v) : v;
        }
      } else {
        const int32_t* Fp = F + p * L;
        for (uint64_t j = 0; j < L; ++j) {
          int32_t d = (j ? Hp[j - 1] : hm1) + pr[j];
          int32_t f = imax(Hp[j] + (g - e), Fp[j]) + e;
          Hi[j] = k ? imax(Hi[j], d) : d;
          Fi[j] = k ? imax(Fi[j], f) : f;
        }
        if (sub == S_CVX) {
          const int32_t* Op = O + p * L;
          for (uint64_t j = 0; j < L; ++j) {
            int32_t o = imax(Hp[j] + (q - c), Op[j]) + c;
            Oi[j] = k ? imax(Oi[j], o) : o;
          }
        }
      }
    }
    /* in-row (horizontal) pass */
    int32_t rowmax = 0; /* _mmxxx_max_value starts from 0 */
    const int32_t fci = fc[i];
    if (sub == S_LIN) {
      int32_t prevf = fci; /* H pre-clamp at j-1 */
      for (uint64_t j = 0; j < L; ++j) {
        int32_t hf = imax(Hi[j], prevf + g);
        prevf = hf;
        int32_t hs = type == T_SW ? imax(hf, 0) : hf;
        Hi[j] = hs;
        rowmax = imax(rowmax, hs);
      }
    } else if (sub == S_AFF) {
      int32_t* Ei = E + i * L;
      int32_t h1p = 0, ep = 0;
      for (uint64_t j = 0; j < L; ++j) {
        int32_t h1 = imax(Hi[j], Fi[j]);
        int32_t ev = j ? imax(h1p + g, ep + e) : fci + g;
        Ei[j] = ev;
        int32_t hf = imax(h1, ev);
        int32_t hs = type == T_SW ? imax(hf, 0) : hf;
        Hi[j] = hs;
        rowmax = imax(rowmax, hs);
        h1p = h1;
        ep = ev;
      }
    } else {
      int32_t* Ei = E + i * L;
      int32_t* Qi = Q + i * L;
      int32_t h1p = 0, ep = 0, qp = 0;
      for (uint64_t j = 0; j < L; ++j) {
        int32_t h1 = imax(Hi[j], imax(Fi[j], Oi[j]));
        int32_t qv = j ? imax(h1p + q, qp + c) : fci + q;
        int32_t ev = fci + g;
        if (j) {
          ev = imax(h1p + g, ep + e);
          if (j % (uint64_t)lanes == 0) ev = imax(ev, qp + g);
        }
        Ei[j] = ev;
        Qi[j] = qv;
        int32_t hf = imax(h1, imax(ev, qv));
        int32_t hs = type == T_SW ? imax(hf, 0) : hf;
        Hi[j] = hs;
        rowmax = imax(rowmax, hs);
        h1p = h1;
        ep = ev;
        qp = qv;
      }
    }
    /* row selection (strict <: the first row in rank order wins) */
    if (type == T_SW) {
      if (max_score < rowmax) {
        max_score = rowmax;
        max_i = (int64_t)i;
      }
    } else if (nd->out.n == 0) {
      int32_t v = type == T_OV ? rowmax : Hi[L - 1];
      if (max_score < v) {
        max_score = v;
        max_i = (int64_t)i;
      }
    }
  }

  if (max_i == -1 && max_j == -1) goto done; /* empty, score untouched */
  if (score) *score = max_score;

  if (type == T_NW) {
    max_j = (int64_t)L - 1;
  } else {
    /* SW and OV (only sink rows are selected in OV): first column equal to
     * the maximum, or -1 when none is (OV with a negative best row). */
    const int32_t* Hm = H + (uint64_t)max_i * L;
    max_j = -1;
    for (uint64_t j = 0; j < L; ++j) {
      if (Hm[j] == max_score) {
        max_j = (int64_t)j;
        break;
      }
    }
  }

  /* traceback (implementation.hpp:955-1124, 1324-1574, 1826-2121) */
  {
    int64_t i = max_i, j = max_j, prev_i = 0, prev_j = 0;
    uint64_t guard = 0, guard_max = 4 * ((uint64_t)V + L) + 64;
    while (1) {
      if (++guard > guard_max) { rc = ORACLE_ERR_TRACEBACK; goto done; }
      if (j == -1 || i == 0) break;
      const uint32_t node = gr->rank_to_node.a[i - 1];
      const onode* nd = &gr->nodes[node];
      const int32_t* Hi = H + (uint64_t)i * L;
      const int32_t h = Hi[j];
      if (type == T_SW && h == 0) break;
      uint32_t np = nd->in.n ? nd->in.n : 1;
      if (nd->in.n == 0) {
        predbuf[0] = 0;
      } else {
        for (uint32_t k = 0; k < nd->in.n; ++k)
          predbuf[k] = n2r[gr->edges[nd->in.a[k]].tail] + 1;
      }
      const int32_t prf = prof[(uint64_t)nd->code * L + j];
      int found = 0, ext_left = 0, ext_up = 0;
      for (uint32_t k = 0; k < np; ++k) {
        uint64_t p = predbuf[k];
        int32_t hd = j ? H[p * L + j - 1] : fc[p];
        if (h == hd + prf) {
          prev_i = (int64_t)p;
          prev_j = j - 1;
          found = 1;
          break;
        }
      }
      if (!found) {
        for (uint32_t k = 0; k < np; ++k) {
          uint64_t p = predbuf[k];
          int32_t hp = H[p * L + j];
          int take = 0;
          if (sub == S_LIN) {
            take = h == hp + g;
          } else if (sub == S_AFF) {
            ext_up = h == F[p * L + j] + e;
            take = ext_up || h == hp + g;
          } else {
            ext_up = h == F[p * L + j] + e;
            if (ext_up) {
              take = 1;
            } else if (h == hp + g) {
              take = 1;
            } else {
              ext_up = h == O[p * L + j] + c;
              take = ext_up || h == hp + q;
            }
          }
          if (take) {
            prev_i = (int64_t)p;
            prev_j = j;
            found = 1;
            break;
          }
        }
      }
      if (!found) {
        int32_t hl = j ? Hi[j - 1] : fc[i];
        int take = 0;
        if (sub == S_LIN) {
          take = h == hl + g;
        } else if (sub == S_AFF) {
          int32_t el = j ? E[(uint64_t)i * L + j - 1] : fc[i];
          ext_left = h == el + e;
          take = ext_left || h == hl + g;
        } else {
          int32_t el = j ? E[(uint64_t)i * L + j - 1] : fc[i];
          int32_t ql = j ? Q[(uint64_t)i * L + j - 1] : fc[i];
          ext_left = h == el + e;
          if (ext_left) {
            take = 1;
          } else if (h == hl + g) {
            take = 1;
          } else {
            ext_left = h == ql + c;
            take = ext_left || h == hl + q;
          }
        }
        if (take) {
          prev_i = i;
          prev_j = j - 1;
          found = 1;
        }
      }
      if (vi_push2(&aln, i == prev_i ? -1 : (int32_t)node,
                   j == prev_j ? -1 : (int32_t)j)) {
        rc = ORACLE_ERR_NO_MEMORY;
        goto done;
      }
      i = prev_i;
      j = prev_j;
      if (ext_left) {
        const int32_t* Ei = E + (uint64_t)i * L;
        const int32_t* Qi = Q ? Q + (uint64_t)i * L : NULL;
        while (1) {
          if (++guard > guard_max) { rc = ORACLE_ERR_TRACEBACK; goto done; }
          if (vi_push2(&aln, -1, (int32_t)j)) { rc = ORACLE_ERR_NO_MEMORY; goto done; }
          --j;
          if (j == -1) break;
          if (Ei[j] + e != Ei[j + 1]) break;
          if (Qi && Qi[j] + c != Qi[j + 1]) break;
        }
      } else if (ext_up) {
        while (1) {
          if (++guard > guard_max) { rc = ORACLE_ERR_TRACEBACK; goto done; }
          const uint32_t un = gr->rank_to_node.a[i - 1];
          const onode* ud = &gr->nodes[un];
          const int32_t fv = F[(uint64_t)i * L + j];
          int stop;
          prev_i = 0;
          if (sub == S_AFF) {
            stop = 0;
            for (uint32_t k = 0; k < ud->in.n; ++k) {
              uint64_t p = n2r[gr->edges[ud->in.a[k]].tail] + 1;
              stop = fv == H[p * L + j] + g;
              if (stop || fv == F[p * L + j] + e) {
                prev_i = (int64_t)p;
                break;
              }
            }
          } else {
            const int32_t ov = O[(uint64_t)i * L + j];
            stop = 1;
            for (uint32_t k = 0; k < ud->in.n; ++k) {
              uint64_t p = n2r[gr->edges[ud->in.a[k]].tail] + 1;
              if (fv == F[p * L + j] + e || ov == O[p * L + j] + c) {
                prev_i = (int64_t)p;
                stop = 0;
                break;
              }
            }
            if (stop) {
              for (uint32_t k = 0; k < ud->in.n; ++k) {
                uint64_t p = n2r[gr->edges[ud->in.a[k]].tail] + 1;
                if (fv == H[p * L + j] + g || ov == H[p * L + j] + q) {
                  prev_i = (int64_t)p;
                  break;
                }
              }
            }
          }
          if (vi_push2(&aln, (int32_t)un, -1)) { rc = ORACLE_ERR_NO_MEMORY; goto done; }
          i = prev_i;
          if (stop || i == 0) break;
        }
      }
    }
    if (type == T_NW) {
      while (i == 0 && j != -1) {
        if (vi_push2(&aln, -1, (int32_t)j)) { rc = ORACLE_ERR_NO_MEMORY; goto done; }
        --j;
      }
      while (i != 0 && j == -1) {
        if (++guard > guard_max) { rc = ORACLE_ERR_TRACEBACK; goto done; }
        const uint32_t un = gr->rank_to_node.a[i - 1];
        const onode* ud = &gr->nodes[un];
        if (vi_push2(&aln, (int32_t)un, -1)) { rc = ORACLE_ERR_NO_MEMORY; goto done; }
        if (ud->in.n == 0) {
          i = 0;
        } else {
          for (uint32_t k = 0; k < ud->in.n; ++k) {
            uint64_t p = n2r[gr->edges[ud->in.a[k]].tail] + 1;
            int hit;
            if (sub == S_LIN) {
              hit = fc[i] == fc[p] + g;
            } else if (sub == S_AFF) {
              hit = fc[i] == fc[p] + e;
            } else {
              hit = fcF[i] == fcF[p] + e || fcO[i] == fcO[p] + c;
            }
            if (hit) {
              i = (int64_t)p;
              break;
            }
          }
        }
      }
    }
  }
  {
    uint64_t np = aln.n / 2;
    if (np > pairs_cap) {
      rc = ORACLE_ERR_CAPACITY;
      goto done;
    }
    for (uint64_t k = 0; k < np; ++k) {
      pairs[2 * k] = aln.p[2 * (np - 1 - k)];
      pairs[2 * k + 1] = aln.p[2 * (np - 1 - k) + 1];
    }
    *n_pairs = (uint32_t)np;
  }
done:
  free(M);
  free(prof);
  free(fc);
  free(n2r);
  free(predbuf);
  free(aln.p);
  return rc;
}

/* ------------------------------------------------------------------ */
/* window driver (src/main.cpp:275-314)                                */
/* ------------------------------------------------------------------ */

/* Reverse complement used for strand-ambiguous mode.  spoa calls
 * biosoup::Sequence::ReverseAndComplement (biosoup 0.10.0, not part of the
 * reference tree): the bases are complemented by Watson-Crick/IUPAC pairing
 * and the string reversed; the quality string is reversed. */
static char complement_base(char ch) {
  switch (ch) {
    case 'A': return 'T';
    case 'C': return 'G';
    case 'G': return 'C';
    case 'T': return 'A';
    case 'U': return 'A';
    case 'R': return 'Y';
    case 'Y': return 'R';
    case 'K': return 'M';
    case 'M': return 'K';
    case 'B': return 'V';
    case 'D': return 'H';
    case 'H': return 'D';
    case 'V': return 'B';
    case 'a': return 't';
    case 'c': return 'g';
    case 'g': return 'c';
    case 't': return 'a';
    case 'u': return 'a';
    default: return ch;
  }
}

static int32_t window_run_impl(const oracle_window_params* p,
                               oracle_graph* g, uint32_t n_reads,
                               const char* seqs, const uint64_t* seq_off,
                               const char* quals, int32_t* scores,
                               uint8_t* reversed, int32_t* aln_pairs,
                               uint64_t aln_cap, uint64_t* aln_off,
                               uint64_t* cells) {
  int32_t st = 0;
  oracle_engine* en =
      oracle_engine_create(p->type, p->m, p->n, p->g, p->e, p->q, p->c, &st);
  if (!en) return st;
  uint32_t maxlen = 0;
  for (uint32_t r = 0; r < n_reads; ++r) {
    uint64_t l = seq_off[r + 1] - seq_off[r];
    if (l > maxlen) maxlen = (uint32_t)l;
  }
  char* rc = (char*)malloc((size_t)maxlen + 1);
  char* rq = (char*)malloc((size_t)maxlen + 1);
  uint32_t* w = (uint32_t*)malloc(((size_t)maxlen + 1) * sizeof(uint32_t));
  uint32_t paircap = 0;
  int32_t* pf = NULL;
  int32_t* pr = NULL;
  uint64_t used = 0;
  if (!rc || !rq || !w) { st = ORACLE_ERR_NO_MEMORY; goto out; }
  if (aln_off) aln_off[0] = 0;
  for (uint32_t r = 0; r < n_reads; ++r) {
    const char* s = seqs + seq_off[r];
    const char* qq = quals ? quals + seq_off[r] : NULL;
    uint32_t len = (uint32_t)(seq_off[r + 1] - seq_off[r]);
    uint32_t need = oracle_graph_num_nodes(g) + len + 8;
    if (need > paircap) {
      free(pf);
      free(pr);
      paircap = need * 2;
      pf = (int32_t*)malloc((size_t)paircap * 2 * sizeof(int32_t));
      pr = (int32_t*)malloc((size_t)paircap * 2 * sizeof(int32_t));
      if (!pf || !pr) { st = ORACLE_ERR_NO_MEMORY; goto out; }
    }
    int32_t score = 0;
    uint32_t nf = 0;
    if (cells)
      *cells += (uint64_t)oracle_graph_num_nodes(g) * len *
                (p->strand_ambiguous ? 2u : 1u);
    st = oracle_align(en, s, len, g, &score, pf, paircap, &nf);
    if (st) goto out;
    const char* data = s;
    const char* qual = qq;
    int32_t* use = pf;
    uint32_t nuse = nf;
    uint8_t rev = 0;
    if (p->strand_ambiguous) {
      for (uint32_t k = 0; k < len; ++k) {
        rc[k] = complement_base(s[len - 1 - k]);
        if (qq) rq[k] = qq[len - 1 - k];
      }
      int32_t score_rev = 0;
      uint32_t nr = 0;
      st = oracle_align(en, rc, len, g, &score_rev, pr, paircap, &nr);
      if (st) goto out;
      if (!(score >= score_rev)) {
        data = rc;
        qual = qq ? rq : NULL;
        use = pr;
        nuse = nr;
        rev = 1;
        score = score_rev;
      }
    }
    for (uint32_t k = 0; k < len; ++k)
      w[k] = qual ? (uint32_t)((int32_t)(uint8_t)qual[k] - 33) : 1u;
    st = oracle_add_alignment(g, use, nuse, data, len, w, len);
    if (st) goto out;
    if (scores) scores[r] = score;
    if (reversed) reversed[r] = rev;
    if (aln_pairs) {
      if (used + 2ull * nuse > aln_cap) { st = ORACLE_ERR_CAPACITY; goto out; }
      if (nuse) memcpy(aln_pairs + used, use, (size_t)nuse * 2 * sizeof(int32_t));
    }
    used += 2ull * nuse;
    if (aln_off) aln_off[r + 1] = used / 2;
  }
out:
  free(rc);
  free(rq);
  free(w);
  free(pf);
  free(pr);
  oracle_engine_destroy(en);
  return st;
}

int32_t oracle_window_run(const oracle_window_params* p, oracle_graph* g,
                          uint32_t n_reads, const char* seqs,
                          const uint64_t* seq_off, const char* quals,
                          int32_t* scores, uint8_t* reversed,
                          int32_t* aln_pairs, uint64_t aln_cap,
                          uint64_t* aln_off) {
  return window_run_impl(p, g, n_reads, seqs, seq_off, quals, scores,
                         reversed, aln_pairs, aln_cap, aln_off, NULL);
}

/* ------------------------------------------------------------------ */
/* multi-threaded batch (one window per task)                           */
/* ------------------------------------------------------------------ */
typedef struct {
  const oracle_window_params* p;
  uint32_t n_windows;
  const uint32_t* win_read_off;
  const char* seqs;
  const uint64_t* seq_off;
  const char* quals;
  char* cons;
  uint64_t cons_cap;
  uint64_t* cons_off; /* per window, fixed stride region start */
  int32_t* read_scores;
  double* win_seconds; /* per window, wall time of its thread, or NULL */
  atomic_uint next;
  atomic_int status;
  atomic_ullong cells;
} batch_ctx;

static double now_seconds(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void* batch_worker(void* arg) {
  batch_ctx* bc = (batch_ctx*)arg;
  oracle_graph* g = oracle_graph_create();
  if (!g) {
    atomic_store(&bc->status, ORACLE_ERR_NO_MEMORY);
    return NULL;
  }
  for (;;) {
    uint32_t w = atomic_fetch_add(&bc->next, 1);
    if (w >= bc->n_windows) break;
    const double t0 = bc->win_seconds ? now_seconds() : 0.0;
    oracle_graph_clear(g);
    uint32_t r0 = bc->win_read_off[w], r1 = bc->win_read_off[w + 1];
    uint64_t cells = 0;
    /* seq_off is global; window_run_impl indexes seq_off[r] - seq_off[r0] */
    int32_t st = window_run_impl(bc->p, g, r1 - r0, bc->seqs, bc->seq_off + r0,
                                 bc->quals,
                                 bc->read_scores ? bc->read_scores + r0 : NULL,
                                 NULL, NULL, 0, NULL, &cells);
    if (st) atomic_store(&bc->status, st);
    atomic_fetch_add(&bc->cells, cells);
    if (bc->cons) {
      uint64_t a = bc->cons_off[w];
      uint64_t cap = bc->cons_off[w + 1] - a;
      uint32_t n = oracle_consensus(g, bc->cons + a, (uint32_t)cap);
      if (n < cap) bc->cons[a + n] = 0;
    }
    if (bc->win_seconds) bc->win_seconds[w] = now_seconds() - t0;
  }
  oracle_graph_destroy(g);
  return NULL;
}

int32_t oracle_batch_run(const oracle_window_params* p, uint32_t n_windows,
                         const uint32_t* win_read_off, const char* seqs,
                         const uint64_t* seq_off, const char* quals,
                         int32_t n_threads, char* cons, uint64_t cons_cap,
                         uint64_t* cons_off, int32_t* read_scores,
                         uint64_t* cells, double* win_seconds) {
  (void)cons_cap;
  batch_ctx bc;
  bc.p = p;
  bc.n_windows = n_windows;
  bc.win_read_off = win_read_off;
  bc.seqs = seqs;
  bc.seq_off = seq_off;
  bc.quals = quals;
  bc.cons = cons;
  bc.cons_cap = cons_cap;
  bc.cons_off = cons_off;
  bc.read_scores = read_scores;
  bc.win_seconds = win_seconds;
  atomic_init(&bc.next, 0);
  atomic_init(&bc.status, 0);
  atomic_init(&bc.cells, 0);
  if (n_threads < 1) n_threads = 1;
  pthread_t* th = (pthread_t*)malloc((size_t)n_threads * sizeof(pthread_t));
  if (!th) return ORACLE_ERR_NO_MEMORY;
  int started = 0;
  for (int t = 0; t < n_threads; ++t) {
    if (pthread_create(&th[t], NULL, batch_worker, &bc) == 0) ++started;
  }
  for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
  free(th);
  if (cells) *cells = atomic_load(&bc.cells);
  if (started == 0) return ORACLE_ERR_NO_MEMORY;
  return atomic_load(&bc.status);
}
