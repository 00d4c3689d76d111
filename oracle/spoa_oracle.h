/*
 * spoa_oracle.h - CPU restatement of spoa's partial-order-alignment path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle for the GPU path: a
 * plain-C restatement of the reference algorithm (spoa v4, AVX2 build of
 * SimdAlignmentEngine + Graph).  Only the test-suite, the smoke check and the
 * CPU-baseline leg of the benchmark may load it; the product library never
 * links or calls it.
 *
 * Pinned against: the 18 golden consensus strings of test/spoa_test.cpp on
 * test/data/sample.fastq.gz, and against outputs of the reference library
 * itself (compiled from its own sources by oracle/Makefile) on seeded
 * synthetic windows (tests/golden/).
 */
#ifndef SPOA_ORACLE_H_
#define SPOA_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes (shared meaning with the GPU library's C-ABI). */
#define ORACLE_OK 0
#define ORACLE_ERR_INVALID_ARGUMENT 1
#define ORACLE_ERR_TOO_LARGE 2
#define ORACLE_ERR_OVERFLOW 3
#define ORACLE_ERR_NO_MEMORY 4
#define ORACLE_ERR_INVALID_ALIGNMENT 5
#define ORACLE_ERR_MISSING_SEQUENCE 6
#define ORACLE_ERR_UNEQUAL_WEIGHTS 7
#define ORACLE_ERR_CAPACITY 8
#define ORACLE_ERR_TRACEBACK 9

typedef struct oracle_engine oracle_engine;
typedef struct oracle_graph oracle_graph;

/* AlignmentEngine::Create (src/alignment_engine.cpp:32-73). type: 0 SW,
 * 1 NW, 2 OV.  Writes the resolved subtype (0 linear, 1 affine, 2 convex). */
oracle_engine* oracle_engine_create(int32_t type, int8_t m, int8_t n, int8_t g,
                                    int8_t e, int8_t q, int8_t c,
                                    int32_t* status);
void oracle_engine_destroy(oracle_engine* en);
int32_t oracle_engine_subtype(const oracle_engine* en);

oracle_graph* oracle_graph_create(void);
void oracle_graph_destroy(oracle_graph* g);
void oracle_graph_clear(oracle_graph* g);

/* AlignmentEngine::Align.  pairs receives 2*n int32 values
 * (node id or -1, sequence position or -1).  *score is written only when
 * the reference writes it.  Returns a status code. */
int32_t oracle_align(oracle_engine* en, const char* seq, uint32_t len,
                     const oracle_graph* g, int32_t* score, int32_t* pairs,
                     uint32_t pairs_cap, uint32_t* n_pairs);

/* Graph::AddAlignment with explicit per-base weights (graph.cpp:155-247). */
int32_t oracle_add_alignment(oracle_graph* g, const int32_t* pairs,
                             uint32_t n_pairs, const char* seq, uint32_t len,
                             const uint32_t* weights, uint32_t n_weights);

/* Graph::GenerateConsensus (graph.cpp:368-375).  Returns the length. */
uint32_t oracle_consensus(oracle_graph* g, char* out, uint32_t cap);

/* Graph::GenerateMultipleSequenceAlignment (graph.cpp:339-366).  Rows are
 * written back to back, each row_len bytes. */
int32_t oracle_msa(oracle_graph* g, int32_t include_consensus, char* out,
                   uint64_t cap, uint32_t* n_rows, uint32_t* row_len);

/* Read accessors used to emit GFA and to compare graph structure. */
uint32_t oracle_graph_num_nodes(const oracle_graph* g);
uint32_t oracle_graph_num_edges(const oracle_graph* g);
uint32_t oracle_graph_num_sequences(const oracle_graph* g);
uint32_t oracle_graph_consensus_len(const oracle_graph* g);
/* codes[n] = decoded character of every node; rank[n] = rank_to_node order;
 * edges as (tail, head) plus weight in node-major out-edge order;
 * seq_begin[s]; consensus node ids; path of sequence s via Successor. */
void oracle_graph_export(const oracle_graph* g, uint8_t* chars,
                         uint32_t* rank_to_node, uint32_t* edge_tail,
                         uint32_t* edge_head, int64_t* edge_weight,
                         uint32_t* seq_begin, uint32_t* consensus);
uint32_t oracle_graph_path(const oracle_graph* g, uint32_t label,
                           uint32_t* out, uint32_t cap);

/* Edges in id order (Graph::edges()) and the aligned-node lists as CSR
 * (aligned_off: n_nodes + 1 entries); NULL skips an array.  Returns the
 * total length of the aligned lists. */
uint32_t oracle_graph_export_ids(const oracle_graph* g, uint32_t* edge_tail,
                                 uint32_t* edge_head, int64_t* edge_weight,
                                 uint32_t* aligned_off, uint32_t* aligned);

/* Labels of every edge in id order as CSR (label_off: n_edges + 1
 * entries); NULL skips an array.  Returns the total number of labels. */
uint32_t oracle_graph_edge_labels(const oracle_graph* g, uint32_t* label_off,
                                  uint32_t* labels);

/* Graph::save then Graph::load (include/spoa/graph.hpp:187-276) of g into
 * `out` (cleared first), with the reference's load order of edge and
 * aligned lists. */
int32_t oracle_graph_reload(const oracle_graph* g, oracle_graph* out);

/* Graph::Subgraph (graph.cpp:518-595) into `out` (cleared first);
 * sub_to_graph receives n_nodes(g) entries: the id in g of every node of
 * out, then UINT32_MAX.  Graph::UpdateAlignment (graph.cpp:597-605) is the
 * map of an alignment's node ids through sub_to_graph. */
int32_t oracle_subgraph(const oracle_graph* g, uint32_t begin, uint32_t end,
                        oracle_graph* out, uint32_t* sub_to_graph);

/* One whole window, the way spoa's CLI drives it (src/main.cpp:275-314):
 * reads are aligned in order and added; with strand_ambiguous both strands
 * are aligned and the forward strand kept if score >= score_rev.
 * quals may be NULL (unit weights).  Outputs per read: score, reversed flag,
 * alignment (pairs written back to back, aln_off[r]..aln_off[r+1]).
 * Returns a status code.  Consensus/MSA are read from the graph after. */
typedef struct {
  int32_t type;
  int8_t m, n, g, e, q, c;
  int8_t strand_ambiguous;
} oracle_window_params;

int32_t oracle_window_run(const oracle_window_params* p, oracle_graph* g,
                          uint32_t n_reads, const char* seqs,
                          const uint64_t* seq_off, const char* quals,
                          int32_t* scores, uint8_t* reversed,
                          int32_t* aln_pairs, uint64_t aln_cap,
                          uint64_t* aln_off);

/* Many independent windows on a pool of host threads, one window per task
 * (each with its own engine and graph, the way spoa's callers scale it).
 * Writes per-window consensus (cons_off[w]..) and returns the number of
 * matrix cells (sum over reads of len x nodes) through *cells; win_seconds
 * (NULL to skip) gets each window's wall time on its thread. */
int32_t oracle_batch_run(const oracle_window_params* p, uint32_t n_windows,
                         const uint32_t* win_read_off, const char* seqs,
                         const uint64_t* seq_off, const char* quals,
                         int32_t n_threads, char* cons, uint64_t cons_cap,
                         uint64_t* cons_off, int32_t* read_scores,
                         uint64_t* cells, double* win_seconds);

#ifdef __cplusplus
}
#endif

#endif /* SPOA_ORACLE_H_ */
