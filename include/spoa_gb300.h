/*
 * spoa_gb300.h - C ABI of the GB300 partial-order-alignment library.
 *
 * Plain pointers and sizes only; every call returns a status code
 * (SPOA_GB300_OK or one of the codes below).  The library runs on one CUDA
 * device (the current device when an object is created) and never falls back
 * to the CPU: without a usable GPU every entry point that computes returns
 * SPOA_GB300_ERR_CUDA.
 *
 * Each declaration names the spoa (v4) interface it replaces.  Paths are
 * relative to the spoa source tree.
 */
#ifndef SPOA_GB300_H_
#define SPOA_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The C++ layer maps them to the reference's
 * std::invalid_argument messages. */
#define SPOA_GB300_OK 0
#define SPOA_GB300_ERR_INVALID_ARGUMENT 1 /* bad type / positive penalty */
#define SPOA_GB300_ERR_TOO_LARGE 2        /* "too large sequence!" */
#define SPOA_GB300_ERR_OVERFLOW 3         /* "possible overflow!" */
#define SPOA_GB300_ERR_NO_MEMORY 4        /* "insufficient memory!" */
#define SPOA_GB300_ERR_INVALID_ALIGNMENT 5
#define SPOA_GB300_ERR_MISSING_SEQUENCE 6
#define SPOA_GB300_ERR_UNEQUAL_WEIGHTS 7
#define SPOA_GB300_ERR_CAPACITY 8 /* a window outgrew its device arena */
#define SPOA_GB300_ERR_TRACEBACK 9
#define SPOA_GB300_ERR_CUDA 10

/* Alignment types and gap models (include/spoa/alignment_engine.hpp:16-26) */
#define SPOA_GB300_SW 0
#define SPOA_GB300_NW 1
#define SPOA_GB300_OV 2
#define SPOA_GB300_LINEAR 0
#define SPOA_GB300_AFFINE 1
#define SPOA_GB300_CONVEX 2

typedef struct spoa_gb300_engine spoa_gb300_engine;
typedef struct spoa_gb300_graph spoa_gb300_graph;
typedef struct spoa_gb300_batch spoa_gb300_batch;

const char* spoa_gb300_status_string(int32_t status);

/* Number of CUDA devices usable by the library (0 when none). */
int32_t spoa_gb300_device_count(void);

/* ---- AlignmentEngine ---------------------------------------------------- */

/* Replaces AlignmentEngine::Create (src/alignment_engine.cpp:32-73, all
 * three overloads funnel into this 7-penalty form): validates, resolves the
 * gap model (linear if g >= e, affine if g <= q or e >= c, else convex) and
 * canonicalises the penalties. */
int32_t spoa_gb300_engine_create(int32_t type, int8_t m, int8_t n, int8_t g, int8_t e,
                                 int8_t q, int8_t c, spoa_gb300_engine** out);
void spoa_gb300_engine_destroy(spoa_gb300_engine* engine);
/* Resolved subtype and canonical penalties (AlignmentEngine::subtype_, m_..c_). */
int32_t spoa_gb300_engine_params(const spoa_gb300_engine* engine, int32_t* type,
                                 int32_t* subtype, int8_t* penalties6);

/* Replaces SimdAlignmentEngine::Prealloc
 * (src/simd_alignment_engine_implementation.hpp:381-422): sizes the device
 * DP arena for reads up to max_len against graphs of max_len*alphabet_size
 * nodes. */
int32_t spoa_gb300_engine_prealloc(spoa_gb300_engine* engine, uint32_t max_len,
                                   uint8_t alphabet_size);

/* Replaces AlignmentEngine::Align (include/spoa/alignment_engine.hpp:61-69;
 * SimdAlignmentEngine::Align, implementation.hpp:703-780).  Writes the
 * alignment as n_pairs (node id | -1, position | -1) int32 pairs.
 * *score_written is 1 when the reference would have written *score. */
int32_t spoa_gb300_engine_align(spoa_gb300_engine* engine, const char* sequence,
                                uint32_t sequence_len, const spoa_gb300_graph* graph,
                                int32_t* score, int32_t* score_written, int32_t* pairs,
                                uint32_t pairs_cap, uint32_t* n_pairs);

/* ---- Graph --------------------------------------------------------------- */

/* Replaces Graph::Graph (src/graph.cpp:65-74): an empty device-resident graph. */
int32_t spoa_gb300_graph_create(spoa_gb300_graph** out);
void spoa_gb300_graph_destroy(spoa_gb300_graph* graph);
/* Replaces Graph::Clear (src/graph.cpp:649-658). */
int32_t spoa_gb300_graph_clear(spoa_gb300_graph* graph);

/* Replaces Graph::AddAlignment (src/graph.cpp:155-247) with explicit
 * per-base weights (weights may be NULL: weight 1 per base, graph.cpp:119-125). */
int32_t spoa_gb300_graph_add_alignment(spoa_gb300_graph* graph, const int32_t* pairs,
                                       uint32_t n_pairs, const char* sequence,
                                       uint32_t sequence_len, const uint32_t* weights,
                                       uint32_t n_weights);
/* Replaces the quality overload (src/graph.cpp:137-146): weight = q - 33. */
int32_t spoa_gb300_graph_add_alignment_quality(spoa_gb300_graph* graph, const int32_t* pairs,
                                               uint32_t n_pairs, const char* sequence,
                                               uint32_t sequence_len, const char* quality,
                                               uint32_t quality_len);

/* Fused Align + AddAlignment of one read with no host round trip of the
 * alignment (the per-read body of src/main.cpp:275-314, including the
 * strand-ambiguous choice of main.cpp:285-302 when strand_ambiguous != 0).
 * quality may be NULL. */
int32_t spoa_gb300_align_add(spoa_gb300_engine* engine, spoa_gb300_graph* graph,
                             const char* sequence, uint32_t sequence_len, const char* quality,
                             int32_t strand_ambiguous, int32_t* score, int32_t* reversed);

/* The per-read loop of src/main.cpp:275-314 over n_reads reads (back to
 * back in seqs, n_reads + 1 offsets; quals with the same offsets or NULL):
 * the same as spoa_gb300_align_add once per read in order, but every read's
 * launch is recorded into one CUDA graph, replayed with no host round trip
 * between reads.  No counterpart in the reference.  scores / reversed get
 * one value per added read (either may be NULL); *n_done is the number of
 * reads added: on an error the reads before the failing one stay in the
 * graph and the failing read's status is returned. */
int32_t spoa_gb300_align_add_reads(spoa_gb300_engine* engine, spoa_gb300_graph* graph,
                                   uint32_t n_reads, const char* seqs, const uint64_t* seq_off,
                                   const char* quals, int32_t strand_ambiguous, int32_t* scores,
                                   int32_t* reversed, uint32_t* n_done);

/* Replaces Graph::GenerateConsensus (src/graph.cpp:368-375). */
int32_t spoa_gb300_graph_consensus(spoa_gb300_graph* graph, char* out, uint32_t cap,
                                   uint32_t* len);

/* Replaces Graph::GenerateMultipleSequenceAlignment (src/graph.cpp:339-366):
 * rows * cols bytes, row-major. */
int32_t spoa_gb300_graph_msa(spoa_gb300_graph* graph, int32_t include_consensus, char* out,
                             uint64_t cap, uint32_t* rows, uint32_t* cols);

/* Sizes of the graph (Graph::nodes(), edges(), sequences(), consensus()
 * accessors, include/spoa/graph.hpp:102-132) and of its label lists. */
int32_t spoa_gb300_graph_counts(const spoa_gb300_graph* graph, uint32_t* nodes,
                                uint32_t* edges, uint32_t* sequences, uint32_t* consensus,
                                uint32_t* labels, uint32_t* num_codes);

/* Flat copy of the graph for the host-side views of Graph (graph.hpp:40-132):
 * node characters and codes, in/out edge lists (CSR, insertion order),
 * aligned-node lists (CSR), edges (tail, head, weight, label CSR), rank
 * order, sequence begins, consensus and the coder/decoder tables.  Any
 * pointer may be NULL to skip that array; sizes follow graph_counts. */
int32_t spoa_gb300_graph_export(const spoa_gb300_graph* graph, uint8_t* chars, uint8_t* codes,
                                uint32_t* in_off, uint32_t* in_edges, uint32_t* out_off,
                                uint32_t* out_edges, uint32_t* aligned_off,
                                uint32_t* aligned_nodes, uint32_t* edge_tail,
                                uint32_t* edge_head, int64_t* edge_weight, uint32_t* label_off,
                                uint32_t* labels, uint32_t* rank_to_node, uint32_t* seq_begin,
                                uint32_t* consensus, int32_t* coder256, int32_t* decoder256);

/* GFA 1.0 text of the graph in the layout of the reference CLI's PrintGfa
 * (src/main.cpp:119-199): headers holds one name per sequence (NULL: read0,
 * read1, ...), is_reversed one flag per sequence for reads kept on the
 * reverse strand (NULL: none), and include_consensus adds the path of the
 * last consensus.  *len gets the byte count; out (when not NULL) the text
 * if cap is large enough (SPOA_GB300_ERR_CAPACITY otherwise). */
int32_t spoa_gb300_graph_gfa(const spoa_gb300_graph* graph, const char* const* headers,
                             const uint8_t* is_reversed, int32_t include_consensus, char* out,
                             uint64_t cap, uint64_t* len);

/* Replaces Graph::Subgraph (src/graph.cpp:518-595): `out` (an existing
 * graph, emptied first) receives the part of `graph` reachable from node
 * `end` over in-edges and aligned nodes, not below node id `begin`,
 * renumbered in id order and topologically sorted; subgraph_to_graph
 * (map_len >= number of nodes of `graph`, the size the reference gives its
 * vector) receives the id in `graph` of every node of `out` and UINT32_MAX
 * after them (the reference's nullptr).  begin and end must be node ids of
 * `graph` (the reference does not check them).  Graph::UpdateAlignment
 * (graph.cpp:597-605) is the host-side map of an alignment's node ids
 * through subgraph_to_graph. */
int32_t spoa_gb300_graph_subgraph(const spoa_gb300_graph* graph, uint32_t begin, uint32_t end,
                                  spoa_gb300_graph* out, uint32_t* subgraph_to_graph,
                                  uint32_t map_len);

/* Graph persistence (the reference archives a Graph with cereal,
 * include/spoa/graph.hpp:187-276; cereal is not used here).  save writes
 * the fields the reference archives (coder tables, nodes, edges with labels
 * and weights, sequence starts, aligned pairs, rank order, last consensus)
 * in this library's own layout: *size gets the byte count, and `out` (when
 * not NULL) the bytes if cap is large enough (SPOA_GB300_ERR_CAPACITY
 * otherwise).  load rebuilds a graph from such bytes into `graph` (its
 * previous contents are dropped) the way the reference's Graph::load
 * rebuilds it; malformed input gives SPOA_GB300_ERR_INVALID_ARGUMENT. */
int32_t spoa_gb300_graph_save(const spoa_gb300_graph* graph, uint8_t* out, uint64_t cap,
                              uint64_t* size);
int32_t spoa_gb300_graph_load(spoa_gb300_graph* graph, const uint8_t* in, uint64_t size);

/* ---- Batched windows (no counterpart in the reference) ------------------- *
 * Many independent windows (each one Graph driven by the per-read loop of
 * src/main.cpp:275-314, then GenerateConsensus) in one persistent kernel:
 * every CTA pulls windows from a device work queue.  Inputs and outputs are
 * host pointers; the device copies happen inside the call.               */
typedef struct {
  int32_t type; /* default type when window_type is NULL */
  int8_t m, n, g, e, q, c;
  int8_t pad;
  uint32_t n_windows;
  const uint32_t* window_read_off; /* [n_windows + 1] */
  const int8_t* window_type;       /* [n_windows] or NULL */
  const int8_t* window_strand;     /* [n_windows] strand-ambiguous flags or NULL */
  const char* seqs;                /* all reads back to back */
  const uint64_t* seq_off;         /* [n_reads + 1] */
  const char* quals;               /* same offsets as seqs, or NULL */
  uint32_t max_nodes;              /* per-window node cap (0: automatic) */
  int32_t threads_per_window;      /* 0: chosen per length class */
  int32_t columns_per_thread;      /* 0: chosen per length class */
  int32_t ctas;                    /* 0: fill the device */
  uint64_t memory_budget;          /* bytes for per-CTA arenas (0: automatic) */
  int32_t want_alignments;         /* also return every read's alignment */
  int32_t want_msa;                /* also return every window's MSA */
  int32_t autotune;                /* time the candidate tiles of every length
                                      class on a sample of its windows at the
                                      first launch and keep the fastest (cached
                                      per process, and per device model in the
                                      file named by SPOA_GB300_TILE_CACHE) */
  int32_t windows_per_cta;         /* 2 or 4: windows of 16-bit width in flight
                                      per CTA, their graph updates on parallel
                                      lanes; otherwise 1 */
  int32_t cluster;                 /* 0: windows of 32-bit scores whose rows pass
                                      1,536 columns run on thread-block clusters
                                      (2, 4 or 8 CTAs per window, each a column
                                      range of every row; more CTAs per window
                                      when few windows share the pass); 1:
                                      never; 2, 4 or 8: that many CTAs per such
                                      window (more when its rows need them) */
  int32_t device_set;              /* nonzero: the batch lives on `device`;
                                      0: on the calling thread's current device
                                      at batch_create.  Every later call on the
                                      batch switches to that device and back. */
  int32_t device;
} spoa_gb300_batch_desc;

typedef struct {
  /* filled by the library: pointers stay valid until batch_destroy */
  const int32_t* read_scores;  /* [n_reads] */
  const uint8_t* read_reversed;
  const int32_t* window_status; /* [n_windows] */
  const char* consensus;        /* back to back */
  const uint64_t* consensus_off; /* [n_windows + 1] */
  const int32_t* alignments;    /* pairs, when want_alignments */
  const uint64_t* alignment_off; /* [n_reads + 1] pair offsets */
  const char* msa;              /* when want_msa */
  const uint64_t* msa_off;       /* [n_windows + 1] byte offsets */
  const uint32_t* msa_rows;      /* [n_windows] */
  const uint32_t* msa_cols;
  uint64_t cells;               /* sum over reads of read length x graph nodes */
  uint64_t pred_cells;          /* sum over reads of read length x predecessor
                                   entries (in-edges, row 0 for sources) */
  double kernel_ms;             /* device time of the persistent launch(es) */
  int32_t threads_per_window, columns_per_thread, ctas, launches;
} spoa_gb300_batch_result;

/* Uploads a batch and sizes the device arenas.  Before any CUDA call it
 * returns SPOA_GB300_ERR_INVALID_ARGUMENT for a null descriptor, output or
 * offset array, an unknown type (default or per window), a positive
 * penalty, window_read_off[0] != 0 or decreasing window offsets. */
int32_t spoa_gb300_batch_create(const spoa_gb300_batch_desc* desc, spoa_gb300_batch** out);
/* Runs the persistent kernel on device-resident inputs (stream may be 0).
 * Windows that outgrow their arena are rerun with a larger one. */
int32_t spoa_gb300_batch_launch(spoa_gb300_batch* batch, void* stream);
/* One launch per window, one CTA each: the plain one-window-per-launch form. */
int32_t spoa_gb300_batch_launch_plain(spoa_gb300_batch* batch, void* stream);
/* Copies the results to the host and fills *result. */
int32_t spoa_gb300_batch_fetch(spoa_gb300_batch* batch, spoa_gb300_batch_result* result);
void spoa_gb300_batch_destroy(spoa_gb300_batch* batch);
/* create + launch + fetch: host buffers in, host results out. */
int32_t spoa_gb300_batch_run(const spoa_gb300_batch_desc* desc, spoa_gb300_batch** out,
                             spoa_gb300_batch_result* result);

/* ---- Served windows (no counterpart in the reference) -------------------- *
 * Continuous batching of windows that arrive over time.  A host thread of
 * the server admits arrived windows in arrival order while the memory their
 * arenas need (graph plus DP-and-traceback bytes) fits a fixed device
 * budget, gathers them into launches of the persistent kernel (one CTA per
 * window) on a pool of streams, so windows that arrive while others run
 * start on the GPU beside them, and frees each launch's memory when it
 * completes.  A window whose reads turn out to need 32-bit scores, or whose
 * graph outgrows its arena, is admitted again with the wider kernel or twice
 * the capacity.  Every window is the CLI loop of src/main.cpp:275-314 (reads
 * in order, optionally strand-ambiguous) followed by GenerateConsensus. */
typedef struct spoa_gb300_server spoa_gb300_server;
typedef struct {
  int32_t type; /* default alignment type of submitted windows */
  int8_t m, n, g, e, q, c, pad;
  uint64_t memory_budget;       /* device bytes for in-flight windows (0: 40% of free) */
  int32_t max_streams;          /* launches in flight (0: 32) */
  int32_t max_windows_per_launch; /* (0: 4096) */
  double gather_seconds;        /* wait this long after the oldest arrival to gather
                                   more windows into one launch (0: none) */
  int32_t device_set;           /* nonzero: serve on `device`; 0: on the calling
                                   thread's current device at server_create */
  int32_t device;
  int32_t resident;             /* nonzero: polishing-sized windows (16-bit scores,
                                   reads of at most 640 bases, at most 255 reads
                                   and 65,534 bases) go to one persistent kernel
                                   that keeps running while work arrives: each
                                   window takes a slot of a ring in host-mapped
                                   memory, its reads are copied to the device,
                                   the slot is published, and a CTA of the
                                   running kernel claims it and writes the
                                   consensus back; the kernel's CTAs leave after
                                   20 ms without work (a bounded wait) and the
                                   server starts it again when work arrives.
                                   Other windows, and windows that outgrow the
                                   resident kernel's arenas, are launched as
                                   above. */
} spoa_gb300_server_desc;

int32_t spoa_gb300_server_create(const spoa_gb300_server_desc* desc, spoa_gb300_server** out);
/* Submits one window: n_reads reads back to back in seqs with n_reads + 1
 * offsets (inputs are copied).  type -1 uses the server's type.  The window
 * counts as arrived `delay_seconds` after the call (0: now), which lets a
 * caller replay an arrival schedule.  Returns a ticket. */
int32_t spoa_gb300_server_submit(spoa_gb300_server* server, const char* seqs,
                                 const uint64_t* seq_off, uint32_t n_reads, int32_t type,
                                 int32_t strand_ambiguous, double delay_seconds,
                                 uint64_t* ticket);
/* Blocks until the window of `ticket` is done (timeout_seconds <= 0: no
 * limit), then copies its consensus (up to cap bytes), its status and its
 * latency (completion minus arrival, seconds).  Each ticket can be waited
 * for once.  SPOA_GB300_ERR_INVALID_ARGUMENT for an unknown ticket,
 * SPOA_GB300_ERR_TIMEOUT when the limit passes first (wait again later);
 * the window's own status is in *status. */
#define SPOA_GB300_ERR_TIMEOUT 12
int32_t spoa_gb300_server_wait(spoa_gb300_server* server, uint64_t ticket,
                               double timeout_seconds, char* consensus, uint32_t cap,
                               uint32_t* len, int32_t* status, double* latency_seconds);
/* Launches issued and windows completed so far. */
int32_t spoa_gb300_server_stats(const spoa_gb300_server* server, uint64_t* launches,
                                uint64_t* completed);
/* Windows the resident kernel finished (or handed back to the launch path)
 * and launches of the resident kernel so far. */
int32_t spoa_gb300_server_resident_stats(const spoa_gb300_server* server, uint64_t* windows,
                                         uint64_t* launches);
/* Stops the server once every submitted window has finished. */
void spoa_gb300_server_destroy(spoa_gb300_server* server);

/* ---- One window without device allocation ------------------------------- *
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (work issued between the captures of a CUDA graph, frameworks whose
 * allocator owns all device memory, loops that cannot afford cudaMalloc's
 * implicit device synchronisation): one window -- every read aligned and
 * added in order, as spoa's CLI loop does, then the consensus -- runs
 * through the persistent kernel with its working memory in a fixed
 * 48 MiB array inside the library, which every device that loads the
 * library holds until the process exits.  Nothing is allocated and the call
 * does not synchronise; it is asynchronous on `stream` (0: the default
 * stream).
 *
 * Inputs and outputs are DEVICE pointers owned by the caller: d_seqs (reads
 * back to back), d_seq_off (n_reads + 1 offsets), d_quals (Phred+33, same
 * offsets, or NULL for weight 1), d_consensus (consensus_cap bytes),
 * d_consensus_len (1 value), d_read_scores (n_reads values, or NULL),
 * d_status (1 value: SPOA_GB300_OK, SPOA_GB300_ERR_CAPACITY when the window
 * outgrew the device-checked limits below, SPOA_GB300_ERR_OVERFLOW, or
 * SPOA_GB300_ERR_NEEDS_INT32 when a read needs 32-bit scores).
 * Limits checked on the host, before anything is launched (larger values
 * return SPOA_GB300_ERR_TOO_LARGE): n_reads <= SPOA_GB300_NOALLOC_MAX_READS
 * and max_read_len <= SPOA_GB300_NOALLOC_MAX_READ_LEN.
 * Limits checked on the device, reported in *d_status as
 * SPOA_GB300_ERR_CAPACITY (the host cannot see device-resident reads or the
 * graph): every read at most as long as the max_read_len passed in (more
 * precisely, the column tile chosen for it), at most
 * SPOA_GB300_NOALLOC_MAX_NODES graph nodes, at most
 * SPOA_GB300_NOALLOC_MAX_ALIGNED nodes aligned to any node (one column of
 * the MSA holds at most that many + 1 different letters), a consensus of at
 * most consensus_cap bases.
 * The first call on a device looks up the array's device address; make it
 * before any stream capture.  All calls share the one array, so calls that
 * overlap on the GPU (other streams, other host threads) race with each
 * other: serialise them. */
#define SPOA_GB300_NOALLOC_SCRATCH_BYTES (48ull << 20)
#define SPOA_GB300_NOALLOC_MAX_READS 256
#define SPOA_GB300_NOALLOC_MAX_READ_LEN 640
#define SPOA_GB300_NOALLOC_MAX_NODES 4096
#define SPOA_GB300_NOALLOC_MAX_ALIGNED 63
#define SPOA_GB300_ERR_NEEDS_INT32 11
int32_t spoa_gb300_window_poa_noalloc(int32_t type, int8_t m, int8_t n, int8_t g, int8_t e,
                                      int8_t q, int8_t c, int32_t strand_ambiguous,
                                      uint32_t n_reads, uint32_t max_read_len,
                                      const char* d_seqs, const uint64_t* d_seq_off,
                                      const char* d_quals, char* d_consensus,
                                      uint32_t consensus_cap, uint32_t* d_consensus_len,
                                      int32_t* d_read_scores, int32_t* d_status, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SPOA_GB300_H_ */
