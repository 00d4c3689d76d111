"""spoa_gb300: spoa's partial-order-alignment path on one GB300 GPU.

Python host side over the C ABI in include/spoa_gb300.h.  It mirrors spoa's
C++ interface (include/spoa/alignment_engine.hpp, include/spoa/graph.hpp):

    engine = AlignmentEngine.create(AlignmentType.kNW, 5, -4, -8, -6)
    graph = Graph()
    for seq in reads:
        alignment, score = engine.align(seq, graph)
        graph.add_alignment(alignment, seq)
    consensus = graph.generate_consensus()
    msa = graph.generate_multiple_sequence_alignment()

plus the batched form (many windows in one persistent kernel):

    result = batch_poa(windows, AlignmentType.kOV, 5, -4, -8, -6, -10, -4)

Every call runs on the GPU.  There is no CPU fallback: without the compiled
library or a CUDA device the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libspoa_gb300.so")
_lib = None


class AlignmentType:
    kSW = 0  # Smith-Waterman (local)
    kNW = 1  # Needleman-Wunsch (global)
    kOV = 2  # overlap (semi-global)


class AlignmentSubtype:
    kLinear = 0
    kAffine = 1
    kConvex = 2


OK = 0
NO_NODE = 0xFFFFFFFF  # subgraph_to_graph entry past the subgraph's nodes
_MESSAGES = {
    1: "invalid argument",
    2: "too large sequence!",
    3: "possible overflow!",
    4: "insufficient memory!",
    5: "invalid alignment",
    6: "missing sequence in alignment",
    7: "sequence and weights are of unequal size!",
    8: "device arena capacity exceeded",
    9: "traceback did not terminate",
    10: "CUDA error",
    11: "a read needs 32-bit scores",
    12: "timed out",
}


class SpoaError(ValueError):
    """Raised where spoa throws std::invalid_argument; .status holds the code."""

    def __init__(self, where: str, status: int, detail: str | None = None):
        self.status = status
        msg = detail or _MESSAGES.get(status, f"status {status}")
        super().__init__(f"[spoa::{where}] error: {msg}")


class _BatchDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("m", C.c_int8), ("n", C.c_int8), ("g", C.c_int8),
                ("e", C.c_int8), ("q", C.c_int8), ("c", C.c_int8), ("pad", C.c_int8),
                ("n_windows", C.c_uint32), ("window_read_off", C.c_void_p),
                ("window_type", C.c_void_p), ("window_strand", C.c_void_p),
                ("seqs", C.c_void_p), ("seq_off", C.c_void_p), ("quals", C.c_void_p),
                ("max_nodes", C.c_uint32), ("threads_per_window", C.c_int32),
                ("columns_per_thread", C.c_int32), ("ctas", C.c_int32),
                ("memory_budget", C.c_uint64), ("want_alignments", C.c_int32),
                ("want_msa", C.c_int32), ("autotune", C.c_int32),
                ("windows_per_cta", C.c_int32), ("cluster", C.c_int32),
                ("device_set", C.c_int32), ("device", C.c_int32)]


class _BatchResult(C.Structure):
    _fields_ = [("read_scores", C.c_void_p), ("read_reversed", C.c_void_p),
                ("window_status", C.c_void_p), ("consensus", C.c_void_p),
                ("consensus_off", C.c_void_p), ("alignments", C.c_void_p),
                ("alignment_off", C.c_void_p), ("msa", C.c_void_p), ("msa_off", C.c_void_p),
                ("msa_rows", C.c_void_p), ("msa_cols", C.c_void_p), ("cells", C.c_uint64),
                ("pred_cells", C.c_uint64),
                ("kernel_ms", C.c_double), ("threads_per_window", C.c_int32),
                ("columns_per_thread", C.c_int32), ("ctas", C.c_int32),
                ("launches", C.c_int32)]


class _ServerDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("m", C.c_int8), ("n", C.c_int8), ("g", C.c_int8),
                ("e", C.c_int8), ("q", C.c_int8), ("c", C.c_int8), ("pad", C.c_int8),
                ("memory_budget", C.c_uint64), ("max_streams", C.c_int32),
                ("max_windows_per_launch", C.c_int32), ("gather_seconds", C.c_double),
                ("device_set", C.c_int32), ("device", C.c_int32), ("resident", C.c_int32)]


# Every symbol of include/spoa_gb300.h
EXPORTED = [
    "spoa_gb300_status_string", "spoa_gb300_device_count", "spoa_gb300_engine_create",
    "spoa_gb300_engine_destroy", "spoa_gb300_engine_params", "spoa_gb300_engine_prealloc",
    "spoa_gb300_engine_align", "spoa_gb300_graph_create", "spoa_gb300_graph_destroy",
    "spoa_gb300_graph_clear", "spoa_gb300_graph_add_alignment",
    "spoa_gb300_graph_add_alignment_quality", "spoa_gb300_align_add",
    "spoa_gb300_align_add_reads",
    "spoa_gb300_graph_consensus", "spoa_gb300_graph_msa", "spoa_gb300_graph_counts",
    "spoa_gb300_graph_export", "spoa_gb300_graph_gfa", "spoa_gb300_graph_subgraph",
    "spoa_gb300_graph_save",
    "spoa_gb300_graph_load", "spoa_gb300_batch_create",
    "spoa_gb300_batch_launch",
    "spoa_gb300_batch_launch_plain", "spoa_gb300_batch_fetch", "spoa_gb300_batch_destroy",
    "spoa_gb300_batch_run", "spoa_gb300_server_create", "spoa_gb300_server_submit",
    "spoa_gb300_server_wait", "spoa_gb300_server_stats", "spoa_gb300_server_resident_stats",
    "spoa_gb300_server_destroy",
    "spoa_gb300_window_poa_noalloc",
]


def lib():
    """Loads the CUDA library (building it when the sources are newer)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -m spoa_gb300.build` "
                "(the GPU path has no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        P, I32, U32, U64 = C.c_void_p, C.c_int32, C.c_uint32, C.c_uint64
        L.spoa_gb300_status_string.restype = C.c_char_p
        L.spoa_gb300_status_string.argtypes = [I32]
        L.spoa_gb300_engine_create.argtypes = [I32] + [C.c_int8] * 6 + [P]
        L.spoa_gb300_engine_destroy.argtypes = [P]
        L.spoa_gb300_engine_destroy.restype = None
        L.spoa_gb300_engine_params.argtypes = [P, P, P, P]
        L.spoa_gb300_engine_prealloc.argtypes = [P, U32, C.c_uint8]
        L.spoa_gb300_engine_align.argtypes = [P, C.c_char_p, U32, P, P, P, P, U32, P]
        L.spoa_gb300_graph_create.argtypes = [P]
        L.spoa_gb300_graph_destroy.argtypes = [P]
        L.spoa_gb300_graph_destroy.restype = None
        L.spoa_gb300_graph_clear.argtypes = [P]
        L.spoa_gb300_graph_add_alignment.argtypes = [P, P, U32, C.c_char_p, U32, P, U32]
        L.spoa_gb300_graph_add_alignment_quality.argtypes = [P, P, U32, C.c_char_p, U32,
                                                             C.c_char_p, U32]
        L.spoa_gb300_align_add.argtypes = [P, P, C.c_char_p, U32, C.c_char_p, I32, P, P]
        L.spoa_gb300_align_add_reads.argtypes = [P, P, U32, C.c_char_p, P, C.c_char_p, I32, P,
                                                 P, P]
        L.spoa_gb300_graph_consensus.argtypes = [P, C.c_char_p, U32, P]
        L.spoa_gb300_graph_msa.argtypes = [P, I32, C.c_char_p, U64, P, P]
        L.spoa_gb300_graph_counts.argtypes = [P] * 7
        L.spoa_gb300_graph_export.argtypes = [P] * 19
        L.spoa_gb300_graph_subgraph.argtypes = [P, U32, U32, P, P, U32]
        L.spoa_gb300_graph_gfa.argtypes = [P, P, P, I32, C.c_char_p, U64, P]
        L.spoa_gb300_graph_save.argtypes = [P, P, U64, P]
        L.spoa_gb300_graph_load.argtypes = [P, P, U64]
        L.spoa_gb300_batch_create.argtypes = [C.POINTER(_BatchDesc), P]
        L.spoa_gb300_batch_launch.argtypes = [P, P]
        L.spoa_gb300_batch_launch_plain.argtypes = [P, P]
        L.spoa_gb300_batch_fetch.argtypes = [P, C.POINTER(_BatchResult)]
        L.spoa_gb300_batch_destroy.argtypes = [P]
        L.spoa_gb300_batch_destroy.restype = None
        L.spoa_gb300_batch_run.argtypes = [C.POINTER(_BatchDesc), P, C.POINTER(_BatchResult)]
        L.spoa_gb300_window_poa_noalloc.argtypes = [I32] + [C.c_int8] * 6 + [I32, U32, U32, P, P,
                                                                              P, P, U32, P, P, P, P]
        L.spoa_gb300_server_create.argtypes = [C.POINTER(_ServerDesc), P]
        L.spoa_gb300_server_submit.argtypes = [P, C.c_char_p, P, U32, I32, I32, C.c_double, P]
        L.spoa_gb300_server_wait.argtypes = [P, U64, C.c_double, C.c_char_p, U32, P, P, P]
        L.spoa_gb300_server_stats.argtypes = [P, P, P]
        L.spoa_gb300_server_resident_stats.argtypes = [P, P, P]
        L.spoa_gb300_server_destroy.argtypes = [P]
        L.spoa_gb300_server_destroy.restype = None
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _check(where: str, st: int):
    if st != OK:
        raise SpoaError(where, st)


def _bytes(s) -> bytes:
    return s.encode() if isinstance(s, str) else bytes(s)


class AlignmentEngine:
    """spoa::AlignmentEngine backed by the GPU (alignment_engine.hpp:31-94)."""

    def __init__(self, handle):
        self._h = handle

    @staticmethod
    def create(type_: int, m: int, n: int, g: int, e: int | None = None,
               q: int | None = None, c: int | None = None) -> "AlignmentEngine":
        # the three overloads of AlignmentEngine::Create (alignment_engine.cpp:15-30)
        if e is None:
            e = g
        if q is None or c is None:
            q, c = g, e
        h = C.c_void_p()
        st = lib().spoa_gb300_engine_create(type_, m, n, g, e, q, c, C.byref(h))
        if st == 1:
            if type_ not in (0, 1, 2):
                raise SpoaError("AlignmentEngine::Create", st, "invalid alignment type!")
            if g > 0 or q > 0:
                raise SpoaError("AlignmentEngine::Create", st,
                                "gap opening penalty must be non-positive!")
            raise SpoaError("AlignmentEngine::Create", st,
                            "gap extension penalty must be non-positive!")
        _check("AlignmentEngine::Create", st)
        return AlignmentEngine(h)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.spoa_gb300_engine_destroy(self._h)
            self._h = None

    @property
    def params(self):
        t, s = C.c_int32(), C.c_int32()
        p = (C.c_int8 * 6)()
        lib().spoa_gb300_engine_params(self._h, C.byref(t), C.byref(s), p)
        return t.value, s.value, tuple(p)

    @property
    def subtype(self) -> int:
        return self.params[1]

    def prealloc(self, max_sequence_len: int, alphabet_size: int = 4):
        st = lib().spoa_gb300_engine_prealloc(self._h, max_sequence_len, alphabet_size)
        _check("AlignmentEngine::Prealloc", st)

    def align(self, sequence, graph: "Graph"):
        """Returns (alignment as an (n, 2) int32 array, score or None when the
        reference leaves the score untouched)."""
        s = _bytes(sequence)
        cap = graph.num_nodes + len(s) + 16
        pairs = np.zeros(2 * cap, np.int32)
        score, written = C.c_int32(0), C.c_int32(0)
        n = C.c_uint32()
        st = lib().spoa_gb300_engine_align(self._h, s, len(s), graph._h, C.byref(score),
                                           C.byref(written), _ptr(pairs), cap, C.byref(n))
        _check("AlignmentEngine::Align", st)
        return pairs[:2 * n.value].reshape(-1, 2).copy(), (score.value if written.value else None)


class Graph:
    """spoa::Graph kept in device memory (graph.hpp:25-318)."""

    def __init__(self):
        h = C.c_void_p()
        _check("Graph::Graph", lib().spoa_gb300_graph_create(C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.spoa_gb300_graph_destroy(self._h)
            self._h = None

    def counts(self) -> dict:
        v = [C.c_uint32() for _ in range(6)]
        lib().spoa_gb300_graph_counts(self._h, *[C.byref(x) for x in v])
        keys = ("nodes", "edges", "sequences", "consensus", "labels", "num_codes")
        return {k: x.value for k, x in zip(keys, v)}

    @property
    def num_nodes(self) -> int:
        return self.counts()["nodes"]

    def clear(self):
        _check("Graph::Clear", lib().spoa_gb300_graph_clear(self._h))

    def add_alignment(self, alignment, sequence, weights=1):
        """weights: an int (every base), a list of per-base weights or a
        quality string (Phred+33)."""
        s = _bytes(sequence)
        a = np.ascontiguousarray(np.asarray(alignment, np.int32).reshape(-1, 2))
        if isinstance(weights, (str, bytes)):
            qv = _bytes(weights)
            st = lib().spoa_gb300_graph_add_alignment_quality(self._h, _ptr(a), a.shape[0], s,
                                                              len(s), qv, len(qv))
        else:
            if isinstance(weights, int):
                w = np.full(len(s), weights, np.uint32)
            else:
                w = np.ascontiguousarray(np.asarray(weights, np.uint32))
            st = lib().spoa_gb300_graph_add_alignment(self._h, _ptr(a), a.shape[0], s, len(s),
                                                      _ptr(w) if w.size else None, w.size)
        _check("Graph::AddAlignment", st)

    def generate_consensus(self) -> str:
        n = self.num_nodes
        buf = C.create_string_buffer(max(n, 1))
        ln = C.c_uint32()
        _check("Graph::GenerateConsensus",
               lib().spoa_gb300_graph_consensus(self._h, buf, max(n, 1), C.byref(ln)))
        return buf.raw[:ln.value].decode()

    def generate_multiple_sequence_alignment(self, include_consensus: bool = False) -> list:
        cnt = self.counts()
        cap = (cnt["sequences"] + 1) * max(cnt["nodes"], 1)
        buf = C.create_string_buffer(cap)
        rows, cols = C.c_uint32(), C.c_uint32()
        _check("Graph::GenerateMultipleSequenceAlignment",
               lib().spoa_gb300_graph_msa(self._h, 1 if include_consensus else 0, buf, cap,
                                          C.byref(rows), C.byref(cols)))
        raw = buf.raw
        return [raw[k * cols.value:(k + 1) * cols.value].decode() for k in range(rows.value)]

    def export(self) -> dict:
        """Flat arrays behind nodes()/edges()/rank_to_node()/sequences()/consensus()."""
        cnt = self.counts()
        N, E, S, Cn, Lb = (cnt["nodes"], cnt["edges"], cnt["sequences"], cnt["consensus"],
                           cnt["labels"])
        z = lambda k, t: np.zeros(max(k, 1), t)  # noqa: E731
        chars, codes = z(N, np.uint8), z(N, np.uint8)
        in_off, in_e, out_off, out_e = z(N + 1, np.uint32), z(E, np.uint32), z(N + 1, np.uint32), z(E, np.uint32)
        al_off, al_n = z(N + 1, np.uint32), z(N * 64, np.uint32)
        et, eh, ew = z(E, np.uint32), z(E, np.uint32), z(E, np.int64)
        lab_off, labs = z(E + 1, np.uint32), z(Lb, np.uint32)
        rank, sb, cons = z(N, np.uint32), z(S, np.uint32), z(Cn, np.uint32)
        coder, decoder = np.zeros(256, np.int32), np.zeros(256, np.int32)
        arrs = [chars, codes, in_off, in_e, out_off, out_e, al_off, al_n, et, eh, ew, lab_off,
                labs, rank, sb, cons, coder, decoder]
        _check("Graph::export", lib().spoa_gb300_graph_export(self._h, *[_ptr(a) for a in arrs]))
        return {"chars": chars[:N], "codes": codes[:N], "in_off": in_off[:N + 1],
                "in_edges": in_e[:E], "out_off": out_off[:N + 1], "out_edges": out_e[:E],
                "aligned_off": al_off[:N + 1], "aligned": al_n[:al_off[N] if N else 0],
                "edge_tail": et[:E], "edge_head": eh[:E], "edge_weight": ew[:E],
                "label_off": lab_off[:E + 1], "labels": labs[:Lb], "rank_to_node": rank[:N],
                "seq_begin": sb[:S], "consensus": cons[:Cn], "coder": coder,
                "decoder": decoder, "num_codes": cnt["num_codes"]}

    def subgraph(self, begin: int, end: int):
        """Graph::Subgraph (graph.cpp:518-595): the part of the graph that
        reaches node `end` over in-edges and aligned nodes without going
        below node id `begin`, as a new device graph, and subgraph_to_graph
        (uint32, one entry per node of this graph: the id here of each
        subgraph node, then NO_NODE)."""
        sub = Graph()
        m = np.zeros(max(self.num_nodes, 1), np.uint32)
        _check("Graph::Subgraph", lib().spoa_gb300_graph_subgraph(
            self._h, begin, end, sub._h, _ptr(m), m.size))
        return sub, m[:self.num_nodes]

    def save(self) -> bytes:
        """The graph as bytes (the fields the reference's cereal
        serialisation archives, include/spoa/graph.hpp:187-233, in this
        library's own layout)."""
        n = C.c_uint64()
        _check("Graph::save", lib().spoa_gb300_graph_save(self._h, None, 0, C.byref(n)))
        buf = np.zeros(max(n.value, 1), np.uint8)
        _check("Graph::save", lib().spoa_gb300_graph_save(self._h, _ptr(buf), buf.size,
                                                          C.byref(n)))
        return buf[:n.value].tobytes()

    def load(self, data: bytes) -> "Graph":
        """Replaces this graph by one saved with save(), rebuilt the way the
        reference's Graph::load rebuilds it (graph.hpp:236-275)."""
        buf = np.frombuffer(bytes(data), np.uint8)
        _check("Graph::load", lib().spoa_gb300_graph_load(
            self._h, _ptr(np.ascontiguousarray(buf)) if buf.size else None, buf.size))
        return self

    @staticmethod
    def update_alignment(subgraph_to_graph, alignment):
        """Graph::UpdateAlignment (graph.cpp:597-605): node ids of an
        alignment against a subgraph mapped back to this graph's."""
        a = np.array(alignment, np.int32).reshape(-1, 2)
        m = np.asarray(subgraph_to_graph, np.uint32)
        hit = a[:, 0] != -1
        a[hit, 0] = m[a[hit, 0]].astype(np.int32)
        return a

    def paths(self, ex: dict | None = None) -> list:
        """Node path of every sequence (Node::Successor walks, graph.cpp:22-30)."""
        ex = ex or self.export()
        out_off, out_e = ex["out_off"], ex["out_edges"]
        lab_off, labs, heads = ex["label_off"], ex["labels"], ex["edge_head"]
        res = []
        for s, b in enumerate(ex["seq_begin"]):
            path, it = [], int(b)
            while it >= 0:
                path.append(it)
                nxt = -1
                for k in range(out_off[it], out_off[it + 1]):
                    e = out_e[k]
                    if s in labs[lab_off[e]:lab_off[e + 1]]:
                        nxt = int(heads[e])
                        break
                it = nxt
            res.append(np.array(path, np.uint32))
        return res

    def gfa_text(self, is_reversed=None, headers=None, include_consensus=True) -> str:
        """The same GFA as gfa(), written by the library
        (spoa_gb300_graph_gfa) into one string."""
        names = None
        if headers is not None:
            enc = [h.encode() if isinstance(h, str) else bytes(h) for h in headers]
            names = (C.c_char_p * len(enc))(*enc)
        rev = (np.ascontiguousarray(np.asarray(is_reversed, np.uint8))
               if is_reversed is not None and len(is_reversed) else None)
        n = C.c_uint64()
        args = (self._h, names, _ptr(rev) if rev is not None else None,
                1 if include_consensus else 0)
        _check("Graph::gfa", lib().spoa_gb300_graph_gfa(*args, None, 0, C.byref(n)))
        buf = C.create_string_buffer(max(n.value, 1))
        _check("Graph::gfa", lib().spoa_gb300_graph_gfa(*args, buf, n.value, C.byref(n)))
        return buf.raw[:n.value].decode()

    def gfa(self, is_reversed=None, headers=None, include_consensus=True) -> list:
        """GFA lines in the layout of spoa's CLI writer (src/main.cpp:119-199);
        the consensus must have been generated."""
        from .gfa import gfa_lines
        ex = self.export()
        out_e = ex["out_edges"]  # node-major, insertion order within a node
        return gfa_lines(ex["chars"], ex["edge_tail"][out_e], ex["edge_head"][out_e],
                         ex["edge_weight"][out_e], self.paths(ex), ex["consensus"], is_reversed,
                         headers, include_consensus)


def align_add_reads(engine: AlignmentEngine, graph: Graph, reads, quals=None,
                    strand_ambiguous: bool = False):
    """The per-read Align + AddAlignment loop over `reads`, recorded into one
    CUDA graph (include/spoa_gb300.h).  Returns (scores, reversed)."""
    rs = [_bytes(r) for r in reads]
    off = np.zeros(len(rs) + 1, np.uint64)
    off[1:] = np.cumsum([len(r) for r in rs])
    qs = b"".join(_bytes(q) for q in quals) if quals is not None else None
    scores = np.zeros(max(len(rs), 1), np.int32)
    rev = np.zeros(max(len(rs), 1), np.int32)
    done = C.c_uint32()
    st = lib().spoa_gb300_align_add_reads(engine._h, graph._h, len(rs), b"".join(rs), _ptr(off),
                                          qs, 1 if strand_ambiguous else 0, _ptr(scores),
                                          _ptr(rev), C.byref(done))
    _check("AlignmentEngine::Align", st)
    return scores[:len(rs)].tolist(), [bool(x) for x in rev[:len(rs)]]


def align_add(engine: AlignmentEngine, graph: Graph, sequence, quality=None,
              strand_ambiguous: bool = False):
    """Align + AddAlignment of one read on the device (src/main.cpp:275-314).
    Returns (score, reversed)."""
    s = _bytes(sequence)
    q = _bytes(quality) if quality is not None else None
    score, rev = C.c_int32(), C.c_int32()
    st = lib().spoa_gb300_align_add(engine._h, graph._h, s, len(s), q,
                                    1 if strand_ambiguous else 0, C.byref(score), C.byref(rev))
    _check("AlignmentEngine::Align", st)
    return score.value, bool(rev.value)


@dataclass
class BatchResult:
    consensus: list
    scores: np.ndarray
    reversed: np.ndarray
    status: np.ndarray
    cells: int
    pred_cells: int
    kernel_ms: float
    threads_per_window: int
    columns_per_thread: int
    ctas: int
    launches: int
    alignments: list | None = None
    msa: list | None = None


class Batch:
    """Many windows in one persistent kernel (spoa_gb300_batch_*)."""

    def __init__(self, windows, type_: int, m: int, n: int, g: int, e: int, q: int, c: int,
                 window_types=None, window_strand=None, quals=None, **kw):
        reads = [_bytes(r) for w in windows for r in w]
        wro = np.zeros(len(windows) + 1, np.uint32)
        wro[1:] = np.cumsum([len(w) for w in windows])
        off = np.zeros(len(reads) + 1, np.uint64)
        off[1:] = np.cumsum([len(r) for r in reads])
        seqs = np.frombuffer(b"".join(reads) + b"\0", np.uint8)
        qarr = (np.frombuffer(b"".join(_bytes(x) for w in quals for x in w) + b"\0", np.uint8)
                if quals is not None else None)
        self._create(seqs, off, wro, type_, m, n, g, e, q, c, window_types, window_strand, qarr,
                     **kw)

    @classmethod
    def from_arrays(cls, seqs, seq_off, window_read_off, type_, m, n, g, e, q, c,
                    window_types=None, window_strand=None, quals=None, **kw) -> "Batch":
        """Batch over already flattened inputs: seqs (uint8, reads back to
        back), seq_off (uint64, n_reads + 1), window_read_off (uint32,
        n_windows + 1); quals shares seq_off."""
        b = cls.__new__(cls)
        b._create(seqs, seq_off, window_read_off, type_, m, n, g, e, q, c, window_types,
                  window_strand, quals, **kw)
        return b

    def _create(self, seqs, off, wro, type_, m, n, g, e, q, c, window_types, window_strand,
                quals, want_alignments=False, want_msa=False, threads_per_window=0,
                columns_per_thread=0, ctas=0, max_nodes=0, memory_budget=0, autotune=False,
                windows_per_cta=1, device=None, cluster=0):
        self._seqs = np.ascontiguousarray(seqs, np.uint8)
        self._off = np.ascontiguousarray(off, np.uint64)
        self._wro = np.ascontiguousarray(wro, np.uint32)
        self._quals = np.ascontiguousarray(quals, np.uint8) if quals is not None else None
        self.n_windows = int(self._wro.size - 1)
        self.n_reads = int(self._off.size - 1)
        self._wt = np.asarray(window_types, np.int8) if window_types is not None else None
        self._ws = np.asarray(window_strand, np.int8) if window_strand is not None else None
        g_ = g
        e_ = e if e is not None else g
        self.subtype = (AlignmentSubtype.kLinear if g_ >= e_ else
                        (AlignmentSubtype.kAffine if (g_ <= q or e_ >= c)
                         else AlignmentSubtype.kConvex))
        d = _BatchDesc()
        d.type, d.m, d.n, d.g, d.e, d.q, d.c = type_, m, n, g, e, q, c
        d.n_windows = self.n_windows
        d.window_read_off = _ptr(self._wro).value
        d.window_type = _ptr(self._wt).value if self._wt is not None else None
        d.window_strand = _ptr(self._ws).value if self._ws is not None else None
        d.seqs = _ptr(self._seqs).value
        d.seq_off = _ptr(self._off).value
        d.quals = _ptr(self._quals).value if self._quals is not None else None
        d.max_nodes = max_nodes
        d.threads_per_window = threads_per_window
        d.columns_per_thread = columns_per_thread
        d.ctas = ctas
        d.memory_budget = memory_budget
        d.want_alignments = 1 if want_alignments else 0
        d.want_msa = 1 if want_msa else 0
        d.autotune = 1 if autotune else 0
        d.windows_per_cta = windows_per_cta
        d.cluster = cluster
        d.device_set = 1 if device is not None else 0
        d.device = int(device) if device is not None else 0
        self._desc = d
        h = C.c_void_p()
        _check("batch_create", lib().spoa_gb300_batch_create(C.byref(d), C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.spoa_gb300_batch_destroy(self._h)
            self._h = None

    def launch(self, stream: int = 0):
        _check("batch_launch", lib().spoa_gb300_batch_launch(self._h, C.c_void_p(stream)))

    def launch_plain(self, stream: int = 0):
        _check("batch_launch_plain",
               lib().spoa_gb300_batch_launch_plain(self._h, C.c_void_p(stream)))

    def fetch(self) -> BatchResult:
        r = _BatchResult()
        _check("batch_fetch", lib().spoa_gb300_batch_fetch(self._h, C.byref(r)))
        W, R = self.n_windows, self.n_reads

        def arr(p, t, k):
            if not p or k == 0:
                return np.zeros(0, t)
            return np.ctypeslib.as_array(C.cast(p, C.POINTER(np.ctypeslib.as_ctypes_type(t))),
                                         shape=(k,)).copy()

        coff = arr(r.consensus_off, np.uint64, W + 1)
        craw = C.string_at(r.consensus, int(coff[-1])) if W else b""
        cons = [craw[int(coff[w]):int(coff[w + 1])].decode() for w in range(W)]
        res = BatchResult(consensus=cons, scores=arr(r.read_scores, np.int32, R),
                          reversed=arr(r.read_reversed, np.uint8, R),
                          status=arr(r.window_status, np.int32, W), cells=r.cells,
                          pred_cells=r.pred_cells,
                          kernel_ms=r.kernel_ms, threads_per_window=r.threads_per_window,
                          columns_per_thread=r.columns_per_thread, ctas=r.ctas,
                          launches=r.launches)
        if self._desc.want_alignments:
            aoff = arr(r.alignment_off, np.uint64, R + 1)
            allp = arr(r.alignments, np.int32, 2 * int(aoff[-1])) if R else np.zeros(0, np.int32)
            res.alignments = [allp[2 * int(aoff[k]):2 * int(aoff[k + 1])].reshape(-1, 2)
                              for k in range(R)]
        if self._desc.want_msa:
            moff = arr(r.msa_off, np.uint64, W + 1)
            rows = arr(r.msa_rows, np.uint32, W)
            cols = arr(r.msa_cols, np.uint32, W)
            raw = C.string_at(r.msa, int(moff[-1])) if W else b""
            res.msa = []
            for w in range(W):
                base = int(moff[w])
                res.msa.append([raw[base + k * int(cols[w]):base + (k + 1) * int(cols[w])].decode()
                                for k in range(int(rows[w]))])
        return res


def batch_poa(windows, type_: int, m: int, n: int, g: int, e: int | None = None,
              q: int | None = None, c: int | None = None, **kw) -> BatchResult:
    """Runs every window (list of reads) through the persistent kernel."""
    if e is None:
        e = g
    if q is None or c is None:
        q, c = g, e
    b = Batch(windows, type_, m, n, g, e, q, c, **kw)
    b.launch()
    return b.fetch()


TIMEOUT = 12


class Server:
    """Served windows (continuous batching, include/spoa_gb300.h): submit
    windows as they arrive, wait for each one's consensus.  Each window is the
    per-read loop of spoa's CLI (src/main.cpp:275-314) and GenerateConsensus."""

    def __init__(self, type_: int, m: int, n: int, g: int, e: int | None = None,
                 q: int | None = None, c: int | None = None, memory_budget: int = 0,
                 max_streams: int = 0, max_windows_per_launch: int = 0,
                 gather_seconds: float = 0.0, device: int | None = None,
                 resident: bool = False):
        e = g if e is None else e
        if q is None or c is None:
            q, c = g, e
        d = _ServerDesc(type_, m, n, g, e, q, c, 0, memory_budget, max_streams,
                        max_windows_per_launch, gather_seconds,
                        1 if device is not None else 0, int(device or 0), 1 if resident else 0)
        h = C.c_void_p()
        _check("Server::Create", lib().spoa_gb300_server_create(C.byref(d), C.byref(h)))
        self._h = h

    def submit(self, reads, type_: int = -1, strand_ambiguous: bool = False,
               delay: float = 0.0) -> int:
        """Queues one window (a list of reads); it counts as arrived `delay`
        seconds from now.  Returns its ticket."""
        rs = [_bytes(r) for r in reads]
        off = np.zeros(len(rs) + 1, np.uint64)
        off[1:] = np.cumsum([len(r) for r in rs])
        t = C.c_uint64()
        _check("Server::Submit", lib().spoa_gb300_server_submit(
            self._h, b"".join(rs), _ptr(off), len(rs), type_, 1 if strand_ambiguous else 0,
            float(delay), C.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout: float = 0.0):
        """(status, consensus, latency seconds) of a submitted window."""
        cap = 1 << 20
        buf = C.create_string_buffer(cap)
        n, st, lat = C.c_uint32(), C.c_int32(), C.c_double()
        r = lib().spoa_gb300_server_wait(self._h, ticket, float(timeout), buf, cap, C.byref(n),
                                         C.byref(st), C.byref(lat))
        _check("Server::Wait", r)
        if n.value > cap:
            raise SpoaError("Server::Wait", 8, "consensus longer than the buffer")
        return st.value, buf.raw[:n.value].decode(), lat.value

    def stats(self):
        la, co = C.c_uint64(), C.c_uint64()
        _check("Server::Stats", lib().spoa_gb300_server_stats(self._h, C.byref(la), C.byref(co)))
        rw, rl = C.c_uint64(), C.c_uint64()
        _check("Server::Stats",
               lib().spoa_gb300_server_resident_stats(self._h, C.byref(rw), C.byref(rl)))
        return {"launches": la.value, "completed": co.value, "resident_windows": rw.value,
                "resident_launches": rl.value}

    def close(self):
        if getattr(self, "_h", None):
            lib().spoa_gb300_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
