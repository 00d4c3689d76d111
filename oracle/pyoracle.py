"""ctypes binding of the C oracle (oracle/spoa_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py.  The product package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_REF_DRIVER = os.path.join(_HERE, "_ref", "spoa_ref_driver")
_REF_BENCH = os.path.join(_HERE, "_ref", "spoa_ref_bench")
# the reference's library sources, staged (unmodified, git-ignored) so they
# travel to machines without the reference tree
_STAGED = os.path.join(os.path.dirname(_HERE), "baseline", "_ref", "spoa")
_lib = None

TYPES = {"SW": 0, "NW": 1, "OV": 2}


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "spoa_oracle.c"))
    ):
        subprocess.run(["make", "-s", "-C", _HERE, "all"], check=True)
    return _LIB_PATH


def reference_tree() -> str:
    """The reference source tree: $SPOA_REFERENCE_TREE, else the directory
    `reference` beside this repository."""
    return os.environ.get("SPOA_REFERENCE_TREE",
                          os.path.join(os.path.dirname(os.path.dirname(_HERE)), "reference"))


def build_reference() -> str | None:
    """Where the reference tree is present: compile the reference driver and
    stage the reference's library sources for the CPU baseline.  Wherever a
    staged copy exists (here, or on a machine the repository was copied to):
    compile the baseline timer from it.  Returns the driver or None."""
    ref = reference_tree()
    if os.path.isdir(os.path.join(ref, "src")):
        subprocess.run(["make", "-s", "-C", _HERE, "ref", "stage", f"REF={ref}"], check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    if os.path.isdir(os.path.join(_STAGED, "src")):
        subprocess.run(["make", "-s", "-C", _HERE, "bench"], check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return _REF_DRIVER if os.path.exists(_REF_DRIVER) else None


def reference_driver() -> str | None:
    return _REF_DRIVER if os.path.exists(_REF_DRIVER) else None


def reference_bench() -> str | None:
    """The timer of the reference's own library (oracle/ref_bench.cpp)."""
    return _REF_BENCH if os.path.exists(_REF_BENCH) else None


def write_windows_file(path: str, windows, types, strands) -> None:
    """Windows in the input format of ref_bench.cpp."""
    import struct
    with open(path, "wb") as fh:
        fh.write(b"SPWB" + struct.pack("<I", len(windows)))
        for reads, t, s in zip(windows, types, strands):
            fh.write(struct.pack("<bbHI", int(t), 1 if s else 0, 0, len(reads)))
            fh.write(np.asarray([len(r) for r in reads], np.uint32).tobytes())
            fh.write(b"".join(reads))


def run_reference_bench(windows, types, strands, params, threads: int,
                        want_consensus: bool = False) -> dict:
    """Times the reference library on `threads` host threads over the
    windows (one window per task).  Returns the timer's JSON record, plus
    the consensus list when asked."""
    import json
    import tempfile
    exe = reference_bench()
    if exe is None:
        raise FileNotFoundError("reference timer not built")
    with tempfile.TemporaryDirectory() as tmp:
        inp = os.path.join(tmp, "windows.bin")
        write_windows_file(inp, windows, types, strands)
        out = os.path.join(tmp, "consensus.txt")
        cmd = [exe, inp] + [str(int(x)) for x in params] + [str(threads)]
        if want_consensus:
            cmd.append(out)
        r = subprocess.run(cmd, capture_output=True, text=True, check=True)
        rec = json.loads(r.stdout.strip().splitlines()[-1])
        if want_consensus:
            with open(out) as fh:
                rec["consensus"] = fh.read().split("\n")[:len(windows)]
    return rec


class WindowParams(C.Structure):
    _fields_ = [("type", C.c_int32), ("m", C.c_int8), ("n", C.c_int8),
                ("g", C.c_int8), ("e", C.c_int8), ("q", C.c_int8),
                ("c", C.c_int8), ("strand_ambiguous", C.c_int8)]


def _sanitized_build() -> str:
    """liboracle built with AddressSanitizer and UndefinedBehaviorSanitizer
    (no recovery), for a process that preloads the ASan runtime; selected
    by SPOA_ORACLE_SANITIZE=1 so that the oracle's own tests can run under
    the sanitizers."""
    out = os.path.join(_HERE, "_build", "liboracle_asan.so")
    src = os.path.join(_HERE, "spoa_oracle.c")
    if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        os.makedirs(os.path.dirname(out), exist_ok=True)
        subprocess.run(["gcc", "-std=c11", "-O1", "-g", "-fPIC", "-shared",
                        "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
                        "-o", out, src, "-lpthread"], check=True)
    return out


def lib():
    global _lib
    if _lib is None:
        if os.environ.get("SPOA_ORACLE_SANITIZE") == "1":
            path = _sanitized_build()
        else:
            build()
            path = _LIB_PATH
        L = C.CDLL(path)
        P = C.c_void_p
        L.oracle_graph_create.restype = P
        L.oracle_graph_destroy.argtypes = [P]
        L.oracle_graph_clear.argtypes = [P]
        L.oracle_engine_create.restype = P
        L.oracle_engine_create.argtypes = [C.c_int32] + [C.c_int8] * 6 + [C.POINTER(C.c_int32)]
        L.oracle_engine_destroy.argtypes = [P]
        L.oracle_engine_subtype.argtypes = [P]
        L.oracle_align.argtypes = [P, C.c_char_p, C.c_uint32, P, C.POINTER(C.c_int32),
                                   P, C.c_uint32, C.POINTER(C.c_uint32)]
        L.oracle_add_alignment.argtypes = [P, P, C.c_uint32, C.c_char_p, C.c_uint32,
                                           P, C.c_uint32]
        L.oracle_consensus.argtypes = [P, C.c_char_p, C.c_uint32]
        L.oracle_consensus.restype = C.c_uint32
        L.oracle_msa.argtypes = [P, C.c_int32, C.c_char_p, C.c_uint64,
                                 C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        for fn in ("num_nodes", "num_edges", "num_sequences", "consensus_len"):
            f = getattr(L, f"oracle_graph_{fn}")
            f.argtypes = [P]
            f.restype = C.c_uint32
        L.oracle_graph_export.argtypes = [P] * 8
        L.oracle_graph_export_ids.argtypes = [P] * 6
        L.oracle_graph_export_ids.restype = C.c_uint32
        L.oracle_subgraph.argtypes = [P, C.c_uint32, C.c_uint32, P, P]
        L.oracle_graph_edge_labels.argtypes = [P, P, P]
        L.oracle_graph_edge_labels.restype = C.c_uint32
        L.oracle_graph_reload.argtypes = [P, P]
        L.oracle_graph_path.argtypes = [P, C.c_uint32, P, C.c_uint32]
        L.oracle_graph_path.restype = C.c_uint32
        L.oracle_window_run.argtypes = [C.POINTER(WindowParams), P, C.c_uint32, C.c_char_p,
                                        P, C.c_char_p, P, P, P, C.c_uint64, P]
        L.oracle_batch_run.argtypes = [C.POINTER(WindowParams), C.c_uint32, P, C.c_char_p,
                                       P, C.c_char_p, C.c_int32, C.c_char_p, C.c_uint64,
                                       P, P, P, P]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


@dataclass
class WindowResult:
    status: int
    scores: list = field(default_factory=list)
    reversed: list = field(default_factory=list)
    alignments: list = field(default_factory=list)  # list of (n, 2) int32 arrays
    consensus: str = ""
    msa: list = field(default_factory=list)
    graph: dict = field(default_factory=dict)


def export_graph(g) -> dict:
    """Node characters, rank order, out-edges in node-major order, sequence
    paths and consensus ids of an oracle graph."""
    L = lib()
    nn = L.oracle_graph_num_nodes(g)
    ne = L.oracle_graph_num_edges(g)
    ns = L.oracle_graph_num_sequences(g)
    nc = L.oracle_graph_consensus_len(g)
    chars = np.zeros(max(nn, 1), np.uint8)
    rank = np.zeros(max(nn, 1), np.uint32)
    et = np.zeros(max(ne, 1), np.uint32)
    eh = np.zeros(max(ne, 1), np.uint32)
    ew = np.zeros(max(ne, 1), np.int64)
    sb = np.zeros(max(ns, 1), np.uint32)
    cons = np.zeros(max(nc, 1), np.uint32)
    L.oracle_graph_export(g, _ptr(chars), _ptr(rank), _ptr(et), _ptr(eh), _ptr(ew),
                          _ptr(sb), _ptr(cons))
    paths = []
    buf = np.zeros(max(nn, 1), np.uint32)
    for s in range(ns):
        k = L.oracle_graph_path(g, s, _ptr(buf), buf.size)
        paths.append(buf[:k].copy())
    return {"chars": chars[:nn].copy(), "rank_to_node": rank[:nn].copy(),
            "edge_tail": et[:ne].copy(), "edge_head": eh[:ne].copy(),
            "edge_weight": ew[:ne].copy(), "seq_begin": sb[:ns].copy(),
            "consensus": cons[:nc].copy(), "paths": paths}


def run_window(type_: int, m: int, n: int, g: int, e: int, q: int, c: int,
               reads: list[bytes], quals: list[bytes] | None = None,
               strand_ambiguous: bool = False, with_msa: bool = True,
               with_graph: bool = False) -> WindowResult:
    """One window the way spoa's CLI runs it: align/add per read in order,
    then consensus and MSA."""
    L = lib()
    p = WindowParams(type_, m, n, g, e, q, c, 1 if strand_ambiguous else 0)
    seqs = b"".join(reads)
    off = np.zeros(len(reads) + 1, np.uint64)
    off[1:] = np.cumsum([len(r) for r in reads])
    qual_blob = b"".join(quals) if quals is not None else None
    nr = len(reads)
    scores = np.zeros(max(nr, 1), np.int32)
    rev = np.zeros(max(nr, 1), np.uint8)
    cap = int(sum(len(r) for r in reads) * 2 + 16) * (nr + 1) * 2
    cap = min(cap, 1 << 31)
    pairs = np.zeros(cap, np.int32)
    aoff = np.zeros(nr + 1, np.uint64)
    gr = L.oracle_graph_create()
    try:
        st = L.oracle_window_run(C.byref(p), gr, nr, seqs, _ptr(off), qual_blob,
                                 _ptr(scores), _ptr(rev), _ptr(pairs), cap, _ptr(aoff))
        res = WindowResult(status=st)
        if st != 0:
            return res
        res.scores = scores[:nr].tolist()
        res.reversed = rev[:nr].tolist()
        res.alignments = [pairs[2 * int(aoff[r]):2 * int(aoff[r + 1])].reshape(-1, 2).copy()
                          for r in range(nr)]
        nn = L.oracle_graph_num_nodes(gr)
        cbuf = C.create_string_buffer(nn + 1)
        k = L.oracle_consensus(gr, cbuf, nn + 1)
        res.consensus = cbuf.raw[:k].decode()
        if with_msa:
            rows = C.c_uint32()
            rl = C.c_uint32()
            mcap = (nr + 1) * (nn + 1)
            mbuf = C.create_string_buffer(mcap)
            st2 = L.oracle_msa(gr, 0, mbuf, mcap, C.byref(rows), C.byref(rl))
            assert st2 == 0
            raw = mbuf.raw
            res.msa = [raw[i * rl.value:(i + 1) * rl.value].decode() for i in range(rows.value)]
        if with_graph:
            res.graph = export_graph(gr)
        return res
    finally:
        L.oracle_graph_destroy(gr)


def batch_run(type_: int, m: int, n: int, g: int, e: int, q: int, c: int,
              windows: list[list[bytes]], strand_ambiguous: bool = False,
              n_threads: int | None = None, window_seconds: list | None = None):
    """Many windows on host threads (one window per task).  Returns
    (consensus list, matrix cells); window_seconds, when a list, gets each
    window's wall time on its thread."""
    L = lib()
    p = WindowParams(type_, m, n, g, e, q, c, 1 if strand_ambiguous else 0)
    reads = [r for w in windows for r in w]
    wro = np.zeros(len(windows) + 1, np.uint32)
    wro[1:] = np.cumsum([len(w) for w in windows])
    off = np.zeros(len(reads) + 1, np.uint64)
    off[1:] = np.cumsum([len(r) for r in reads])
    seqs = b"".join(reads)
    # consensus can exceed the longest read; give each window a generous slot
    slot = np.array([4 * max(len(r) for r in w) + 64 if w else 64 for w in windows],
                    np.uint64)
    coff = np.zeros(len(windows) + 1, np.uint64)
    coff[1:] = np.cumsum(slot)
    cons = C.create_string_buffer(int(coff[-1]) + 1)
    cells = C.c_uint64()
    scores = np.zeros(max(len(reads), 1), np.int32)
    secs = np.zeros(max(len(windows), 1), np.float64)
    st = L.oracle_batch_run(C.byref(p), len(windows), _ptr(wro), seqs, _ptr(off), None,
                            n_threads or os.cpu_count() or 1, cons, int(coff[-1]),
                            _ptr(coff), _ptr(scores), C.byref(cells), _ptr(secs))
    if window_seconds is not None:
        window_seconds.extend(secs[:len(windows)].tolist())
    if st != 0:
        raise RuntimeError(f"oracle batch failed with status {st}")
    raw = cons.raw
    out = []
    for w in range(len(windows)):
        seg = raw[int(coff[w]):int(coff[w + 1])]
        out.append(seg.split(b"\0", 1)[0].decode())
    return out, cells.value


def run_reference(windows_text: str, timing: bool = False) -> str:
    """Feed the reference driver a window description (see ref_driver.cpp)."""
    drv = reference_driver()
    if drv is None:
        raise FileNotFoundError("reference driver not built")
    args = [drv] + (["--time"] if timing else [])
    return subprocess.run(args, input=windows_text, capture_output=True, text=True,
                          check=True).stdout


def format_windows(specs) -> str:
    """specs: iterable of (type, (m, n, g, e, q, c), reads, quals|None, strand)."""
    out = []
    for typ, (m, n, g, e, q, c), reads, quals, strand in specs:
        hq = 1 if quals is not None else 0
        out.append(f"W {typ} {m} {n} {g} {e} {q} {c} {1 if strand else 0} {hq} {len(reads)}\n")
        for k, r in enumerate(reads):
            out.append(r.decode() + "\n")
            if hq:
                out.append(quals[k].decode() + "\n")
    return "".join(out)


def parse_reference_output(text: str) -> list:
    """Parse ref_driver output into a list of per-window dicts."""
    wins = []
    cur = None
    for line in text.split("\n"):
        if not line:
            continue
        tag, _, rest = line.partition(" ")
        if tag == "W":
            cur = {"scores": [], "reversed": [], "alignments": [], "consensus": "",
                   "msa": [], "gfa": [], "error": None, "summary": None,
                   "summary_verbose": None}
        elif tag == "R":
            parts = rest.split(" ")
            cur["scores"].append(int(parts[1]))
            cur["reversed"].append(int(parts[2]))
            npairs = int(parts[3])
            arr = np.array([[int(x) for x in p.split(",")] for p in parts[4:4 + npairs]],
                           np.int32).reshape(-1, 2)
            cur["alignments"].append(arr)
        elif tag == "C":
            cur["consensus"] = rest
        elif tag == "M":
            cur["msa"].append(rest)
        elif tag in ("Y", "V"):
            vals = [int(x) for x in rest.split(",")] if rest else []
            cur["summary" if tag == "Y" else "summary_verbose"] = vals
        elif tag == "G":
            cur["gfa"].append(rest)
        elif tag == "U":
            cur.setdefault("slices", []).append({"U": rest})
        elif tag in ("K", "O", "L", "A", "Q", "S"):
            # lines of the last subgraph (after a U line), else of the graph
            # as loaded (persisted windows)
            if cur.get("slices") and tag not in cur["slices"][-1] and tag != "S":
                cur["slices"][-1][tag] = rest
            else:
                cur.setdefault("loaded", {})[tag] = rest
        elif tag == "X":
            cur["error"] = rest
        elif tag == "E":
            wins.append(cur)
            cur = None
    return wins


# ---- slices: Graph::Subgraph + UpdateAlignment (graph.cpp:518-605) ---------

def format_slices(specs) -> str:
    """specs: iterable of (type, (m, n, g, e, q, c), reads, slices) with one
    (begin, end) per read after the first ((-1, -1): the whole graph)."""
    out = []
    for typ, (m, n, g, e, q, c), reads, slices in specs:
        out.append(f"S {typ} {m} {n} {g} {e} {q} {c} {len(reads)}\n")
        out.extend(r.decode() + "\n" for r in reads)
        out.extend(f"{b} {e_} \n" for b, e_ in slices)
    return "".join(out)


def slice_lines(read: int, sub_to_graph, chars, rank, edge_tail, edge_head, edge_weight,
                aligned_off, aligned, consensus: str) -> dict:
    """The U/K/O/L/A/Q lines of the reference driver for one subgraph, from
    its arrays (ids in subgraph numbering, edges in id order)."""
    n = len(chars)
    al = []
    for v in range(n):
        lst = aligned[aligned_off[v]:aligned_off[v + 1]]
        if len(lst):
            al.append(f"{v}:" + ",".join(str(int(x)) for x in lst))
    return {
        "U": f"{read} {n}" + "".join(f" {int(x)}" for x in sub_to_graph[:n]),
        "K": bytes(np.asarray(chars, np.uint8)).decode(),
        "O": " ".join(str(int(x)) for x in rank),
        "L": " ".join(f"{int(t)},{int(h)},{int(w)}"
                      for t, h, w in zip(edge_tail, edge_head, edge_weight)),
        "A": " ".join(al),
        "Q": consensus,
    }


def run_slices(type_: int, params, reads: list[bytes], slices) -> dict:
    """The slice protocol of ref_driver.cpp on the C oracle: read 0 added
    whole; every later read aligned to Subgraph(begin, end) (or the whole
    graph), its alignment mapped back (UpdateAlignment) and added."""
    L = lib()
    st = C.c_int32()
    en = L.oracle_engine_create(type_, *params, C.byref(st))
    if not en:
        raise RuntimeError(f"oracle engine: status {st.value}")
    g = L.oracle_graph_create()
    sub = L.oracle_graph_create()
    res = {"scores": [], "alignments": [], "slices": [], "consensus": "", "msa": []}
    try:
        for r, seq in enumerate(reads):
            w = np.ones(max(len(seq), 1), np.uint32)
            pairs = np.zeros(2 * (L.oracle_graph_num_nodes(g) + len(seq) + 16), np.int32)
            npairs = C.c_uint32(0)
            score = C.c_int32(0)
            if r > 0:
                b, e_ = slices[r - 1]
                target = g
                if b >= 0:
                    nn = L.oracle_graph_num_nodes(g)
                    m = np.zeros(max(nn, 1), np.uint32)
                    assert L.oracle_subgraph(g, b, e_, sub, _ptr(m)) == 0
                    target = sub
                assert L.oracle_align(en, seq, len(seq), target, C.byref(score), _ptr(pairs),
                                      pairs.size // 2, C.byref(npairs)) == 0
                aln = pairs[:2 * npairs.value].reshape(-1, 2).copy()
                if b >= 0:
                    sn = L.oracle_graph_num_nodes(sub)
                    se = L.oracle_graph_num_edges(sub)
                    chars = np.zeros(max(sn, 1), np.uint8)
                    rank = np.zeros(max(sn, 1), np.uint32)
                    L.oracle_graph_export(sub, _ptr(chars), _ptr(rank), None, None, None, None,
                                          None)
                    et, eh = np.zeros(max(se, 1), np.uint32), np.zeros(max(se, 1), np.uint32)
                    ew = np.zeros(max(se, 1), np.int64)
                    aoff = np.zeros(sn + 1, np.uint32)
                    na = L.oracle_graph_export_ids(sub, None, None, None, _ptr(aoff), None)
                    al = np.zeros(max(na, 1), np.uint32)
                    L.oracle_graph_export_ids(sub, _ptr(et), _ptr(eh), _ptr(ew), _ptr(aoff),
                                              _ptr(al))
                    cb = C.create_string_buffer(sn + 1)
                    k = L.oracle_consensus(sub, cb, sn + 1)
                    res["slices"].append(slice_lines(r, m, chars[:sn], rank[:sn], et[:se],
                                                     eh[:se], ew[:se], aoff, al,
                                                     cb.raw[:k].decode()))
                    hit = aln[:, 0] != -1
                    aln[hit, 0] = m[aln[hit, 0]].astype(np.int32)
                res["scores"].append(score.value)
                res["alignments"].append(aln)
            else:
                aln = np.zeros((0, 2), np.int32)
            assert L.oracle_add_alignment(g, _ptr(np.ascontiguousarray(aln)), aln.shape[0], seq,
                                          len(seq), _ptr(w), len(seq)) == 0
        nn = L.oracle_graph_num_nodes(g)
        cb = C.create_string_buffer(nn + 1)
        k = L.oracle_consensus(g, cb, nn + 1)
        res["consensus"] = cb.raw[:k].decode()
        rows, rl = C.c_uint32(), C.c_uint32()
        mcap = (len(reads) + 1) * (nn + 1)
        mb = C.create_string_buffer(mcap)
        assert L.oracle_msa(g, 0, mb, mcap, C.byref(rows), C.byref(rl)) == 0
        res["msa"] = [mb.raw[i * rl.value:(i + 1) * rl.value].decode()
                      for i in range(rows.value)]
        return res
    finally:
        L.oracle_graph_destroy(sub)
        L.oracle_graph_destroy(g)
        L.oracle_engine_destroy(en)


# ---- persisted windows: Graph::save / Graph::load (graph.hpp:187-276) -------

def format_persist(specs) -> str:
    """specs: iterable of (type, (m, n, g, e, q, c), reads, quals|None, split)."""
    out = []
    for typ, (m, n, g, e, q, c), reads, quals, split in specs:
        hq = 1 if quals is not None else 0
        out.append(f"P {typ} {m} {n} {g} {e} {q} {c} {hq} {len(reads)} {split}\n")
        for k, r in enumerate(reads):
            out.append(r.decode() + "\n")
            if hq:
                out.append(quals[k].decode() + "\n")
    return "".join(out)


def loaded_lines(chars, rank, seq_begin, consensus, edge_tail, edge_head, edge_weight,
                 label_off, labels, aligned_off, aligned) -> dict:
    """The K/O/S/Q/L/A lines of the reference driver for a loaded graph."""
    al = []
    for v in range(len(chars)):
        lst = aligned[aligned_off[v]:aligned_off[v + 1]]
        if len(lst):
            al.append(f"{v}:" + ",".join(str(int(x)) for x in lst))
    edges = []
    for e in range(len(edge_tail)):
        lab = "|".join(str(int(x)) for x in labels[label_off[e]:label_off[e + 1]])
        edges.append(f"{int(edge_tail[e])},{int(edge_head[e])},{int(edge_weight[e])},{lab}")
    return {"K": bytes(np.asarray(chars, np.uint8)).decode(),
            "O": " ".join(str(int(x)) for x in rank),
            "S": " ".join(str(int(x)) for x in seq_begin),
            "Q": " ".join(str(int(x)) for x in consensus),
            "L": " ".join(edges), "A": " ".join(al)}


def run_persist(type_: int, params, reads: list[bytes], quals, split: int) -> dict:
    """The persisted-window protocol of ref_driver.cpp on the C oracle:
    reads before `split` added (then GenerateConsensus), the graph saved and
    loaded (oracle_graph_reload), the rest added to the loaded graph."""
    from spoa_gb300.gfa import gfa_lines
    L = lib()
    st = C.c_int32()
    en = L.oracle_engine_create(type_, *params, C.byref(st))
    if not en:
        raise RuntimeError(f"oracle engine: status {st.value}")
    first, g = L.oracle_graph_create(), L.oracle_graph_create()
    res = {"scores": [], "alignments": []}

    def add(graph, k):
        seq = reads[k]
        pairs = np.zeros(2 * (L.oracle_graph_num_nodes(graph) + len(seq) + 16), np.int32)
        n, score = C.c_uint32(0), C.c_int32(0)
        assert L.oracle_align(en, seq, len(seq), graph, C.byref(score), _ptr(pairs),
                              pairs.size // 2, C.byref(n)) == 0
        w = (np.frombuffer(quals[k], np.uint8).astype(np.uint32) - 33 if quals is not None
             else np.ones(len(seq), np.uint32))
        w = np.ascontiguousarray(w, np.uint32)
        aln = pairs[:2 * n.value].reshape(-1, 2).copy()
        assert L.oracle_add_alignment(graph, _ptr(np.ascontiguousarray(aln)), aln.shape[0], seq,
                                      len(seq), _ptr(w), len(seq)) == 0
        return score.value, aln

    try:
        for k in range(split):
            add(first, k)
        if split:
            nn = L.oracle_graph_num_nodes(first)
            L.oracle_consensus(first, C.create_string_buffer(nn + 1), nn + 1)
        assert L.oracle_graph_reload(first, g) == 0
        ex = export_graph(g)
        ne = L.oracle_graph_num_edges(g)
        nn = L.oracle_graph_num_nodes(g)
        et, eh = np.zeros(max(ne, 1), np.uint32), np.zeros(max(ne, 1), np.uint32)
        ew = np.zeros(max(ne, 1), np.int64)
        aoff = np.zeros(nn + 1, np.uint32)
        na = L.oracle_graph_export_ids(g, None, None, None, _ptr(aoff), None)
        al = np.zeros(max(na, 1), np.uint32)
        L.oracle_graph_export_ids(g, _ptr(et), _ptr(eh), _ptr(ew), _ptr(aoff), _ptr(al))
        loff = np.zeros(ne + 1, np.uint32)
        nl = L.oracle_graph_edge_labels(g, _ptr(loff), None)
        labs = np.zeros(max(nl, 1), np.uint32)
        L.oracle_graph_edge_labels(g, _ptr(loff), _ptr(labs))
        res["loaded"] = loaded_lines(ex["chars"], ex["rank_to_node"], ex["seq_begin"],
                                     ex["consensus"], et[:ne], eh[:ne], ew[:ne], loff, labs,
                                     aoff, al)
        for k in range(split, len(reads)):
            score, aln = add(g, k)
            res["scores"].append(score)
            res["alignments"].append(aln)
        nn = L.oracle_graph_num_nodes(g)
        cb = C.create_string_buffer(nn + 1)
        k = L.oracle_consensus(g, cb, nn + 1)
        res["consensus"] = cb.raw[:k].decode()
        rows, rl = C.c_uint32(), C.c_uint32()
        mcap = (len(reads) + 1) * (nn + 1)
        mb = C.create_string_buffer(mcap)
        assert L.oracle_msa(g, 0, mb, mcap, C.byref(rows), C.byref(rl)) == 0
        res["msa"] = [mb.raw[i * rl.value:(i + 1) * rl.value].decode()
                      for i in range(rows.value)]
        ex = export_graph(g)
        res["gfa"] = gfa_lines(ex["chars"], ex["edge_tail"], ex["edge_head"], ex["edge_weight"],
                               ex["paths"], ex["consensus"], None)
        return res
    finally:
        L.oracle_graph_destroy(first)
        L.oracle_graph_destroy(g)
        L.oracle_engine_destroy(en)
