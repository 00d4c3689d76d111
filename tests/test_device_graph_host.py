"""The device graph code (spoa_gb300/csrc/poa_device.cuh: AddAlignment, the
topological sort, consensus, Subgraph, graph loading) compiled for the host
by tests/host/device_graph_host.cpp and compared with the oracle on the CPU,
read by read: node characters, rank order, every edge (tail, head, weight,
labels), aligned lists, sequence starts and the consensus."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import ROOT, host_library
from oracle import pyoracle as po
from spoa_gb300 import synth

SRC = os.path.join(ROOT, "tests", "host", "device_graph_host.cpp")
OUT = os.path.join(ROOT, "tests", "host", "_build", "libdevice_graph_host.so")
P, U32 = C.c_void_p, C.c_uint32


@pytest.fixture(scope="module")
def dg():
    deps = [os.path.join(ROOT, "spoa_gb300", "csrc", "poa_device.cuh")]
    L = C.CDLL(host_library(SRC, OUT, deps, "c++17", "-O2"))
    L.dg_create.restype = P
    L.dg_create.argtypes = [U32] * 5
    L.dg_destroy.argtypes = [P]
    L.dg_add.argtypes = [P, P, U32, C.c_char_p, U32, P, C.c_int32]
    L.dg_counts.argtypes = [P, P]
    L.dg_export.argtypes = [P] * 12
    L.dg_consensus.argtypes = [P, C.c_char_p, U32]
    L.dg_consensus.restype = U32
    L.dg_subgraph.argtypes = [P, U32, U32, P, P]
    L.dg_reload.argtypes = [P, P]
    return L


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _new(L, total):
    # capacities of a per-call graph holding reads of `total` bases
    return L.dg_create(total + 8, 2 * total + 64, 2 * total + 64, 256, 31)


def dg_state(L, g) -> dict:
    cnt = np.zeros(6, np.uint32)
    L.dg_counts(g, _ptr(cnt))
    N, E, S, Cn, Lb = (int(x) for x in cnt[:5])
    z = lambda k, t: np.zeros(max(k, 1), t)  # noqa: E731
    chars, rank = z(N, np.uint8), z(N, np.uint32)
    et, eh, ew = z(E, np.uint32), z(E, np.uint32), z(E, np.int64)
    loff, labs = z(E + 1, np.uint32), z(Lb, np.uint32)
    aoff, al = z(N + 1, np.uint32), z(N * 31, np.uint32)
    sb, cons = z(S, np.uint32), z(Cn, np.uint32)
    L.dg_export(g, *[_ptr(a) for a in (chars, rank, et, eh, ew, loff, labs, aoff, al, sb, cons)])
    edges = [(int(et[e]), int(eh[e]), int(ew[e]), tuple(labs[loff[e]:loff[e + 1]].tolist()))
             for e in range(E)]
    return {"chars": chars[:N].tobytes(), "rank": rank[:N].tolist(), "edges": edges,
            "aligned": [tuple(al[aoff[v]:aoff[v + 1]].tolist()) for v in range(N)],
            "seq_begin": sb[:S].tolist(), "consensus": cons[:Cn].tolist()}


def oracle_state(g) -> dict:
    L = po.lib()
    ex = po.export_graph(g)
    N = L.oracle_graph_num_nodes(g)
    E = L.oracle_graph_num_edges(g)
    z = lambda k, t: np.zeros(max(k, 1), t)  # noqa: E731
    et, eh, ew = z(E, np.uint32), z(E, np.uint32), z(E, np.int64)
    aoff = np.zeros(N + 1, np.uint32)
    na = L.oracle_graph_export_ids(g, None, None, None, _ptr(aoff), None)
    al = z(na, np.uint32)
    L.oracle_graph_export_ids(g, _ptr(et), _ptr(eh), _ptr(ew), _ptr(aoff), _ptr(al))
    loff = np.zeros(E + 1, np.uint32)
    nl = L.oracle_graph_edge_labels(g, _ptr(loff), None)
    labs = z(nl, np.uint32)
    L.oracle_graph_edge_labels(g, _ptr(loff), _ptr(labs))
    edges = [(int(et[e]), int(eh[e]), int(ew[e]), tuple(labs[loff[e]:loff[e + 1]].tolist()))
             for e in range(E)]
    return {"chars": ex["chars"].tobytes(), "rank": ex["rank_to_node"].tolist(), "edges": edges,
            "aligned": [tuple(al[aoff[v]:aoff[v + 1]].tolist()) for v in range(N)],
            "seq_begin": ex["seq_begin"].tolist(), "consensus": ex["consensus"].tolist()}


def _window(L, type_, params, reads, quals=None, check_every_read=True, prepass=True):
    """Replays a window on the oracle and on the host-built device graph
    with the oracle's alignments; returns both graphs (caller frees)."""
    O = po.lib()
    st = C.c_int32()
    en = O.oracle_engine_create(type_, *params, C.byref(st))
    og = O.oracle_graph_create()
    g = _new(L, sum(len(r) for r in reads))
    for k, r in enumerate(reads):
        pairs = np.zeros(2 * (O.oracle_graph_num_nodes(og) + len(r) + 16), np.int32)
        n, score = C.c_uint32(0), C.c_int32(0)
        assert O.oracle_align(en, r, len(r), og, C.byref(score), _ptr(pairs), pairs.size // 2,
                              C.byref(n)) == 0
        w = (np.frombuffer(quals[k], np.uint8).astype(np.uint32) - 33 if quals
             else np.ones(len(r), np.uint32))
        w = np.ascontiguousarray(w, np.uint32)
        aln = np.ascontiguousarray(pairs[:2 * n.value])
        assert O.oracle_add_alignment(og, _ptr(aln), n.value, r, len(r), _ptr(w), len(r)) == 0
        assert L.dg_add(g, _ptr(aln), n.value, r, len(r), _ptr(w), 1 if prepass else 0) == 0
        if check_every_read or k == len(reads) - 1:
            assert dg_state(L, g) == oracle_state(og), k
    O.oracle_engine_destroy(en)
    return og, g


def test_add_alignment_and_sort_match_the_oracle(dg, ref_windows):
    """Every read of 60 recorded windows (adversarial lengths, N bases,
    qualities, long insertions, polishing and uneven shapes): the graph after
    each AddAlignment + sort, then the consensus; half the windows add with
    the read-only pre-pass (g_add_prepass), half without."""
    O = po.lib()
    for i, rec in enumerate(ref_windows[::3][:60]):
        reads = [r.encode() for r in rec["reads"]]
        quals = [q.encode() for q in rec["quals"]] if rec["quals"] else None
        # the add with and without its read-only pre-pass
        og, g = _window(dg, rec["type"], tuple(rec["params"]), reads, quals, prepass=i % 2 == 0)
        n = O.oracle_graph_num_nodes(og)
        a, b = C.create_string_buffer(n + 1), C.create_string_buffer(n + 1)
        ka = O.oracle_consensus(og, a, n + 1)
        kb = dg.dg_consensus(g, b, n + 1)
        assert a.raw[:ka] == b.raw[:kb] == rec["expect"]["consensus"].encode(), rec["name"]
        assert dg_state(dg, g) == oracle_state(og), rec["name"]
        O.oracle_graph_destroy(og)
        dg.dg_destroy(g)


def test_subgraph_and_reload_match_the_oracle(dg):
    """Subgraph of a grown window for many (begin, end) pairs, including
    inverted and single-node ranges, and save-then-load of the window."""
    O = po.lib()
    w = synth.batch_window(7)
    reads = w.reads[:20]
    og, g = _window(dg, 2, synth.SCORING["batch_10k"][1], reads, check_every_read=False)
    n = O.oracle_graph_num_nodes(og)
    nb = C.create_string_buffer(n + 1)
    O.oracle_consensus(og, nb, n + 1)
    dg.dg_consensus(g, nb, n + 1)
    rng = np.random.Generator(np.random.PCG64(9))
    for _ in range(25):
        b, e = (int(x) for x in rng.integers(0, n, size=2))
        osub, gsub = O.oracle_graph_create(), _new(dg, n)
        m1, m2 = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        assert O.oracle_subgraph(og, b, e, osub, _ptr(m1)) == 0
        assert dg.dg_subgraph(g, b, e, gsub, _ptr(m2)) == 0
        ns = O.oracle_graph_num_nodes(osub)
        assert m1[:ns].tolist() == m2[:ns].tolist()
        assert dg_state(dg, gsub) == oracle_state(osub), (b, e)
        O.oracle_graph_destroy(osub)
        dg.dg_destroy(gsub)
    orl, grl = O.oracle_graph_create(), _new(dg, sum(len(r) for r in reads))
    assert O.oracle_graph_reload(og, orl) == 0
    assert dg.dg_reload(g, grl) == 0
    assert dg_state(dg, grl) == oracle_state(orl)
    for x in (og, orl):
        O.oracle_graph_destroy(x)
    for x in (g, grl):
        dg.dg_destroy(x)


def test_random_windows_with_subgraphs_and_reloads(dg):
    """Seeded random windows (alphabets of 2 to 20 letters, so up to 19
    nodes aligned to one another; error rates up to 60 %; qualities; random
    scoring and type): the graph after every read, then a few subgraphs and
    a save-then-load, each against the oracle."""
    O = po.lib()
    rng = np.random.Generator(np.random.PCG64(31))
    alphabets = (b"ACGT", b"AC", b"ACDEFGHIKLMNPQRSTVWY")
    for k in range(40):
        alpha = list(alphabets[k % 3])
        tpl = rng.choice(alpha, size=int(rng.integers(5, 120)))
        err = float(rng.choice([0.05, 0.2, 0.6]))
        reads = []
        for _ in range(int(rng.integers(2, 8))):
            out = []
            for b in tpl:
                u = rng.random()
                if u < err / 3:
                    continue
                if u < 2 * err / 3:
                    out.append(int(rng.choice(alpha)))
                out.append(int(rng.choice(alpha)) if u < err else int(b))
            reads.append(bytes(out) or bytes([alpha[0]]))
        quals = ([bytes((rng.integers(0, 41, size=len(r)) + 33).astype(np.uint8)) for r in reads]
                 if k % 2 else None)
        params = (int(rng.integers(1, 11)), int(rng.integers(-10, 0)),
                  *(int(x) for x in -rng.integers(1, 13, size=4)))
        og, g = _window(dg, int(rng.integers(0, 3)), params, reads, quals, prepass=k % 2 == 0)
        n = O.oracle_graph_num_nodes(og)
        nb = C.create_string_buffer(n + 1)
        assert O.oracle_consensus(og, nb, n + 1) == dg.dg_consensus(g, nb, n + 1)
        assert dg_state(dg, g) == oracle_state(og), k
        for _ in range(3):
            b, e = (int(x) for x in rng.integers(0, n, size=2))
            osub, gsub = O.oracle_graph_create(), _new(dg, n)
            m1, m2 = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
            assert O.oracle_subgraph(og, b, e, osub, _ptr(m1)) == 0
            assert dg.dg_subgraph(g, b, e, gsub, _ptr(m2)) == 0
            ns = O.oracle_graph_num_nodes(osub)
            assert m1[:ns].tolist() == m2[:ns].tolist()
            assert dg_state(dg, gsub) == oracle_state(osub), (k, b, e)
            O.oracle_graph_destroy(osub)
            dg.dg_destroy(gsub)
        orl, grl = O.oracle_graph_create(), _new(dg, sum(len(r) for r in reads))
        assert O.oracle_graph_reload(og, orl) == 0
        assert dg.dg_reload(g, grl) == 0
        assert dg_state(dg, grl) == oracle_state(orl), k
        for x in (og, orl):
            O.oracle_graph_destroy(x)
        for x in (g, grl):
            dg.dg_destroy(x)
