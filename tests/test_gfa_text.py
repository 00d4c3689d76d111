"""The C ABI's GFA writer (spoa_gb300/csrc/gfa_text.h, behind
spoa_gb300_graph_gfa) on the oracle's graphs of recorded windows, byte for
byte against the oracle's GFA text (which the recorded reference GFA pins)."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import ROOT, host_library
from oracle import pyoracle as po
from spoa_gb300.gfa import gfa_lines

SRC = os.path.join(ROOT, "tests", "host", "gfa_host.cpp")
OUT = os.path.join(ROOT, "tests", "host", "_build", "libgfa_host.so")


@pytest.fixture(scope="module")
def gh():
    deps = [os.path.join(ROOT, "spoa_gb300", "csrc", "gfa_text.h")]
    L = C.CDLL(host_library(SRC, OUT, deps, "c++17", "-O2"))
    P = C.c_void_p
    L.gh_gfa.argtypes = [C.c_uint32] * 3 + [P] * 11 + [C.c_int32, C.c_char_p, C.c_uint64]
    L.gh_gfa.restype = C.c_uint64
    return L


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def test_gfa_text_matches_the_oracle(gh, ref_windows):
    for rec in ref_windows[::9]:
        reads = [r.encode() for r in rec["reads"]]
        quals = [q.encode() for q in rec["quals"]] if rec["quals"] else None
        res = po.run_window(rec["type"], *rec["params"], reads, quals,
                            strand_ambiguous=rec["strand_ambiguous"], with_msa=False,
                            with_graph=True)
        g = res.graph
        n = len(g["chars"])
        # out-edge CSR by edge id from the node-major edge order, and labels
        # by edge id, rebuilt from the oracle's per-sequence paths
        tails, heads, weights = g["edge_tail"], g["edge_head"], g["edge_weight"]
        ne = len(tails)
        out_off = np.zeros(n + 1, np.uint32)
        for t in tails:
            out_off[int(t) + 1] += 1
        out_off = np.cumsum(out_off).astype(np.uint32)
        out_edges = np.arange(max(ne, 1), dtype=np.uint32)
        key = {(int(t), int(h)): e for e, (t, h) in enumerate(zip(tails, heads))}
        labs = [[] for _ in range(ne)]
        for s, path in enumerate(g["paths"]):
            for a, b in zip(path[:-1], path[1:]):
                labs[key[(int(a), int(b))]].append(s)
        label_off = np.zeros(ne + 1, np.uint32)
        label_off[1:] = np.cumsum([len(x) for x in labs])
        labels = np.array([x for lst in labs for x in lst] or [0], np.uint32)
        rev = np.array(res.reversed if rec["strand_ambiguous"] else [0] * len(reads), np.uint8)
        names = [f"r{s}".encode() for s in range(len(reads))]
        arr = (C.c_char_p * len(names))(*names)
        buf = C.create_string_buffer(1 << 22)
        ln = gh.gh_gfa(n, len(reads), len(g["consensus"]), _ptr(g["chars"]), _ptr(out_off),
                       _ptr(out_edges), _ptr(np.ascontiguousarray(heads, np.uint32)),
                       _ptr(np.ascontiguousarray(weights, np.int64)), _ptr(label_off),
                       _ptr(labels), _ptr(np.ascontiguousarray(g["seq_begin"], np.uint32)),
                       _ptr(np.ascontiguousarray(g["consensus"], np.uint32)), arr,
                       _ptr(rev) if rec["strand_ambiguous"] else None, 1, buf, len(buf))
        text = buf.raw[:ln].decode()
        want = gfa_lines(g["chars"], tails, heads, weights, g["paths"], g["consensus"],
                         res.reversed if rec["strand_ambiguous"] else None,
                         [x.decode() for x in names], True)
        assert text == "\n".join(want) + "\n", rec["name"]
        # default names and no consensus line
        ln2 = gh.gh_gfa(n, len(reads), len(g["consensus"]), _ptr(g["chars"]), _ptr(out_off),
                        _ptr(out_edges), _ptr(np.ascontiguousarray(heads, np.uint32)),
                        _ptr(np.ascontiguousarray(weights, np.int64)), _ptr(label_off),
                        _ptr(labels), _ptr(np.ascontiguousarray(g["seq_begin"], np.uint32)),
                        _ptr(np.ascontiguousarray(g["consensus"], np.uint32)), None, None, 0,
                        buf, len(buf))
        want2 = gfa_lines(g["chars"], tails, heads, weights, g["paths"], g["consensus"], None,
                          None, False)
        assert buf.raw[:ln2].decode() == "\n".join(want2) + "\n", rec["name"]
