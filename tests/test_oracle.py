"""The C oracle against the reference's own golden vectors and against
recorded outputs of the compiled reference (CPU only)."""
import numpy as np
import pytest

from conftest import check_against_expect
from oracle import pyoracle as po
from spoa_gb300 import synth
from spoa_gb300.gfa import gfa_lines


def _gfa(res):
    g = res.graph
    return gfa_lines(g["chars"], g["edge_tail"], g["edge_head"], g["edge_weight"],
                     g["paths"], g["consensus"], res.reversed)


def test_spoa_test_known_answers(sample_reads, spoa_test_cases):
    """The 18 consensus strings of test/spoa_test.cpp:154-440."""
    reads = [s for s, _ in sample_reads]
    quals = [q for _, q in sample_reads]
    assert len(reads) == 55
    for case in spoa_test_cases:
        res = po.run_window(case["type"], *case["params"], reads,
                            quals if case["quality"] else None)
        assert res.status == 0, case["name"]
        assert res.consensus == case["consensus"], case["name"]
        # Check() of spoa_test.cpp:56-78
        assert len(res.msa) == 55
        rs = len(res.msa[0])
        gaps = [0] * rs
        for row in res.msa:
            assert len(row) == rs
            for k, ch in enumerate(row):
                gaps[k] += ch == "-"
        assert all(gc < len(res.msa) for gc in gaps)
        for row, read in zip(res.msa, reads):
            assert row.replace("-", "") == read.decode()


def test_spoa_test_full_outputs(sample_reads, spoa_test_cases, spoa_test_outputs):
    """Per-read scores/alignments, MSA and GFA of the same 18 runs, as the
    compiled reference printed them."""
    reads = [s for s, _ in sample_reads]
    quals = [q for _, q in sample_reads]
    for case in spoa_test_cases:
        res = po.run_window(case["type"], *case["params"], reads,
                            quals if case["quality"] else None, with_graph=True)
        check_against_expect(spoa_test_outputs[case["name"]], res.scores, res.reversed,
                             res.alignments, res.consensus, res.msa, _gfa(res))


def test_reference_windows(ref_windows):
    """209 seeded windows: every L mod 16, N characters, qualities, strand
    ambiguity, long insertions (convex lane-boundary E), int32 width."""
    for rec in ref_windows:
        reads = [r.encode() for r in rec["reads"]]
        quals = [q.encode() for q in rec["quals"]] if rec["quals"] else None
        res = po.run_window(rec["type"], *rec["params"], reads, quals,
                            rec["strand_ambiguous"], with_graph=True)
        assert res.status == 0, rec["name"]
        check_against_expect(rec["expect"], res.scores, res.reversed, res.alignments,
                             res.consensus, res.msa, _gfa(res))


def test_slice_windows(slice_windows):
    """Graph::Subgraph + UpdateAlignment (graph.cpp:518-605) on backbone
    windows: every subgraph (nodes, order, edges, aligned lists, consensus),
    score, mapped alignment, consensus and MSA against the reference."""
    from conftest import check_slices
    for rec in slice_windows:
        res = po.run_slices(rec["type"], tuple(rec["params"]),
                            [r.encode() for r in rec["reads"]], rec["slices"])
        check_slices(rec["expect"], res["scores"], res["alignments"], res["slices"],
                     res["consensus"], res["msa"])


def test_persist_windows(persist_windows):
    """Graph::save then Graph::load (graph.hpp:187-276): the graph as the
    reference's load rebuilds it, then the remaining reads, against the
    reference's own save/load."""
    from conftest import canon_alignment, sha
    for rec in persist_windows:
        quals = [q.encode() for q in rec["quals"]] if rec["quals"] else None
        res = po.run_persist(rec["type"], tuple(rec["params"]), [r.encode() for r in rec["reads"]],
                             quals, rec["split"])
        exp = rec["expect"]
        if exp["loaded"]:
            assert res["loaded"] == exp["loaded"], rec["name"]
        assert {k: sha(v) for k, v in res["loaded"].items()} == exp["loaded_sha"], rec["name"]
        assert res["scores"] == exp["scores"], rec["name"]
        assert [sha(canon_alignment(a)) for a in res["alignments"]] == exp["aln_sha"]
        assert res["consensus"] == exp["consensus"], rec["name"]
        assert sha("\n".join(res["msa"])) == exp["msa_sha"], rec["name"]
        assert sha("\n".join(res["gfa"])) == exp["gfa_sha"], rec["name"]


def test_engine_errors():
    L = po.lib()
    import ctypes as C
    st = C.c_int32()
    assert not L.oracle_engine_create(4, 1, -1, -1, -1, -1, -1, C.byref(st))
    assert st.value == 1
    assert not L.oracle_engine_create(0, 1, -1, 1, -1, -1, -1, C.byref(st))
    en = L.oracle_engine_create(0, 5, -4, -8, -6, -10, -4, C.byref(st))
    assert en and L.oracle_engine_subtype(en) == 2
    L.oracle_engine_destroy(en)
    en = L.oracle_engine_create(0, 5, -4, -8, -8, -8, -8, C.byref(st))
    assert L.oracle_engine_subtype(en) == 0
    L.oracle_engine_destroy(en)
    en = L.oracle_engine_create(0, 5, -4, -8, -6, -8, -6, C.byref(st))
    assert L.oracle_engine_subtype(en) == 1
    L.oracle_engine_destroy(en)


def test_empty_inputs():
    res = po.run_window(0, 1, -1, -1, -1, -1, -1, [b"ACGT", b""])
    assert res.status == 0 and res.scores == [0, 0]
    assert len(res.alignments[0]) == 0 and len(res.alignments[1]) == 0


@pytest.mark.skipif(po.build_reference() is None, reason="reference tree not present")
def test_live_differential_against_reference():
    """Fresh random windows through the compiled reference and the oracle."""
    rng = np.random.default_rng(7)
    params = [(5, -4, -8, -6, -10, -2), (5, -4, -8, -6, -8, -6), (5, -4, -8, -8, -8, -8),
              (4, -2, -4, -3, -12, -1)]
    specs = []
    for k in range(80):
        reads = synth.random_window(rng, int(rng.integers(1, 90)), int(rng.integers(1, 9)),
                                    err=float(rng.uniform(0.05, 0.35)))
        specs.append((k % 3, params[k % 4], reads, None, k % 5 == 0))
    outs = po.parse_reference_output(po.run_reference(po.format_windows(specs)))
    for (typ, par, reads, quals, strand), ref in zip(specs, outs):
        res = po.run_window(typ, *par, reads, quals, strand)
        assert res.scores == ref["scores"]
        assert all(np.array_equal(a, b) for a, b in zip(res.alignments, ref["alignments"]))
        assert res.consensus == ref["consensus"] and res.msa == ref["msa"]


@pytest.mark.skipif(po.build_reference() is None, reason="reference tree not present")
def test_live_differential_random_scoring():
    """Seeded random windows with random scoring through the compiled
    reference and the oracle: alphabets of 2 to 20 letters, reads of 1-150
    bases at error rates up to 60 %, match 0-10, mismatch -10-0, every gap
    model with penalties 0 to -12 (equal ones included), every alignment
    type, strands and qualities.  Pins the oracle where the recorded
    fixtures do not reach."""
    rng = np.random.default_rng(11)
    alphabets = (b"ACGT", b"ACGTN", b"AC", b"ACDEFGHIKLMNPQRSTVWY")
    specs = []
    for k in range(150):
        alpha = list(alphabets[int(rng.integers(len(alphabets)))])
        tpl = rng.choice(alpha, size=int(rng.integers(1, 150)))
        err = float(rng.choice([0.0, 0.05, 0.15, 0.6]))
        reads = []
        for _ in range(int(rng.integers(1, 8))):
            out = []
            for b in tpl:
                u = rng.random()
                if u < err / 3:
                    continue
                if u < 2 * err / 3:
                    out.append(int(rng.choice(alpha)))
                out.append(int(rng.choice(alpha)) if u < err else int(b))
            reads.append(bytes(out) or bytes([alpha[0]]))
        par = (int(rng.integers(0, 11)), int(rng.integers(-10, 1)),
               *(int(x) for x in -rng.integers(0, 13, size=4)))
        quals = ([bytes((rng.integers(0, 41, size=len(r)) + 33).astype(np.uint8)) for r in reads]
                 if rng.random() < 0.3 else None)
        specs.append((int(rng.integers(0, 3)), par, reads, quals, bool(rng.random() < 0.3)))
    outs = po.parse_reference_output(po.run_reference(po.format_windows(specs)))
    assert len(outs) == len(specs)
    for (typ, par, reads, quals, strand), ref in zip(specs, outs):
        res = po.run_window(typ, *par, reads, quals, strand)
        assert res.scores == ref["scores"], (typ, par)
        assert all(np.array_equal(a, b) for a, b in zip(res.alignments, ref["alignments"]))
        assert res.consensus == ref["consensus"] and res.msa == ref["msa"], (typ, par)
