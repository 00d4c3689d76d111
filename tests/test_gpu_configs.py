"""Whole windows of the single-window and uneven workloads on the GPU against
the oracle, bit-exact: every read's score, strand and alignment, the
consensus and the MSA.

* The single 500-nt window (30 full-length reads, NW affine 5/-4/-8/-6)
  through the drop-in per-call API (Align, then AddAlignment, read by read)
  and through the persistent kernel.
* Uneven windows at full depth (no read dropped): templates of 3-4.7 kb,
  which need 32-bit scores from their second read on, and windows whose
  graph crosses the reference's int16 rule part-way through
  (implementation.hpp:719-775: the width is chosen per read from read length
  and graph size), both strands aligned (main.cpp:285-302).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

sg = pytest.importorskip("spoa_gb300")
from oracle import pyoracle as po  # noqa: E402
from spoa_gb300 import synth  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if sg.lib().spoa_gb300_device_count() <= 0:
        pytest.fail("no CUDA device visible to the GPU library")


def _int16_ok(params, L, V):
    """The reference's width rule (alignment_engine.cpp:101-110 with
    implementation.hpp:719-726): 16-bit lanes when the worst case fits."""
    m, _, g, e, q, c = params

    def gap(n):
        return 0 if n == 0 else min(g + (n - 1) * e, q + (n - 1) * c)
    i, j = L + 8, V
    wc = min(-(m * min(i, j) + gap(abs(i - j))), gap(i) + gap(j))
    return wc >= -32768 + 1024


def test_single_500_window_per_call_and_batched():
    w = synth.single_500(1)
    typ, params = synth.SCORING["single_500"]
    ref = po.run_window(typ, *params, w.reads)
    assert ref.status == 0
    engine = sg.AlignmentEngine.create(typ, *params)
    graph = sg.Graph()
    for k, r in enumerate(w.reads):
        aln, score = engine.align(r, graph)
        if k == 0:
            assert score is None and aln.shape == (0, 2)
        else:
            assert score == ref.scores[k], k
        assert np.array_equal(aln, ref.alignments[k]), k
        graph.add_alignment(aln, r)
    assert graph.generate_consensus() == ref.consensus
    assert graph.generate_multiple_sequence_alignment() == ref.msa
    res = sg.batch_poa([w.reads], typ, *params, want_alignments=True, want_msa=True)
    assert res.status[0] == 0
    assert res.scores.tolist()[1:] == ref.scores[1:]
    for a, b in zip(res.alignments, ref.alignments):
        assert np.array_equal(a, b)
    assert res.consensus[0] == ref.consensus
    assert res.msa[0] == ref.msa


# uneven windows (synth.uneven_window ids): four templates of 3.1-4.7 kb
# (32-bit from the second read) and four whose graph passes the int16 rule
# part-way (1.7-2.1 kb templates, 20-36 reads; NW and OV)
LONG_IDS = (346, 375, 12, 266)
CROSSING_IDS = (38, 83, 175, 184)


def test_uneven_windows_at_full_depth():
    _, params = synth.SCORING["uneven_2k"]
    wins = [synth.uneven_window(k) for k in LONG_IDS + CROSSING_IDS]
    for k, w in zip(LONG_IDS, wins[:4]):
        assert len(w.reads[0]) >= 3000, k
    refs = [po.run_window(w.type, *params, w.reads, strand_ambiguous=True) for w in wins]
    for k, w, ref in zip(LONG_IDS + CROSSING_IDS, wins, refs):
        assert ref.status == 0, k
        if k in CROSSING_IDS:  # 16-bit at the second read, 32-bit at the last
            before_last = po.run_window(w.type, *params, w.reads[:-1], strand_ambiguous=True,
                                        with_msa=False, with_graph=True)
            v_last = len(before_last.graph["chars"])  # graph nodes the last read meets
            assert _int16_ok(params, len(w.reads[1]), len(w.reads[0])), k
            assert not _int16_ok(params, len(w.reads[-1]), v_last), k
    res = sg.batch_poa([w.reads for w in wins], 1, *params, window_types=[w.type for w in wins],
                       window_strand=[1] * len(wins), want_alignments=True, want_msa=True)
    assert (res.status == 0).all(), res.status
    r0 = 0
    for k, (w, ref) in enumerate(zip(wins, refs)):
        n = len(w.reads)
        assert res.scores[r0:r0 + n].tolist() == ref.scores, k
        assert res.reversed[r0:r0 + n].tolist() == ref.reversed, k
        for a, b in zip(res.alignments[r0:r0 + n], ref.alignments):
            assert np.array_equal(a, b), k
        assert res.consensus[k] == ref.consensus, k
        assert res.msa[k] == ref.msa, k
        r0 += n
