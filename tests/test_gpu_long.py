"""The long-window case: a 10-kb template, reads of 2-10 kb, SW convex on
the int32 width (graphs of ~20k nodes), through the batched kernel and the
fused per-read call, against the oracle."""
import numpy as np
import pytest

import spoa_gb300 as sg
from spoa_gb300 import synth
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _check(res, ref, k=0, r0=0):
    n = len(ref.scores)
    assert res.scores[r0:r0 + n].tolist() == ref.scores
    for a, b in zip(res.alignments[r0:r0 + n], ref.alignments):
        assert np.array_equal(a, b)
    assert res.consensus[k] == ref.consensus


def test_long_window_reduced_vs_oracle():
    """8 reads: batched and fused per-read forms, every alignment."""
    w = synth.long_10k(7, n_reads=8)
    typ, params = synth.SCORING["long_10k"]
    ref = po.run_window(typ, *params, w.reads, with_msa=True)
    res = sg.batch_poa([w.reads], typ, *params, want_alignments=True, want_msa=True)
    assert (res.status == 0).all()
    _check(res, ref)
    assert res.msa[0] == ref.msa
    engine = sg.AlignmentEngine.create(typ, *params)
    graph = sg.Graph()
    scores = [sg.align_add(engine, graph, r)[0] for r in w.reads]
    assert scores == ref.scores
    assert graph.generate_consensus() == ref.consensus


@pytest.mark.timeout(900)
def test_long_window_full_vs_oracle():
    """The full case: 40 reads, every score and alignment and the consensus."""
    w = synth.long_10k(2)
    typ, params = synth.SCORING["long_10k"]
    res = sg.batch_poa([w.reads], typ, *params, want_alignments=True)
    assert (res.status == 0).all()
    assert res.cells > 3e9  # the int32 path over graphs of ~20k nodes
    ref = po.run_window(typ, *params, w.reads, with_msa=False)
    _check(res, ref)


GAPS = {"linear": (5, -4, -8, -8, -8, -8), "affine": (5, -4, -8, -6, -8, -6),
        "convex": (5, -4, -8, -6, -10, -4)}


@pytest.mark.timeout(900)
@pytest.mark.parametrize("gap", sorted(GAPS))
def test_segmented_rows_vs_oracle(gap):
    """Rows of 6.5-7.2k columns on the int32 width: past 12 x 512 columns,
    where each thread holds two 12-column strips of the row; NW, SW and OV,
    every score and alignment and the consensus."""
    w = synth.long_10k(11, n_reads=3, tpl_len=7200, min_len=6500)
    params = GAPS[gap]
    for typ in (0, 1, 2):
        ref = po.run_window(typ, *params, w.reads, with_msa=False)
        # cluster=1: one CTA per window, the segmented kernel
        res = sg.batch_poa([w.reads], typ, *params, want_alignments=True, cluster=1)
        assert (res.status == 0).all()
        _check(res, ref)


@pytest.mark.timeout(900)
@pytest.mark.parametrize("gap", sorted(GAPS))
def test_cluster_rows_vs_oracle(gap):
    """Rows of 2-2.4k and 4.2-4.8k columns on the int32 width: clusters of
    2 and 4 CTAs split each row; NW, SW and OV, both strands, two windows
    per batch, every score, strand choice and alignment and the consensus.
    (Single windows take 8-CTA clusters in the other tests here.)"""
    params = GAPS[gap]
    ws = [synth.long_10k(21, n_reads=3, tpl_len=2400, min_len=2000),
          synth.long_10k(22, n_reads=3, tpl_len=4800, min_len=4200)]
    reads = [[synth.revcomp(r) if j == 1 else r for j, r in enumerate(w.reads)] for w in ws]
    for typ, cl in ((0, 2), (1, 4), (2, 2), (2, 4)):
        strand = typ != 0
        res = sg.batch_poa(reads, typ, *params, want_alignments=True,
                           window_strand=[strand] * 2, cluster=cl)
        assert (res.status == 0).all()
        r0 = 0
        for k, rs in enumerate(reads):
            ref = po.run_window(typ, *params, rs, strand_ambiguous=strand, with_msa=False)
            _check(res, ref, k, r0)
            assert res.reversed[r0:r0 + len(rs)].tolist() == [int(x) for x in ref.reversed]
            r0 += len(rs)


@pytest.mark.timeout(900)
def test_rows_past_16k_columns_vs_oracle():
    """Reads of 16.5-17k columns (four 12-column strips per thread; no
    single strip per thread covers them), SW convex."""
    w = synth.long_10k(12, n_reads=2, tpl_len=17000, min_len=16500)
    typ, params = synth.SCORING["long_10k"]
    ref = po.run_window(typ, *params, w.reads, with_msa=False)
    res = sg.batch_poa([w.reads], typ, *params, want_alignments=True)
    assert (res.status == 0).all()
    _check(res, ref)
