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
