"""The batched kernel with 2 or 4 windows in flight per CTA (the windows'
serial graph updates on parallel lanes) against the oracle, bit-exact:
every read's score, strand and alignment and every consensus, for
polishing windows, strand-ambiguous uneven windows (whose 32-bit windows
run in the one-window kernel of the same batch), quality weights, and
fewer windows than slots."""
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


def _check(res, wins, refs):
    assert (res.status == 0).all(), res.status
    r0 = 0
    for k, (w, ref) in enumerate(zip(wins, refs)):
        n = len(w)
        assert res.scores[r0:r0 + n].tolist() == ref.scores, k
        assert res.reversed[r0:r0 + n].tolist() == ref.reversed, k
        for a, b in zip(res.alignments[r0:r0 + n], ref.alignments):
            assert np.array_equal(a, b), k
        assert res.consensus[k] == ref.consensus, k
        r0 += n


@pytest.mark.parametrize("wpc", [2, 4])
def test_polishing_windows(wpc):
    params = synth.SCORING["batch_10k"][1]
    wins = [w.reads for w in synth.batch_windows(30, start=1200)]
    refs = [po.run_window(2, *params, w, with_msa=False) for w in wins]
    res = sg.batch_poa(wins, 2, *params, want_alignments=True, windows_per_cta=wpc)
    _check(res, wins, refs)


@pytest.mark.parametrize("wpc", [2, 4])
def test_uneven_strand_ambiguous_windows(wpc):
    _, params = synth.SCORING["uneven_2k"]
    src = [synth.uneven_window(k) for k in range(40, 56)]
    wins = [w.reads[:24] for w in src]
    types = [w.type for w in src]
    refs = [po.run_window(t, *params, w, strand_ambiguous=True, with_msa=False)
            for t, w in zip(types, wins)]
    res = sg.batch_poa(wins, 1, *params, window_types=types, window_strand=[1] * len(wins),
                       want_alignments=True, windows_per_cta=wpc)
    _check(res, wins, refs)


@pytest.mark.parametrize("wpc", [2, 4])
def test_quality_weights(wpc):
    params = synth.SCORING["batch_10k"][1]
    wins = [w.reads for w in synth.batch_windows(12, start=1300)]
    rng = np.random.Generator(np.random.PCG64(1301))
    quals = [[bytes((rng.integers(0, 41, size=len(r)) + 33).astype(np.uint8)) for r in w]
             for w in wins]
    refs = [po.run_window(2, *params, w, quals=q, with_msa=False) for w, q in zip(wins, quals)]
    res = sg.batch_poa(wins, 2, *params, quals=quals, want_alignments=True, windows_per_cta=wpc)
    _check(res, wins, refs)


def test_fewer_windows_than_slots():
    params = synth.SCORING["batch_10k"][1]
    wins = [w.reads for w in synth.batch_windows(3, start=1400)]
    refs = [po.run_window(2, *params, w, with_msa=False) for w in wins]
    res = sg.batch_poa(wins, 2, *params, want_alignments=True, windows_per_cta=4)
    _check(res, wins, refs)
    one = sg.batch_poa(wins, 2, *params, want_msa=True)
    four = sg.batch_poa(wins, 2, *params, want_msa=True, windows_per_cta=4)
    assert one.msa == four.msa
