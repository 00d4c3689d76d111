"""Failure paths, all made on the host or through device status words (no
GPU fault, trap or hang is involved):

* a poisoned window in a batch -- one column with more distinct letters
  than a node's aligned-node slots hold (63), which no rerun can fix --
  fails alone with SPOA_GB300_ERR_CAPACITY while every other window of the
  batch finishes bit-exact against the oracle (the reference's own limits
  are its exceptions, graph.cpp:162-194, implementation.hpp:723-725);
* a served window whose working memory exceeds the server's whole device
  budget fails at once with SPOA_GB300_ERR_NO_MEMORY instead of waiting,
  and the windows around it are served normally;
* a preallocation larger than the device maps to the reference's
  "insufficient memory!" (implementation.hpp:404-406), and the engine stays
  usable.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

sg = pytest.importorskip("spoa_gb300")
from oracle import pyoracle as po  # noqa: E402
from spoa_gb300 import synth  # noqa: E402

CAPACITY, NO_MEMORY = 8, 4


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if sg.lib().spoa_gb300_device_count() <= 0:
        pytest.fail("no CUDA device visible to the GPU library")


def _wide_column_window(n_reads=80, ln=60, col=30):
    """Reads equal to one template except at one column, where every read
    carries its own letter (printable ASCII from '!'): that column's node
    collects one aligned node per read."""
    rng = np.random.Generator(np.random.PCG64(91))
    tpl = bytearray(synth.ACGT[rng.integers(0, 4, size=ln)].tobytes())
    letters = [x for x in range(33, 127) if x not in b"ACGT"]  # 90 letters
    reads = []
    for k in range(n_reads):
        r = bytearray(tpl)
        r[col] = letters[k]
        reads.append(bytes(r))
    return reads


@pytest.mark.parametrize("wpc", [1, 2])
def test_poisoned_window_fails_alone(wpc):
    params = synth.SCORING["batch_10k"][1]
    good = [w.reads for w in synth.batch_windows(10, start=1500)]
    bad = _wide_column_window()
    wins = good[:5] + [bad] + good[5:]
    res = sg.batch_poa(wins, 2, *params, want_alignments=True, windows_per_cta=wpc)
    assert res.status[5] == CAPACITY
    assert res.consensus[5] == ""
    r0 = 0
    for k, w in enumerate(wins):
        n = len(w)
        if k != 5:
            assert res.status[k] == 0, k
            ref = po.run_window(2, *params, w, with_msa=False)
            assert res.scores[r0:r0 + n].tolist() == ref.scores, k
            for a, b in zip(res.alignments[r0:r0 + n], ref.alignments):
                assert np.array_equal(a, b), k
            assert res.consensus[k] == ref.consensus, k
        r0 += n


def test_served_window_larger_than_the_budget_fails_at_once():
    params = synth.SCORING["batch_10k"][1]
    small = [w.reads for w in synth.batch_windows(4, start=1600)]
    huge = synth.uneven_window(266).reads  # 4.7-kb reads: far more than 64 MiB of arenas
    with sg.Server(2, *params, memory_budget=64 << 20) as sv:
        tickets = [sv.submit(small[0]), sv.submit(huge, 1, True)] + \
                  [sv.submit(w) for w in small[1:]]
        got = [sv.wait(t, timeout=300) for t in tickets]
    assert got[1][0] == NO_MEMORY and got[1][1] == ""
    for (st, cons, _), w in zip([got[0]] + got[2:], small):
        assert st == 0
        assert cons == po.run_window(2, *params, w, with_msa=False).consensus


def test_preallocation_beyond_the_device_reports_insufficient_memory():
    engine = sg.AlignmentEngine.create(sg.AlignmentType.kSW, 1, -1, -1)
    # 30,000 columns x 7.65 M rows of 32-bit cells: about 940 GB
    with pytest.raises(sg.SpoaError, match="insufficient memory!") as ex:
        engine.prealloc(30000, 255)
    assert ex.value.status == NO_MEMORY
    graph = sg.Graph()
    reads = synth.single_500(3).reads[:4]
    ref = po.run_window(0, 1, -1, -1, -1, -1, -1, reads, with_msa=False)
    for k, r in enumerate(reads):
        aln, score = engine.align(r, graph)
        if k:
            assert score == ref.scores[k]
        graph.add_alignment(aln, r)
    assert graph.generate_consensus() == ref.consensus
