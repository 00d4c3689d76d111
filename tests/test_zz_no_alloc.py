"""The single-window entry point that allocates no device memory.

Some callers cannot call cudaMalloc: work issued between the captures of a
CUDA graph, frameworks whose allocator owns all device memory, or loops that
cannot afford cudaMalloc's implicit synchronisation.  For them
spoa_gb300_window_poa_noalloc runs one window through the persistent kernel
with its working memory in a fixed 48 MiB array inside the library; the
caller owns every input and output buffer.  These tests call it through the
C ABI several times in a row (the array keeps the previous call's contents)
and compare its consensus and per-read scores with the batched entry point
and with the oracle, exactly (the path is integer arithmetic).  They also
drive every status the device reports (capacity, 32-bit scores needed) with
inputs whose bounds checks stop the kernel before any access past a buffer.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

sg = pytest.importorskip("spoa_gb300")
torch = pytest.importorskip("torch")
from oracle import pyoracle as po  # noqa: E402
from spoa_gb300 import synth  # noqa: E402

CONS_CAP = 4096
OK, TOO_LARGE, CAPACITY, NEEDS_INT32 = 0, 2, 8, 11


def _run_noalloc(reads, type_, params, strand=False, quals=None, max_len=None,
                 cons_cap=CONS_CAP):
    L = sg.lib()
    blob = np.frombuffer(b"".join(reads), np.uint8)
    off = np.zeros(len(reads) + 1, np.int64)
    off[1:] = np.cumsum([len(r) for r in reads])
    # the caller's own device buffers: the entry point allocates nothing
    d_seqs = torch.tensor(blob, device="cuda")
    d_off = torch.tensor(off, device="cuda")  # same bytes as uint64
    d_quals = (torch.tensor(np.frombuffer(b"".join(quals), np.uint8), device="cuda")
               if quals is not None else None)
    d_cons = torch.zeros(max(cons_cap, 1), dtype=torch.uint8, device="cuda")
    d_len = torch.zeros(1, dtype=torch.int32, device="cuda")
    d_scores = torch.zeros(len(reads), dtype=torch.int32, device="cuda")
    d_status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = L.spoa_gb300_window_poa_noalloc(
        type_, *params, 1 if strand else 0, len(reads),
        max_len if max_len is not None else max(len(r) for r in reads),
        C.c_void_p(d_seqs.data_ptr()), C.c_void_p(d_off.data_ptr()),
        C.c_void_p(d_quals.data_ptr()) if d_quals is not None else None,
        C.c_void_p(d_cons.data_ptr()), cons_cap, C.c_void_p(d_len.data_ptr()),
        C.c_void_p(d_scores.data_ptr()), C.c_void_p(d_status.data_ptr()), None)
    assert st == OK, st
    torch.cuda.synchronize()
    n = min(int(d_len.item()), cons_cap)
    return (int(d_status.item()), bytes(d_cons[:n].cpu().numpy()).decode(),
            d_scores.cpu().numpy())


def _run_batched(reads, type_, params, strand=False, quals=None):
    res = sg.batch_poa([reads], type_, *params, window_strand=[1 if strand else 0],
                       quals=[quals] if quals is not None else None)
    assert res.status[0] == 0
    return res.consensus[0], res.scores


@pytest.mark.parametrize("strand", [False, True])
def test_matches_batched_entry_point_twice(strand):
    params = synth.SCORING["batch_10k"][1]
    wins = [synth.batch_window(7001), synth.batch_window(7002)]
    if strand:  # half of the reads on the other strand
        wins = [synth.Window(reads=[synth.revcomp(r) if k % 2 else r
                                    for k, r in enumerate(w.reads)], type=2) for w in wins]
    for w in wins + wins[:1]:  # two different windows, then the first again
        status, cons, scores = _run_noalloc(w.reads, 2, params, strand)
        assert status == OK
        ref_cons, ref_scores = _run_batched(w.reads, 2, params, strand)
        assert cons == ref_cons
        assert np.array_equal(scores, ref_scores)


def _quals_for(reads, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return [bytes((rng.integers(0, 41, size=len(r)) + 33).astype(np.uint8)) for r in reads]


@pytest.mark.parametrize("type_", [0, 1, 2])
@pytest.mark.parametrize("with_quals", [False, True])
def test_every_mode_against_batched_and_oracle(type_, with_quals):
    """SW, NW and OV, with and without quality weights (affine and convex
    gaps): each window twice in a row, equal to the batched entry point and
    to the oracle, score by score."""
    sub_params = {0: (5, -4, -8, -6, -10, -4), 1: (5, -4, -8, -6, -8, -6),
                  2: synth.SCORING["batch_10k"][1]}[type_]
    wins = [synth.batch_window(7100 + type_), synth.single_500(7200 + type_)]
    for w in wins + wins[:1]:
        reads = w.reads[:30]
        quals = _quals_for(reads, 7300 + type_) if with_quals else None
        status, cons, scores = _run_noalloc(reads, type_, sub_params, quals=quals)
        assert status == OK
        ref_cons, ref_scores = _run_batched(reads, type_, sub_params, quals=quals)
        assert cons == ref_cons
        assert np.array_equal(scores, ref_scores)
        ref = po.run_window(type_, *sub_params, reads, quals=quals, with_msa=False)
        assert cons == ref.consensus
        assert scores.tolist() == ref.scores


def test_rejects_sizes_beyond_the_limits():
    L = sg.lib()
    params = synth.SCORING["batch_10k"][1]
    dummy = C.c_void_p(1)
    too_many = L.spoa_gb300_window_poa_noalloc(2, *params, 0, 257, 500, dummy, dummy, None,
                                               dummy, CONS_CAP, dummy, None, dummy, None)
    too_long = L.spoa_gb300_window_poa_noalloc(2, *params, 0, 10, 641, dummy, dummy, None,
                                               dummy, CONS_CAP, dummy, None, dummy, None)
    assert too_many == TOO_LARGE and too_long == TOO_LARGE


def test_device_checked_limits_report_capacity():
    """The limits the host cannot check (it never sees the device-resident
    reads or the graph) end the window with SPOA_GB300_ERR_CAPACITY in
    *d_status: a graph past 4,096 nodes, a consensus longer than its
    buffer, and a first read longer than the max_read_len passed in (both
    strands, so the reverse-complement staging is covered).  A normal window
    run afterwards still matches the batched entry point."""
    params = synth.SCORING["batch_10k"][1]
    rng = np.random.Generator(np.random.PCG64(79))
    big = synth.random_window(rng, 300, 60, err=0.6, alphabet=b"ACDEFGHIKLMNPQRSTVWY")
    status, _, _ = _run_noalloc(big, 2, params)
    assert status == CAPACITY
    w = synth.batch_window(7401)
    status, _, _ = _run_noalloc(w.reads, 2, params, cons_cap=16)
    assert status == CAPACITY
    reads = [b"ACGT" * 125] + w.reads[:5]  # 500 bases against a 384-column tile
    status, _, _ = _run_noalloc(reads, 2, params, strand=True, max_len=320)
    assert status == CAPACITY
    status, cons, scores = _run_noalloc(w.reads, 2, params)
    assert status == OK
    ref_cons, ref_scores = _run_batched(w.reads, 2, params)
    assert cons == ref_cons and np.array_equal(scores, ref_scores)


def test_reads_that_need_32_bit_scores_report_it():
    """With gap penalties of -20 the reference's width rule leaves 16 bits
    once read length + graph nodes pass about 1,580; the window then ends
    with SPOA_GB300_ERR_NEEDS_INT32 (this entry point has only the 16-bit
    kernels)."""
    params = (5, -4, -20, -20, -20, -20)
    rng = np.random.Generator(np.random.PCG64(81))
    reads = [synth.ACGT[rng.integers(0, 4, size=500)].tobytes() for _ in range(6)]
    status, _, _ = _run_noalloc(reads, 0, params)
    assert status == NEEDS_INT32
