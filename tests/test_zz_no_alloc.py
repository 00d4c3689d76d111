"""The single-window entry point that allocates no device memory.

Some callers cannot call cudaMalloc: work issued between the captures of a
CUDA graph, frameworks whose allocator owns all device memory, or loops that
cannot afford cudaMalloc's implicit synchronisation.  For them
spoa_gb300_window_poa_noalloc runs one window through the persistent kernel
with its working memory in a fixed 48 MiB array inside the library; the
caller owns every input and output buffer.  These tests call it through the
C ABI twice in a row (the array keeps the previous call's contents) and
compare its consensus and per-read scores with the batched entry point,
exactly (the path is integer arithmetic).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

sg = pytest.importorskip("spoa_gb300")
torch = pytest.importorskip("torch")
from spoa_gb300 import synth  # noqa: E402

CONS_CAP = 4096


def _run_noalloc(reads, type_, params, strand=False):
    L = sg.lib()
    blob = np.frombuffer(b"".join(reads), np.uint8)
    off = np.zeros(len(reads) + 1, np.int64)
    off[1:] = np.cumsum([len(r) for r in reads])
    # the caller's own device buffers: the entry point allocates nothing
    d_seqs = torch.tensor(blob, device="cuda")
    d_off = torch.tensor(off, device="cuda")  # same bytes as uint64
    d_cons = torch.zeros(CONS_CAP, dtype=torch.uint8, device="cuda")
    d_len = torch.zeros(1, dtype=torch.int32, device="cuda")
    d_scores = torch.zeros(len(reads), dtype=torch.int32, device="cuda")
    d_status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = L.spoa_gb300_window_poa_noalloc(
        type_, *params, 1 if strand else 0, len(reads), max(len(r) for r in reads),
        C.c_void_p(d_seqs.data_ptr()), C.c_void_p(d_off.data_ptr()), None,
        C.c_void_p(d_cons.data_ptr()), CONS_CAP, C.c_void_p(d_len.data_ptr()),
        C.c_void_p(d_scores.data_ptr()), C.c_void_p(d_status.data_ptr()), None)
    assert st == 0, st
    torch.cuda.synchronize()
    n = int(d_len.item())
    return (int(d_status.item()), bytes(d_cons[:n].cpu().numpy()).decode(),
            d_scores.cpu().numpy())


def _run_batched(reads, type_, params, strand=False):
    res = sg.batch_poa([reads], type_, *params, window_strand=[1 if strand else 0])
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
        assert status == 0
        ref_cons, ref_scores = _run_batched(w.reads, 2, params, strand)
        assert cons == ref_cons
        assert np.array_equal(scores, ref_scores)


def test_rejects_sizes_beyond_the_limits():
    L = sg.lib()
    params = synth.SCORING["batch_10k"][1]
    dummy = C.c_void_p(1)
    too_many = L.spoa_gb300_window_poa_noalloc(2, *params, 0, 257, 500, dummy, dummy, None,
                                               dummy, CONS_CAP, dummy, None, dummy, None)
    too_long = L.spoa_gb300_window_poa_noalloc(2, *params, 0, 10, 641, dummy, dummy, None,
                                               dummy, CONS_CAP, dummy, None, dummy, None)
    assert too_many == 2 and too_long == 2  # SPOA_GB300_ERR_TOO_LARGE
