"""The batched loop with W windows per CTA (spoa_gb300/csrc/poa_batch_mw.cuh)
run on the host by the SIMT emulation (tests/host/batch_mw_host.cpp): one
CTA takes every window of a small batch from the queue; each window's read
scores, strand choices and consensus must equal the oracle's, for W = 2
(one strand, quality weights) and W = 4 (strand-ambiguous).  (W = 1 is the one-window loop of
the batched kernel; tests/test_window_host.py covers its device code.)"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import ROOT, host_library, random_test_window
from oracle import pyoracle as po
from spoa_gb300 import synth

SRC = os.path.join(ROOT, "tests", "host", "batch_mw_host.cpp")
OUT = os.path.join(ROOT, "tests", "host", "_build", "libbatch_mw_host.so")
CSRC = os.path.join(ROOT, "spoa_gb300", "csrc")


@pytest.fixture(scope="module")
def mw():
    deps = [os.path.join(ROOT, "tests", "host", "simt_host.h")] + [
        os.path.join(CSRC, f) for f in ("poa_device.cuh", "poa_dp.cuh", "poa_window.cuh",
                                        "poa_batch_mw.cuh")]
    L = C.CDLL(host_library(SRC, OUT, deps, "c++20", "-O1"))
    I32, U32, P = C.c_int32, C.c_uint32, C.c_void_p
    L.mw_run.argtypes = [I32] * 8 + [U32, P, C.c_char_p, P, P, P, P, C.c_char_p, P, P, P,
                                     C.c_char_p]
    return L


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def run_mw(L, windows, type_, params, W, strand, quals=None):
    reads = [r for w in windows for r in w]
    wro = np.zeros(len(windows) + 1, np.uint32)
    wro[1:] = np.cumsum([len(w) for w in windows])
    off = np.zeros(len(reads) + 1, np.uint64)
    off[1:] = np.cumsum([len(r) for r in reads])
    st = np.full(len(windows), 1 if strand else 0, np.int8)
    scores, rev = np.zeros(len(reads), np.int32), np.zeros(len(reads), np.uint8)
    coff = np.zeros(len(windows) + 1, np.uint64)
    coff[1:] = np.cumsum([4 * max(len(r) for r in w) + 64 for w in windows])
    cons = C.create_string_buffer(int(coff[-1]) + 1)
    clen = np.zeros(len(windows), np.uint32)
    status = np.full(len(windows), -1, np.int32)
    L.mw_run(type_, *params, W, len(windows), _ptr(wro), b"".join(reads), _ptr(off), _ptr(st),
             _ptr(scores), _ptr(rev), cons, _ptr(coff), _ptr(clen), _ptr(status),
             b"".join(q for w in quals for q in w) if quals else None)
    return (status.tolist(), scores.tolist(), rev.tolist(),
            [cons.raw[int(coff[w]):int(coff[w]) + int(clen[w])].decode()
             for w in range(len(windows))])


@pytest.mark.parametrize("W,strand,with_quals", [(2, False, True), (4, True, False)])
def test_windows_per_cta_match_the_oracle(mw, W, strand, with_quals):
    rng = np.random.default_rng(77)
    windows = [synth.random_window(rng, 50 + 9 * k, 2 + k % 5, err=0.12) for k in range(7)]
    quals = ([[bytes(rng.integers(33, 75, size=len(r)).astype(np.uint8)) for r in w]
              for w in windows] if with_quals else None)
    params = synth.SCORING["batch_10k"][1]
    status, scores, rev, cons = run_mw(mw, windows, 2, params, W, strand, quals)
    assert status == [0] * len(windows)
    r0 = 0
    for w, win in enumerate(windows):
        ref = po.run_window(2, *params, win, quals[w] if quals else None,
                            strand_ambiguous=strand, with_msa=False)
        n = len(win)
        assert scores[r0:r0 + n] == ref.scores, (W, strand, w)
        assert rev[r0:r0 + n] == [int(x) for x in ref.reversed], (W, strand, w)
        assert cons[w] == ref.consensus, (W, strand, w)
        r0 += n


@pytest.mark.parametrize("W,type_,params", [(2, 1, (5, -4, -8, -6, -8, -6)),
                                             (4, 0, (5, -4, -8, -8, -8, -8)),
                                             (4, 1, (5, -4, -8, -6, -10, -4))])
def test_other_alignment_types_and_gap_models(mw, W, type_, params):
    """NW affine, SW linear and NW convex windows of the polishing shape
    (450-550 bases) on W slots, both strands, against the oracle."""
    windows = [synth.batch_window(880 + k).reads[:5] for k in range(W + 1)]
    status, scores, rev, cons = run_mw(mw, windows, type_, params, W, True)
    assert status == [0] * len(windows)
    r0 = 0
    for w, win in enumerate(windows):
        ref = po.run_window(type_, *params, win, strand_ambiguous=True, with_msa=False)
        n = len(win)
        assert scores[r0:r0 + n] == ref.scores, (W, type_, w)
        assert rev[r0:r0 + n] == [int(x) for x in ref.reversed], (W, type_, w)
        assert cons[w] == ref.consensus, (W, type_, w)
        r0 += n


def test_fewer_windows_than_slots(mw):
    """One window on a CTA of four slots: the empty slots stay idle."""
    rng = np.random.default_rng(5)
    windows = [synth.random_window(rng, 70, 4, err=0.1)]
    params = synth.SCORING["batch_10k"][1]
    status, scores, rev, cons = run_mw(mw, windows, 2, params, 4, False)
    ref = po.run_window(2, *params, windows[0], with_msa=False)
    assert status == [0] and scores == ref.scores and cons == [ref.consensus]


def test_recorded_windows_through_the_w_windows_loop(mw, ref_windows):
    """The 200 recorded windows of up to 12 reads of up to 512 bases (N
    bases, qualities, both strands, long insertions), grouped by scoring,
    type, strand mode and qualities into batches that run with 2 or 4
    windows per CTA, against the oracle window by window."""
    groups = {}
    for rec in ref_windows:
        if max(len(r) for r in rec["reads"]) > 512 or len(rec["reads"]) > 12:
            continue
        key = (tuple(rec["params"]), rec["type"], bool(rec["quals"]), rec["strand_ambiguous"])
        groups.setdefault(key, []).append(rec)
    done = 0
    for g, ((params, type_, has_q, strand), recs) in enumerate(sorted(groups.items())):
        W = 2 if g % 2 else 4
        windows = [[r.encode() for r in rec["reads"]] for rec in recs]
        quals = ([[q.encode() for q in rec["quals"]] for rec in recs] if has_q else None)
        status, scores, rev, cons = run_mw(mw, windows, type_, params, W, strand, quals)
        assert status == [0] * len(windows), (params, type_, W)
        r0 = 0
        for w, win in enumerate(windows):
            ref = po.run_window(type_, *params, win, quals[w] if quals else None,
                                strand_ambiguous=strand, with_msa=False)
            n = len(win)
            assert scores[r0:r0 + n] == ref.scores, (recs[w].get("name"), W)
            assert rev[r0:r0 + n] == [int(x) for x in ref.reversed], (recs[w].get("name"), W)
            assert cons[w] == ref.consensus, (recs[w].get("name"), W)
            r0 += n
            done += 1
    assert done == 200


def test_random_windows_through_the_w_windows_loop(mw):
    """Seeded random windows (alphabets of 2 to 20 letters, empty reads,
    error rates up to 60 %, qualities) with random scoring and type, in
    batches of W + 1 windows on W = 2 and 4 slots, against the oracle; a
    window that needs 32-bit scores reports it (this loop is 16-bit only)
    and is left out of the comparison."""
    rng = np.random.Generator(np.random.PCG64(404))
    done = 0
    for b in range(24):
        W = 2 if b % 2 else 4
        params = (int(rng.integers(0, 11)), int(rng.integers(-10, 1)),
                  *(int(x) for x in -rng.integers(0, 13, size=4)))
        type_, strand = int(rng.integers(0, 3)), bool(b % 3 == 0)
        windows = []
        while len(windows) < W + 1:
            reads = random_test_window(rng)
            if any(reads):
                windows.append(reads)
        quals = ([[bytes((rng.integers(0, 41, size=len(r)) + 33).astype(np.uint8)) for r in w]
                  for w in windows] if b % 4 == 1 else None)
        status, scores, rev, cons = run_mw(mw, windows, type_, params, W, strand, quals)
        r0 = 0
        for w, win in enumerate(windows):
            n = len(win)
            if status[w] == 11:  # needs the 32-bit kernel
                r0 += n
                continue
            assert status[w] == 0, (b, w, status[w])
            ref = po.run_window(type_, *params, win, quals[w] if quals else None,
                                strand_ambiguous=strand, with_msa=False)
            assert scores[r0:r0 + n] == ref.scores, (b, w)
            assert rev[r0:r0 + n] == [int(x) for x in ref.reversed], (b, w)
            assert cons[w] == ref.consensus, (b, w)
            r0 += n
            done += 1
    assert done >= 60
