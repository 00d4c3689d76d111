"""The batched kernel's device code for one window (poa_window.cuh: forward
pass with its CTA scans, traceback, strand choice, AddAlignment, sort,
consensus) run on the host by a SIMT emulation (tests/host/simt_host.h,
tests/host/window_host.cpp) and compared with the oracle: every score,
strand choice, alignment and the consensus, for one- and two-warp CTAs and
both score widths."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, host_library, random_test_window
from oracle import pyoracle as po

SRC = os.path.join(ROOT, "tests", "host", "window_host.cpp")
OUT = os.path.join(ROOT, "tests", "host", "_build", "libwindow_host.so")
CSRC = os.path.join(ROOT, "spoa_gb300", "csrc")
NEEDS_WIDE = 11


@pytest.fixture(scope="module")
def wh():
    deps = [os.path.join(ROOT, "tests", "host", "simt_host.h")] + [
        os.path.join(CSRC, f) for f in ("poa_device.cuh", "poa_dp.cuh", "poa_window.cuh")]
    L = C.CDLL(host_library(SRC, OUT, deps, "c++20", "-O1"))
    I32, U32, P = C.c_int32, C.c_uint32, C.c_void_p
    L.wh_run.argtypes = [I32] * 9 + [U32, U32, C.c_char_p, P, C.c_char_p, I32, P, P, P,
                                     C.c_uint64, P, C.c_char_p, U32, P, C.c_char_p,
                                     C.c_uint64, P]
    L.wh_run_cl.argtypes = [I32] * 8 + [U32, U32, C.c_char_p, P, C.c_char_p, I32, P, P, P,
                                        C.c_uint64, P, C.c_char_p, U32, P]
    return L


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def run_host(L, type_, params, reads, quals, strand, cpt, nt, wide, msa=None):
    """One window through the emulated CTA; with msa=[] the window's MSA
    rows (the batched kernel's window_msa) are appended to that list."""
    off = np.zeros(len(reads) + 1, np.uint64)
    off[1:] = np.cumsum([len(r) for r in reads])
    nr = len(reads)
    scores, rev = np.zeros(nr, np.int32), np.zeros(nr, np.int32)
    cap = int(off[-1]) * 2 + 64 * nr + 64
    aln = np.zeros(2 * cap, np.int32)
    aoff = np.zeros(nr + 1, np.uint64)
    cons = C.create_string_buffer(int(off[-1]) + 16)
    clen = C.c_uint32()
    mcap = (nr + 1) * (int(off[-1]) + 1)
    mbuf = C.create_string_buffer(mcap) if msa is not None else None
    dims = (C.c_uint32 * 2)()
    st = L.wh_run(type_, *params, 1 if wide else 0, cpt, nt, nr, b"".join(reads), _ptr(off),
                  b"".join(quals) if quals else None, 1 if strand else 0, _ptr(scores), _ptr(rev),
                  _ptr(aln), cap, _ptr(aoff), cons, len(cons), C.byref(clen), mbuf, mcap, dims)
    alns = [aln[2 * int(aoff[r]):2 * int(aoff[r + 1])].reshape(-1, 2) for r in range(nr)]
    if msa is not None and st == 0:
        rows, cols = dims[0], dims[1]
        msa.extend(mbuf.raw[k * cols:(k + 1) * cols].decode() for k in range(rows))
    return st, scores.tolist(), rev.tolist(), alns, cons.raw[:clen.value].decode()


def _check_window(L, rec, cpt=8, wide=False, with_msa=False):
    reads = [r.encode() for r in rec["reads"]]
    quals = [q.encode() for q in rec["quals"]] if rec["quals"] else None
    lmax = max(len(r) for r in reads)
    nt = 32 * max(1, -(-lmax // (cpt * 32)))
    strand = rec["strand_ambiguous"]
    msa = [] if with_msa else None
    st, scores, rev, alns, cons = run_host(L, rec["type"], rec["params"], reads, quals, strand,
                                           cpt, nt, wide, msa)
    if st == NEEDS_WIDE:
        msa = [] if with_msa else None
        st, scores, rev, alns, cons = run_host(L, rec["type"], rec["params"], reads, quals,
                                               strand, cpt, nt, True, msa)
    assert st == 0, (rec.get("name"), st)
    ref = po.run_window(rec["type"], *rec["params"], reads, quals, strand_ambiguous=strand,
                        with_msa=with_msa)
    if with_msa:
        assert msa == ref.msa, rec.get("name")
    assert scores == ref.scores, rec.get("name")
    assert rev == [int(x) for x in ref.reversed], rec.get("name")
    for a, b in zip(alns, ref.alignments):
        assert np.array_equal(a, b), rec.get("name")
    assert cons == ref.consensus, rec.get("name")
    return nt


def test_window_device_code_matches_the_oracle(wh, ref_windows):
    """Every recorded window of up to 12 reads of up to 512 bases (200 of
    the fixture's 209: adversarial lengths, N bases, qualities, both
    strands, long insertions) through the emulated CTA, its MSA included;
    reads up to 256 columns take one warp, longer ones two."""
    nts, strands, done = set(), 0, 0
    for rec in ref_windows:
        if max(len(r) for r in rec["reads"]) > 512 or len(rec["reads"]) > 12:
            continue
        nts.add(_check_window(wh, rec, with_msa=True))
        strands += rec["strand_ambiguous"]
        done += 1
    assert done == 200 and nts == {32, 64} and strands >= 40


def test_two_warp_ctas_and_int32_rows(wh):
    """Two-warp CTAs (the scans' cross-warp carry through shared memory) on
    one synthetic window per gap model and alignment type, each on both
    lane widths (the 32-bit kernel runs 16-bit-width reads with the 16-lane
    semantics)."""
    from spoa_gb300 import synth
    w = synth.long_10k(5, n_reads=3, tpl_len=330, min_len=290)
    gaps = ((5, -4, -8, -8, -8, -8), (5, -4, -8, -6, -8, -6), (5, -4, -8, -6, -10, -4))
    for k, params in enumerate(gaps):
        rec = {"reads": [r.decode() for r in w.reads], "quals": None, "type": k,
               "params": list(params), "strand_ambiguous": False, "name": f"{k}{params}"}
        assert _check_window(wh, rec) == 64
        assert _check_window(wh, rec, wide=True) == 64


def test_segmented_rows(wh):
    """The segmented forward (dp_forward_seg: two 12-column strips per
    thread, the scan carries handed from strip to strip) on 32-bit rows."""
    from spoa_gb300 import synth
    w = synth.long_10k(8, n_reads=3, tpl_len=560, min_len=500)
    reads = list(w.reads)
    for typ, params in ((0, (5, -4, -8, -6, -10, -4)), (1, (5, -4, -8, -6, -8, -6))):
        st, scores, rev, alns, cons = run_host(wh, typ, params, reads, None, False, -12, 32, True)
        assert st == 0
        ref = po.run_window(typ, *params, reads, with_msa=False)
        assert scores == ref.scores
        for a, b in zip(alns, ref.alignments):
            assert np.array_equal(a, b)
        assert cons == ref.consensus


def test_one_warp_build_of_the_forward(wh, ref_windows):
    """The forward pass built for exactly 32 threads (row offsets fixed at
    compile time, scans without the cross-warp path), as the batched kernel
    runs every polishing-sized window, on every recorded window of up to 12
    reads of up to 512 columns (16 columns per thread), both strands
    included."""
    done = 0
    for rec in ref_windows:
        if max(len(r) for r in rec["reads"]) > 512 or len(rec["reads"]) > 12:
            continue
        assert _check_window(wh, rec, cpt=16) == 32
        done += 1
    assert done == 200


def run_host_cl(L, type_, params, reads, quals, strand, cl, nt):
    nr = len(reads)
    off = np.zeros(nr + 1, np.uint64)
    off[1:] = np.cumsum([len(r) for r in reads])
    cap = int(off[-1]) * 2 + 64 * nr + 64
    aln = np.zeros(2 * cap, np.int32)
    aoff = np.zeros(nr + 1, np.uint64)
    cons = C.create_string_buffer(int(off[-1]) + 16)
    clen = C.c_uint32()
    scores = np.zeros(nr, np.int32)
    rev = np.zeros(nr, np.int32)
    qb = b"".join(quals) if quals is not None else None
    st = L.wh_run_cl(type_, *params, cl, nt, nr, b"".join(reads), _ptr(off), qb,
                     1 if strand else 0, _ptr(scores), _ptr(rev), _ptr(aln), cap, _ptr(aoff),
                     cons, len(cons), C.byref(clen))
    alns = [aln[2 * int(aoff[r]):2 * int(aoff[r + 1])].reshape(-1, 2) for r in range(nr)]
    return st, scores.tolist(), rev.tolist(), alns, cons.raw[:clen.value].decode()


def test_cluster_rows(wh):
    """The cluster form of a window (window_read_cl: each row spread over 2,
    4 or 8 emulated CTAs of one or two warps, one exchange of scan tails per
    row and the final reductions crossing CTAs through their shared state
    behind cluster barriers; the serial phases on the lead CTA) against the
    oracle for every alignment type and gap model, both strands, quality
    weights, 32-bit lanes.  The 8-CTA cases leave the last CTAs columns
    beyond the reads (a row narrower than the cluster)."""
    from spoa_gb300 import synth
    short = list(synth.long_10k(12, n_reads=3, tpl_len=420, min_len=380).reads)
    long_ = list(synth.long_10k(13, n_reads=3, tpl_len=860, min_len=800).reads)
    rng = np.random.Generator(np.random.PCG64(12))
    lin, aff, cvx = (5, -4, -8, -8, -8, -8), (5, -4, -8, -6, -8, -6), (5, -4, -8, -6, -10, -4)
    # (scoring, type, CTAs, strand-ambiguous, threads per CTA, qualities, reads):
    # a cluster holds 12 columns per thread, so 2 x 32 threads take 768
    cases = ((lin, 0, 2, False, 32, False, short), (aff, 1, 4, True, 32, False, long_),
             (cvx, 2, 2, False, 32, True, short), (cvx, 0, 4, True, 32, False, short),
             (cvx, 1, 2, True, 64, True, long_), (cvx, 2, 8, True, 32, False, short),
             (aff, 0, 8, False, 32, True, long_))
    for params, typ, cl, strand, nt, with_q, reads in cases:
        rs = reads if not strand else [synth.revcomp(r) if j % 2 else r
                                      for j, r in enumerate(reads)]
        qs = ([bytes((rng.integers(0, 41, size=len(r)) + 33).astype(np.uint8)) for r in rs]
              if with_q else None)
        st, scores, rev, alns, cons = run_host_cl(wh, typ, params, rs, qs, strand, cl, nt)
        case = (params, typ, cl, strand, nt, with_q, len(reads))
        assert st == 0, (case, st)
        ref = po.run_window(typ, *params, rs, qs, strand_ambiguous=strand, with_msa=False)
        assert scores == ref.scores, case
        assert rev == [int(x) for x in ref.reversed], case
        for a, b in zip(alns, ref.alignments):
            assert np.array_equal(a, b), case
        assert cons == ref.consensus, case


def test_mq_path_is_the_best_vector_start(wh):
    """The closed form the cluster forward uses for a Q' carry entering E':
    max over vector starts u' <= u ((u' + 1) % lanes == 0) of
    u' * c + (u - u') * e, -infinity before the first vector start."""
    wh.wh_mq_path.restype = C.c_int32
    wh.wh_mq_path.argtypes = [C.c_int32] * 4
    neg = -(1 << 28)
    rng = np.random.default_rng(5)
    for lanes in (8, 16):
        for c, e in [(-4, -6), (-6, -4), (-5, -5), (-1, -10), (-10, -1), (0, -3)]:
            for u in list(range(0, 70)) + list(rng.integers(0, 6144, 40)):
                starts = [v for v in range(0, u + 1) if (v + 1) % lanes == 0]
                want = max(v * c + (u - v) * e for v in starts) if starts else neg
                assert wh.wh_mq_path(int(u), c, e, lanes) == want, (u, c, e, lanes)


def test_emulation_reports_a_skipped_barrier():
    """The SIMT emulation itself: shuffles, CTA barriers and the split
    cluster barrier give a GPU's values; a thread that leaves before a
    __syncthreads the others wait at (a hang on a GPU) ends the emulated
    launch with a barrier-deadlock report instead of hanging the suite, and
    threads of a CTA that wait at two different __syncthreads (undefined on
    a GPU) end it with both places named."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = os.path.join(ROOT, "tests", "host", "simt_selftest.cpp")
    exe = os.path.join(ROOT, "tests", "host", "_build", "simt_selftest")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    subprocess.run(["g++", "-std=c++20", "-O1", src, "-o", exe], check=True)
    ok = subprocess.run([exe, "ok"], capture_output=True, text=True, timeout=60)
    assert ok.returncode == 0 and ok.stdout.strip() == "ok", ok.stdout
    bad = subprocess.run([exe, "skip"], capture_output=True, text=True, timeout=60)
    assert bad.returncode != 0
    assert "barrier deadlock" in bad.stderr
    assert "thread 0 waits at a CTA barrier" in bad.stderr
    split = subprocess.run([exe, "split"], capture_output=True, text=True, timeout=60)
    assert split.returncode != 0
    assert "meet at different __syncthreads barriers" in split.stderr


def test_recorded_windows_on_32_bit_lanes_and_clusters(wh, ref_windows):
    """The 200 recorded windows of the tests above (N bases, qualities, both
    strands, long insertions) on the 32-bit width of the one-CTA kernel,
    every fourth one through the segmented forward and every second one on a
    cluster of 2 or 4 CTAs (window_read_cl), each against the oracle."""
    done_wide = done_cl = done_seg = 0
    k = 0
    for rec in ref_windows:
        if max(len(r) for r in rec["reads"]) > 512 or len(rec["reads"]) > 12:
            continue
        k += 1
        _check_window(wh, rec, wide=True)
        done_wide += 1
        if k % 4 == 1:  # the segmented forward: two 12-column strips per thread
            reads = [r.encode() for r in rec["reads"]]
            quals = [q.encode() for q in rec["quals"]] if rec["quals"] else None
            st, scores, rev, alns, cons = run_host(wh, rec["type"], rec["params"], reads, quals,
                                                   rec["strand_ambiguous"], -12, 32, True)
            ref = po.run_window(rec["type"], *rec["params"], reads, quals,
                                strand_ambiguous=rec["strand_ambiguous"], with_msa=False)
            assert st == 0 and scores == ref.scores and cons == ref.consensus, rec.get("name")
            for a, b in zip(alns, ref.alignments):
                assert np.array_equal(a, b), rec.get("name")
            done_seg += 1
        if k % 2:
            continue
        reads = [r.encode() for r in rec["reads"]]
        quals = [q.encode() for q in rec["quals"]] if rec["quals"] else None
        strand = rec["strand_ambiguous"]
        cl = 2 if k % 4 else 4
        st, scores, rev, alns, cons = run_host_cl(wh, rec["type"], rec["params"], reads, quals,
                                                  strand, cl, 32)
        assert st == 0, (rec.get("name"), cl, st)
        ref = po.run_window(rec["type"], *rec["params"], reads, quals, strand_ambiguous=strand,
                            with_msa=False)
        assert scores == ref.scores, (rec.get("name"), cl)
        assert rev == [int(x) for x in ref.reversed], (rec.get("name"), cl)
        for a, b in zip(alns, ref.alignments):
            assert np.array_equal(a, b), (rec.get("name"), cl)
        assert cons == ref.consensus, (rec.get("name"), cl)
        done_cl += 1
    assert done_wide == 200 and done_cl == 100 and done_seg == 50


N_RANDOM = int(os.environ.get("SPOA_RANDOM_WINDOWS", "300"))


def test_random_windows_and_scoring_against_the_oracle(wh):
    """Seeded random windows with random scoring (match 0-10, mismatch
    -10-0 and sometimes positive, gap penalties 0 to -12 in all three gap
    models, equal penalties included), every alignment type, strands and
    qualities, through the emulated CTA (the 32-bit width when the
    reference's width rule asks for it) against the oracle, MSA included;
    every fifth one also on a 2-CTA cluster and another fifth through the
    one-warp build."""
    rng = np.random.Generator(np.random.PCG64(2024))
    done = 0
    for k in range(N_RANDOM):
        reads = random_test_window(rng)
        m = int(rng.integers(0, 11))
        n = int(rng.integers(-10, 1)) if rng.random() < 0.9 else int(rng.integers(1, 4))
        g, e, q, c = (int(x) for x in -rng.integers(0, 13, size=4))
        rec = {"reads": [r.decode() for r in reads], "type": int(rng.integers(0, 3)),
               "params": [m, n, g, e, q, c], "strand_ambiguous": bool(rng.random() < 0.3),
               "name": f"random {k}"}
        if rng.random() < 0.3 and any(reads):
            rec["quals"] = ["".join(chr(33 + int(x)) for x in rng.integers(0, 41, size=len(r)))
                            for r in reads]
        else:
            rec["quals"] = None
        if not any(reads):
            continue
        _check_window(wh, rec, with_msa=True)
        done += 1
        if k % 5 == 1:  # the one-warp build of the forward pass
            _check_window(wh, rec, cpt=16)
        if k % 5 == 0:  # the same window on a 2-CTA cluster (32-bit lanes)
            quals = [q.encode() for q in rec["quals"]] if rec["quals"] else None
            st, scores, rev, alns, cons = run_host_cl(wh, rec["type"], rec["params"], reads,
                                                      quals, rec["strand_ambiguous"], 2, 32)
            ref = po.run_window(rec["type"], *rec["params"], reads, quals,
                                strand_ambiguous=rec["strand_ambiguous"], with_msa=False)
            assert st == 0 and scores == ref.scores and cons == ref.consensus, rec["name"]
            assert rev == [int(x) for x in ref.reversed], rec["name"]
            for a, b in zip(alns, ref.alignments):
                assert np.array_equal(a, b), rec["name"]
    assert done >= N_RANDOM * 7 // 8


def test_many_warp_ctas(wh):
    """CTAs of 9, 16 and 32 warps, as the per-call form's latency tiles use
    for long reads (the scans' carries across many warps, rows much wider
    than the reads), against the oracle."""
    from spoa_gb300 import synth
    cases = ((288, 2, (5, -4, -8, -6, -10, -4), 2, 2100, False),
             (512, 1, (5, -4, -8, -8, -8, -8), 3, 900, True),
             (1024, 0, (5, -4, -8, -6, -8, -6), 3, 300, False))
    for nt, typ, params, n_reads, length, strand in cases:
        w = synth.long_10k(nt, n_reads=n_reads, tpl_len=length, min_len=length * 9 // 10)
        reads = list(w.reads)
        if strand:
            reads = [synth.revcomp(r) if j % 2 else r for j, r in enumerate(reads)]
        st, scores, rev, alns, cons = run_host(wh, typ, params, reads, None, strand, 8, nt,
                                               False)
        if st == NEEDS_WIDE:
            st, scores, rev, alns, cons = run_host(wh, typ, params, reads, None, strand, 8, nt,
                                                   True)
        assert st == 0, (nt, st)
        ref = po.run_window(typ, *params, reads, strand_ambiguous=strand, with_msa=False)
        assert scores == ref.scores, nt
        assert rev == [int(x) for x in ref.reversed], nt
        for a, b in zip(alns, ref.alignments):
            assert np.array_equal(a, b), nt
        assert cons == ref.consensus, nt
