"""Served windows (continuous batching): windows submitted over time, each
result identical to the same window run alone and to the oracle."""
import numpy as np
import pytest

import spoa_gb300 as sg
from spoa_gb300 import synth
from oracle import pyoracle as po

PARAMS = synth.SCORING["batch_10k"][1]


def _mix(n, seed):
    """70/30 polishing-shaped (OV, convex) and uneven-shaped windows (NW/OV,
    strand-ambiguous), the uneven ones kept short so the test stays small."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(n):
        if rng.random() < 0.7:
            w = synth.batch_window(10_000 + k)
            out.append((w.reads, 2, False))
        else:
            w = synth.uneven_window(20_000 + k)
            out.append(([r[:700] for r in w.reads[:12]], w.type, True))
    return out


@pytest.mark.skipif(sg.lib().spoa_gb300_device_count() > 0, reason="a GPU is visible")
def test_server_fails_loudly_without_a_gpu():
    with pytest.raises(sg.SpoaError):
        sg.Server(2, *PARAMS)


@pytest.mark.gpu
def test_served_results_are_the_same_alone_and_in_the_mix():
    wins = _mix(40, 1)
    rng = np.random.Generator(np.random.PCG64(2))
    delays = np.sort(rng.uniform(0, 0.05, len(wins)))
    with sg.Server(2, *PARAMS, max_streams=4, gather_seconds=0.002) as sv:
        tickets = [sv.submit(r, t, s, d) for (r, t, s), d in zip(wins, delays)]
        got = [sv.wait(t, timeout=600) for t in tickets]
        stats = sv.stats()
    assert stats["completed"] == len(wins)
    assert stats["launches"] >= 2  # arrivals spread over time: several launches overlap
    for (reads, typ, strand), (st, cons, lat) in zip(wins, got):
        assert st == 0
        assert lat >= 0
        alone = sg.batch_poa([reads], typ, *PARAMS, window_strand=[1 if strand else 0])
        assert alone.consensus[0] == cons
    for (reads, typ, strand), (st, cons, lat) in list(zip(wins, got))[:8]:
        ref = po.run_window(typ, *PARAMS, reads, strand_ambiguous=strand, with_msa=False)
        assert ref.consensus == cons


@pytest.mark.gpu
def test_admission_waits_for_memory():
    """A budget that holds only a few windows at a time: windows queue for
    memory and still all finish with the batched results."""
    wins = _mix(24, 3)
    with sg.Server(2, *PARAMS, memory_budget=400 << 20, max_streams=8) as sv:
        tickets = [sv.submit(r, t, s) for r, t, s in wins]
        got = [sv.wait(t, timeout=600) for t in tickets]
        stats = sv.stats()
    ref = sg.batch_poa([w[0] for w in wins], 2, *PARAMS, window_types=[w[1] for w in wins],
                       window_strand=[1 if w[2] else 0 for w in wins])
    assert [g[1] for g in got] == ref.consensus
    assert all(g[0] == 0 for g in got)
    assert stats["launches"] > 3


@pytest.mark.gpu
def test_wait_timeout_and_unknown_ticket():
    with sg.Server(2, *PARAMS) as sv:
        t = sv.submit(synth.batch_window(5).reads, delay=1.0)
        with pytest.raises(sg.SpoaError) as ex:
            sv.wait(t, timeout=0.05)
        assert ex.value.status == sg.TIMEOUT
        with pytest.raises(sg.SpoaError):
            sv.wait(t + 1000)
        st, cons, lat = sv.wait(t, timeout=120)
        assert st == 0 and cons


@pytest.mark.gpu
def test_long_window_served():
    """Windows of 2-2.4k, 4.2-4.8k and 6.5-7k-column int32 rows through the
    server (thread-block clusters of 2, 4 and 8 CTAs; the two shorter ones
    strand-ambiguous, submitted together), against the oracle."""
    ws = [(synth.long_10k(11, n_reads=3, tpl_len=7200, min_len=6500).reads, False),
          (synth.long_10k(21, n_reads=3, tpl_len=2400, min_len=2000).reads, True),
          (synth.long_10k(22, n_reads=3, tpl_len=4800, min_len=4200).reads, True)]
    ws[1] = ([synth.revcomp(r) if j == 1 else r for j, r in enumerate(ws[1][0])], True)
    with sg.Server(2, *PARAMS) as sv:
        tickets = [sv.submit(reads, 2, strand) for reads, strand in ws]
        got = [sv.wait(t, timeout=600) for t in tickets]
    for (reads, strand), (st, cons, lat) in zip(ws, got):
        assert st == 0
        assert cons == po.run_window(2, *PARAMS, reads, strand_ambiguous=strand,
                                     with_msa=False).consensus


@pytest.mark.gpu
def test_resident_kernel_results_alone_and_in_the_mix():
    """Resident mode: polishing-sized windows go to one persistent kernel fed
    through a ring while it runs, the others are launched; every window's
    consensus equals the same window run alone, arrivals spread over time.
    Two windows that outgrow the resident kernel's arenas (20-letter noisy
    reads) come back from it and finish through the launch path."""
    wins = _mix(40, 5)
    rng = np.random.Generator(np.random.PCG64(79))
    big = [synth.random_window(rng, 300, 40, err=0.6, alphabet=b"ACDEFGHIKLMNPQRSTVWY")
           for _ in range(2)]
    wins = wins[:10] + [(big[0], 2, False)] + wins[10:30] + [(big[1], 2, False)] + wins[30:]
    delays = np.sort(np.random.Generator(np.random.PCG64(6)).uniform(0, 0.05, len(wins)))
    with sg.Server(2, *PARAMS, max_streams=4, resident=True) as sv:
        tickets = [sv.submit(r, t, s, d) for (r, t, s), d in zip(wins, delays)]
        got = [sv.wait(t, timeout=600) for t in tickets]
        stats = sv.stats()
    assert stats["completed"] == len(wins)
    resident = sum(1 for r, _, s in wins if max(len(x) for x in r) <= 640 and not s)
    assert stats["resident_windows"] >= resident
    assert stats["resident_launches"] >= 1
    for (reads, typ, strand), (st, cons, lat) in zip(wins, got):
        assert st == 0
        alone = sg.batch_poa([reads], typ, *PARAMS, window_strand=[1 if strand else 0])
        assert alone.consensus[0] == cons


@pytest.mark.gpu
def test_resident_kernel_leaves_when_idle_and_starts_again():
    """The resident kernel's CTAs leave after 20 ms without work (a bounded
    wait); windows arriving later start it again."""
    wins = [synth.batch_window(30_000 + k).reads for k in range(6)]
    with sg.Server(2, *PARAMS, resident=True) as sv:
        tickets = [sv.submit(w, delay=0.2 * k) for k, w in enumerate(wins)]
        got = [sv.wait(t, timeout=600) for t in tickets]
        stats = sv.stats()
    assert stats["resident_windows"] == len(wins)
    assert stats["resident_launches"] >= 2
    ref = sg.batch_poa(wins, 2, *PARAMS)
    assert [g[1] for g in got] == ref.consensus and all(g[0] == 0 for g in got)
