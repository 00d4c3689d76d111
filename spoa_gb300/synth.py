"""Seeded synthetic POA windows with the shapes of the five workloads.

Every window w of a workload is generated from its own numpy PCG64 stream
seeded with ``base_seed + w``, so a window is identical wherever it is
regenerated (GPU path, oracle, reference driver).  Reads are uppercase ACGT
bytes; no public dataset is used or imitated.

Error model per template base (shared by all workloads, rates per workload):
  deletion with p_del (base dropped), otherwise substitution with p_sub (one
  of the three other bases, uniformly), otherwise kept; then an insertion of
  one random base with p_ins.  In the long-window workload an inserted base
  repeats the preceding base with weight 3 against weight 1 for each of the
  other three bases (a 3x homopolymer-extension bias).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)
_COMP = np.zeros(256, np.uint8)
for _a, _b in zip(b"ACGT", b"TGCA"):
    _COMP[_a] = _b


@dataclass
class Window:
    reads: list            # list[bytes]
    type: int              # 0 SW, 1 NW, 2 OV
    strand_ambiguous: bool = False


# Scoring of each workload (m, n, g, e, q, c) and alignment type.
SCORING = {
    "single_500": (1, (5, -4, -8, -6, -8, -6)),        # NW affine (q=g, c=e)
    "long_10k": (0, (5, -4, -8, -6, -10, -4)),         # SW convex
    "batch_10k": (2, (5, -4, -8, -6, -10, -4)),        # OV convex default
    "uneven_2k": (None, (5, -4, -8, -6, -8, -6)),      # NW/OV per window, affine
}


def _mutate(rng: np.random.Generator, tpl: np.ndarray, p_sub: float, p_ins: float,
            p_del: float, homopolymer_bias: bool = False) -> bytes:
    n = tpl.size
    u = rng.random(n)
    dele = u < p_del
    sub = (~dele) & (u < p_del + p_sub)
    base = tpl.copy()
    if sub.any():
        idx = np.searchsorted(ACGT, base[sub])
        base[sub] = ACGT[(idx + rng.integers(1, 4, size=int(sub.sum()))) % 4]
    ins = rng.random(n) < p_ins
    ins_base = ACGT[rng.integers(0, 4, size=n)]
    if homopolymer_bias and ins.any():
        # weight 3 for the preceding base, 1 for each other base
        pick = rng.random(n) < 0.5
        ins_base = np.where(pick, base, ins_base)
    slots = np.zeros((n, 2), np.uint8)
    keep = np.zeros((n, 2), bool)
    slots[:, 0] = base
    keep[:, 0] = ~dele
    slots[:, 1] = ins_base
    keep[:, 1] = ins
    out = slots.reshape(-1)[keep.reshape(-1)]
    if out.size == 0:
        out = tpl[:1].copy()
    return out.tobytes()


def revcomp(read: bytes) -> bytes:
    a = np.frombuffer(read, np.uint8)
    return _COMP[a[::-1]].tobytes()


def single_500(seed: int = 1) -> Window:
    """500-nt template, 30 full-length reads, 6% sub / 3% ins / 3% del; NW."""
    rng = np.random.Generator(np.random.PCG64(seed))
    tpl = ACGT[rng.integers(0, 4, size=500)]
    reads = [_mutate(rng, tpl, 0.06, 0.03, 0.03) for _ in range(30)]
    return Window(reads=reads, type=1)


def long_10k(seed: int = 2, n_reads: int = 40, tpl_len: int = 10000,
             min_len: int = 2000) -> Window:
    """10-kb template, reads are random substrings of length U[2k, 10k]
    with 2% sub / 4% ins / 4% del and homopolymer-biased insertions; SW."""
    rng = np.random.Generator(np.random.PCG64(seed))
    tpl = ACGT[rng.integers(0, 4, size=tpl_len)]
    reads = []
    for _ in range(n_reads):
        ln = int(rng.integers(min_len, tpl_len + 1))
        st = int(rng.integers(0, tpl_len - ln + 1))
        reads.append(_mutate(rng, tpl[st:st + ln], 0.02, 0.04, 0.04, homopolymer_bias=True))
    return Window(reads=reads, type=0)


def batch_window(w: int, base_seed: int = 3_000_000) -> Window:
    """One polishing window: L ~ U[450, 550], depth U[10, 60], 3% sub,
    2.5% ins, 2.5% del; 20% of reads lose U[10%, 50%] of their length at a
    random end; OV."""
    rng = np.random.Generator(np.random.PCG64(base_seed + w))
    ln = int(rng.integers(450, 551))
    depth = int(rng.integers(10, 61))
    tpl = ACGT[rng.integers(0, 4, size=ln)]
    reads = []
    for _ in range(depth):
        r = _mutate(rng, tpl, 0.03, 0.025, 0.025)
        if rng.random() < 0.2:
            cut = int(len(r) * rng.uniform(0.10, 0.50))
            r = r[cut:] if rng.random() < 0.5 else r[:len(r) - cut]
            if not r:
                r = tpl[:1].tobytes()
        reads.append(r)
    return Window(reads=reads, type=2)


def uneven_window(w: int, base_seed: int = 4_000_000) -> Window:
    """Uneven window: L log-uniform [100, 5000], depth U[5, 100], NW or OV
    50/50, half of the reads reverse-complemented, strand-ambiguous on; the
    polishing error rates (3% / 2.5% / 2.5%)."""
    rng = np.random.Generator(np.random.PCG64(base_seed + w))
    ln = int(round(np.exp(rng.uniform(np.log(100), np.log(5000)))))
    depth = int(rng.integers(5, 101))
    typ = 1 if rng.random() < 0.5 else 2
    tpl = ACGT[rng.integers(0, 4, size=ln)]
    reads = []
    for _ in range(depth):
        r = _mutate(rng, tpl, 0.03, 0.025, 0.025)
        if rng.random() < 0.5:
            r = revcomp(r)
        reads.append(r)
    return Window(reads=reads, type=typ, strand_ambiguous=True)


def batch_windows(n: int, start: int = 0) -> list:
    return [batch_window(w) for w in range(start, start + n)]


def uneven_windows(n: int, start: int = 0) -> list:
    return [uneven_window(w) for w in range(start, start + n)]


def serving_stream(n: int, rate: float, seed: int = 5) -> list:
    """Poisson arrivals at `rate` windows/s drawn 70/30 from the polishing
    and uneven distributions.  Returns [(arrival_s, Window)]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    out = []
    for k in range(n):
        if rng.random() < 0.7:
            win = batch_window(int(rng.integers(0, 1 << 30)))
        else:
            win = uneven_window(int(rng.integers(0, 1 << 30)))
        out.append((float(t[k]), win))
    return out


def random_window(rng: np.random.Generator, ln: int, depth: int, err: float = 0.1,
                  alphabet: bytes = b"ACGT") -> list:
    """Small adversarial window for parity tests: high error, arbitrary
    alphabet (may include characters that appear late)."""
    alpha = np.frombuffer(alphabet, np.uint8)
    tpl = alpha[rng.integers(0, alpha.size, size=ln)]
    reads = []
    for _ in range(depth):
        n = tpl.size
        u = rng.random(n)
        dele = u < err / 3
        sub = (~dele) & (u < 2 * err / 3)
        base = tpl.copy()
        base[sub] = alpha[rng.integers(0, alpha.size, size=int(sub.sum()))]
        ins = rng.random(n) < err / 3
        slots = np.stack([base, alpha[rng.integers(0, alpha.size, size=n)]], 1)
        keep = np.stack([~dele, ins], 1)
        r = slots.reshape(-1)[keep.reshape(-1)]
        if r.size == 0:
            r = tpl[:1]
        if rng.random() < 0.3:
            cut = int(r.size * rng.uniform(0.0, 0.6))
            r = r[cut:] if rng.random() < 0.5 else r[:r.size - cut]
            if r.size == 0:
                r = tpl[:1]
        reads.append(r.tobytes())
    return reads


def slice_window(seed: int, base_seed: int = 6_000_000):
    """A polishing window with a backbone, for Graph::Subgraph: read 0 is
    the template (L ~ U[200, 600]) and is added whole, so its bases are graph
    nodes 0..L-1; each later read (depth U[5, 25]) copies a random span of
    U[30%, 100%] of the template with 3% sub / 2.5% ins / 2.5% del.  Returns
    (reads, slices): per read after the first the backbone node range
    (begin, end) its span covers, except every 7th read (-1, -1: align to the
    whole graph), every 11th an inverted range (an empty subgraph) and every
    13th a single node."""
    rng = np.random.Generator(np.random.PCG64(base_seed + seed))
    ln = int(rng.integers(200, 601))
    tpl = ACGT[rng.integers(0, 4, size=ln)]
    reads, slices = [tpl.tobytes()], []
    for r in range(1, int(rng.integers(5, 26)) + 1):
        span = int(ln * rng.uniform(0.3, 1.0))
        st = int(rng.integers(0, ln - span + 1))
        reads.append(_mutate(rng, tpl[st:st + span], 0.03, 0.025, 0.025))
        if r % 7 == 0:
            slices.append((-1, -1))
        elif r % 11 == 0:
            slices.append((st + span - 1, st))
        elif r % 13 == 0:
            slices.append((st, st))
        else:
            slices.append((st, st + span - 1))
    return reads, slices
