import gzip
import hashlib
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def host_library(src: str, out: str, deps, std: str, opt: str) -> str:
    """Builds a host test library from `src` (rebuilt when a dependency is
    newer) and returns its path.  With SPOA_HOST_SANITIZE=1 in the
    environment it is built with AddressSanitizer (arena red zones:
    SPOA_GB300_HOST_REDZONE) and UndefinedBehaviorSanitizer, no recovery,
    into a file of its own, for a process that preloads the ASan runtime:
    an overrun or undefined behaviour of the product code it compiles ends
    the process with a report."""
    import shutil
    import subprocess
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    flags = ["g++", f"-std={std}", opt, "-shared", "-fPIC", "-pthread"]
    if os.environ.get("SPOA_HOST_SANITIZE") == "1":
        flags += ["-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
                  "-DSPOA_GB300_HOST_REDZONE"]
        out = out.replace(".so", "_asan.so")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    if not os.path.exists(out) or any(os.path.getmtime(d) > os.path.getmtime(out)
                                      for d in [src] + list(deps)):
        subprocess.run(flags + [src, "-o", out], check=True)
    return out


def random_test_window(rng):
    """A window whose corners the recorded ones may not reach: 1-20 letter
    alphabets, reads of 0-200 bases (empty ones included), depth 1-8, error
    rates up to 60 %, random qualities."""
    alphabets = (b"ACGT", b"ACGTN", b"AC", b"ACDEFGHIKLMNPQRSTVWY")
    alpha = alphabets[int(rng.integers(len(alphabets)))]
    tpl = rng.choice(list(alpha), size=int(rng.integers(1, 200)))
    err = float(rng.choice([0.0, 0.05, 0.15, 0.6]))
    reads = []
    for _ in range(int(rng.integers(1, 9))):
        if rng.random() < 0.05:
            reads.append(b"")
            continue
        out = []
        for b in tpl:
            u = rng.random()
            if u < err / 3:
                continue
            if u < 2 * err / 3:
                out.append(int(rng.choice(list(alpha))))
            out.append(int(rng.choice(list(alpha))) if u < err else int(b))
        s = bytes(out[:200])
        if rng.random() < 0.2 and len(s) > 4:
            s = s[int(rng.integers(0, len(s) // 2)):]
        reads.append(s)
    return reads


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def sha(text: str) -> str:
    return hashlib.sha256(text.encode()).hexdigest()


def canon_alignment(arr) -> str:
    return " ".join(f"{int(a)},{int(b)}" for a, b in arr)


@pytest.fixture(scope="session")
def sample_reads():
    with gzip.open(os.path.join(GOLDEN, "sample_reads.tsv.gz"), "rt") as fh:
        rows = [ln.rstrip("\n").split("\t") for ln in fh if ln.strip()]
    return [(s.encode(), q.encode()) for s, q in rows]


@pytest.fixture(scope="session")
def spoa_test_cases():
    with open(os.path.join(GOLDEN, "spoa_test_cases.json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="session")
def spoa_test_outputs():
    with open(os.path.join(GOLDEN, "spoa_test_outputs.json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="session")
def ref_windows():
    with gzip.open(os.path.join(GOLDEN, "ref_windows.json.gz"), "rt") as fh:
        return json.load(fh)


@pytest.fixture(scope="session")
def slice_windows():
    with gzip.open(os.path.join(GOLDEN, "slice_windows.json.gz"), "rt") as fh:
        return json.load(fh)


@pytest.fixture(scope="session")
def persist_windows():
    with gzip.open(os.path.join(GOLDEN, "persist_windows.json.gz"), "rt") as fh:
        return json.load(fh)


def check_slices(expect, scores, alignments, subgraphs, consensus, msa):
    """Compare one backbone window run through Subgraph/UpdateAlignment
    against a recorded reference run (subgraphs: driver lines per slice)."""
    assert list(scores) == expect["scores"]
    assert [sha(canon_alignment(a)) for a in alignments] == expect["aln_sha"]
    for got, want in zip(subgraphs, expect["subgraph_first"]):
        assert got == want
    assert [{k: sha(v) for k, v in x.items()} for x in subgraphs] == expect["subgraph_sha"]
    assert consensus == expect["consensus"]
    assert sha("\n".join(msa)) == expect["msa_sha"]


def check_against_expect(expect, scores, reversed_, alignments, consensus, msa, gfa):
    """Compare one window's outputs against a recorded reference run."""
    assert list(scores) == expect["scores"]
    assert [int(x) for x in reversed_] == expect["reversed"]
    assert [len(a) for a in alignments] == expect["n_pairs"]
    assert [sha(canon_alignment(a)) for a in alignments] == expect["aln_sha"]
    assert consensus == expect["consensus"]
    assert sha("\n".join(msa)) == expect["msa_sha"]
    if gfa is not None:
        assert sha("\n".join(gfa)) == expect["gfa_sha"]
