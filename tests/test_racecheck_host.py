"""Race and undefined-behaviour check of the device code on the CPU.

The SIMT emulation (tests/host/simt_host.h) does the work of a GPU race
checker on the host, with no GPU: built with
-fsanitize=thread, its emulated threads are fibers that the race detector
sees as threads ordered only by what orders them on a GPU (barrier
arrive -> barrier completion, launch -> threads -> launch end, atomics).
tests/host/racecheck_main.cpp drives the window code (one-, two- and
nine-warp CTAs, both widths, the one-warp build, the segmented forward,
clusters of 2, 4 and 8 CTAs, the MSA) and the W-windows-per-CTA loop over every alignment type
and gap model, strands and qualities; any pair of threads that touch the
same shared or global bytes between barriers with one of them writing, and
any undefined behaviour (-fsanitize=undefined: signed overflow, shifts,
misaligned access), fails the test.  The same driver built with
-fsanitize=address and SPOA_GB300_HOST_REDZONE puts a poisoned red zone
after every region of the device arenas (poa_device.cuh), so an access
past a region (a write that on the GPU would land in the next region of
the arena, unnoticed) fails it too.  Planted mistakes in
tests/host/simt_selftest.cpp show that both detectors see one.
"""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

HOST = os.path.join(ROOT, "tests", "host")
BUILD = os.path.join(HOST, "_build")
FLAGS = ["g++", "-std=c++20", "-O1", "-g", "-fsanitize=thread,undefined",
         "-fno-sanitize-recover=undefined"]
ASAN = ["g++", "-std=c++20", "-O1", "-g", "-fsanitize=address,undefined",
        "-fno-sanitize-recover=undefined", "-DSPOA_GB300_HOST_REDZONE"]


@pytest.fixture(scope="module")
def sanitizers():
    """Skips unless g++ builds and runs a -fsanitize=thread,undefined program
    (probed when the first test of this file runs, not at collection)."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    os.makedirs(BUILD, exist_ok=True)
    probe = os.path.join(BUILD, "tsan_probe")
    r = subprocess.run(FLAGS + ["-x", "c++", "-", "-o", probe], input="int main() {}",
                       text=True, capture_output=True)
    if r.returncode != 0 or subprocess.run([probe]).returncode != 0:
        pytest.skip("g++ with ThreadSanitizer not available")
    r = subprocess.run(ASAN + ["-x", "c++", "-", "-o", probe], input="int main() {}",
                       text=True, capture_output=True)
    if r.returncode != 0 or subprocess.run([probe]).returncode != 0:
        pytest.skip("g++ with AddressSanitizer not available")


def _sources_mtime():
    """Newest change of the files these programs compile: the host test
    sources and the device code's headers."""
    import glob
    files = glob.glob(os.path.join(HOST, "*.cpp")) + glob.glob(os.path.join(HOST, "*.h")) + \
        glob.glob(os.path.join(ROOT, "spoa_gb300", "csrc", "*.cuh"))
    return max(os.path.getmtime(f) for f in files)


def _build_all(targets):
    """targets: (source, output, extra flags, base flags) built in parallel
    (those older than their sources)."""
    newest = _sources_mtime()
    targets = [t for t in targets if not os.path.exists(t[1]) or os.path.getmtime(t[1]) < newest]
    procs = [subprocess.Popen(base + extra + [src, "-o", out], stderr=subprocess.PIPE,
                              text=True) for src, out, extra, base in targets]
    for p in procs:
        _, err = p.communicate()
        assert p.returncode == 0, err


def _report(r):
    return (r.stdout + r.stderr)[-4000:]


def test_detectors_see_planted_mistakes(sanitizers):
    src = os.path.join(HOST, "simt_selftest.cpp")
    tsan, asan = os.path.join(BUILD, "simt_selftest_tsan"), os.path.join(BUILD, "simt_selftest_asan")
    _build_all([(src, tsan, [], FLAGS), (src, asan, [], ASAN)])
    for exe in (tsan, asan):
        ok = subprocess.run([exe, "ok"], capture_output=True, text=True, timeout=120)
        assert ok.returncode == 0 and "ERROR" not in ok.stderr, _report(ok)
        assert "WARNING: ThreadSanitizer" not in ok.stderr, _report(ok)
    bad = subprocess.run([tsan, "race"], capture_output=True, text=True, timeout=120)
    assert bad.returncode != 0
    assert "WARNING: ThreadSanitizer: data race" in bad.stderr
    assert "simt_selftest.cpp" in bad.stderr
    bad = subprocess.run([asan, "redzone"], capture_output=True, text=True, timeout=120)
    assert bad.returncode != 0
    assert "AddressSanitizer: use-after-poison" in bad.stderr
    assert "simt_selftest.cpp" in bad.stderr


def test_device_code_has_no_races_overruns_or_undefined_behaviour(sanitizers):
    src = os.path.join(HOST, "racecheck_main.cpp")
    exes = {name: os.path.join(BUILD, name) for name in
            ("racecheck_window", "racecheck_mw", "redzone_window", "redzone_mw")}
    _build_all([(src, exes["racecheck_window"], [], FLAGS),
                (src, exes["racecheck_mw"], ["-DRACECHECK_MW"], FLAGS),
                (src, exes["redzone_window"], [], ASAN),
                (src, exes["redzone_mw"], ["-DRACECHECK_MW"], ASAN)])
    procs = [subprocess.Popen([exe], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
             for exe in exes.values()]
    for p in procs:
        out, err = p.communicate(timeout=900)
        r = subprocess.CompletedProcess(p.args, p.returncode, out, err)
        assert "WARNING: ThreadSanitizer" not in err, _report(r)
        assert "ERROR: AddressSanitizer" not in err, _report(r)
        assert "runtime error" not in err, _report(r)
        assert p.returncode == 0 and out.strip().endswith("statuses ok"), _report(r)


def test_graph_code_and_gfa_writer_under_asan_and_ubsan(sanitizers):
    """The parts of the product's code the driver above does not run -- the
    device graph code's Subgraph and graph loading, and the GFA writer --
    rebuilt for the host with AddressSanitizer (arena red zones) and
    UndefinedBehaviorSanitizer and run through their CPU tests in a child
    process that preloads the ASan runtime: an overrun or undefined
    behaviour ends it with a report."""
    import sys
    libasan = subprocess.run(["g++", "-print-file-name=libasan.so"], capture_output=True,
                             text=True).stdout.strip()
    if not os.path.isabs(libasan) or not os.path.exists(libasan):
        pytest.skip("no shared ASan runtime to preload")
    env = dict(os.environ, SPOA_HOST_SANITIZE="1", LD_PRELOAD=libasan,
               ASAN_OPTIONS="detect_leaks=0")
    r = subprocess.run(
        [sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider", "-m", "not gpu",
         "tests/test_device_graph_host.py", "tests/test_gfa_text.py"],
        cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    out = r.stdout + r.stderr
    assert "ERROR: AddressSanitizer" not in out and "runtime error" not in out, _report(r)
    assert r.returncode == 0 and " passed" in r.stdout, _report(r)


def test_oracle_under_asan_and_ubsan(sanitizers):
    """The oracle itself (the C restatement every parity test trusts),
    built with AddressSanitizer and UndefinedBehaviorSanitizer
    (SPOA_ORACLE_SANITIZE=1) and run through its tests against the recorded
    reference windows, slices and saved graphs in a child process that
    preloads the ASan runtime."""
    import sys
    libasan = subprocess.run(["g++", "-print-file-name=libasan.so"], capture_output=True,
                             text=True).stdout.strip()
    if not os.path.isabs(libasan) or not os.path.exists(libasan):
        pytest.skip("no shared ASan runtime to preload")
    env = dict(os.environ, SPOA_ORACLE_SANITIZE="1", LD_PRELOAD=libasan,
               ASAN_OPTIONS="detect_leaks=0")
    r = subprocess.run(
        [sys.executable, "-m", "pytest", "-q", "-s", "-x", "-p", "no:cacheprovider",
         "tests/test_oracle.py", "-k", "not spoa_test and not random"],
        cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    out = r.stdout + r.stderr
    assert "ERROR: AddressSanitizer" not in out and "runtime error" not in out, _report(r)
    assert r.returncode == 0 and " passed" in r.stdout, _report(r)
