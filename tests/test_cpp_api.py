"""The C++ drop-in API (include/spoa/*.hpp, spoa_gb300/libspoa.so) driven the
way spoa's own tests drive spoa (test/spoa_test.cpp), by the C++ program
tests/cpp/spoa_api_test.cpp."""
import os
import shutil
import subprocess

import pytest

import spoa_gb300 as sg
from spoa_gb300 import build as sgb
from conftest import sha

DRIVER = sgb.CPPTEST


def _driver():
    if not (os.path.exists(sgb.CPPLIB) and os.path.exists(DRIVER)):
        pytest.skip("C++ API not built (python -m spoa_gb300.build)")
    return DRIVER


def _run(tmp_path, sample_reads, cases, slices=None):
    reads = tmp_path / "reads.tsv"
    reads.write_text("".join(f"{s.decode()}\t{q.decode()}\n" for s, q in sample_reads))
    cf = tmp_path / "cases.txt"
    cf.write_text("".join(
        f"{c['name']} {c['type']} {' '.join(str(x) for x in c['params'])} {int(c['quality'])}\n"
        for c in cases))
    args = [_driver(), str(reads), str(cf)]
    if slices is not None:
        sf = tmp_path / "slices.txt"
        sf.write_text("".join(
            f"S {w['type']} {' '.join(str(x) for x in w['params'])} {len(w['reads'])}\n"
            + "".join(r + "\n" for r in w["reads"])
            + "".join(f"{b} {e}\n" for b, e in w["slices"]) for w in slices))
        args.append(str(sf))
    r = subprocess.run(args, capture_output=True, text=True, timeout=1200)
    return r


@pytest.mark.skipif(shutil.which("nm") is None, reason="nm not available")
def test_library_exports_the_spoa_api():
    if not os.path.exists(sgb.CPPLIB):
        pytest.skip("C++ API not built")
    out = subprocess.run(["nm", "-DC", "--defined-only", sgb.CPPLIB], capture_output=True,
                         text=True, check=True).stdout
    for sym in ["spoa::AlignmentEngine::Create(spoa::AlignmentType, signed char, signed char, signed char)",
                "spoa::AlignmentEngine::Create(spoa::AlignmentType, signed char, signed char, signed char, signed char)",
                "spoa::AlignmentEngine::Create(spoa::AlignmentType, signed char, signed char, signed char, signed char, signed char, signed char)",
                "spoa::AlignmentEngine::Align(",
                "spoa::Graph::AddAlignment(",
                "spoa::Graph::GenerateConsensus[abi:cxx11]()",
                "spoa::Graph::GenerateConsensus[abi:cxx11](std::vector<unsigned int",
                "spoa::Graph::GenerateMultipleSequenceAlignment[abi:cxx11](bool)",
                "spoa::Graph::Clear()", "spoa::Graph::PrintDot(",
                "spoa::Graph::nodes() const", "spoa::Graph::edges() const",
                "spoa::Graph::rank_to_node() const", "spoa::Graph::sequences() const",
                "spoa::Graph::consensus() const", "spoa::Graph::Node::Successor(unsigned int) const",
                "spoa::Graph::Node::Coverage() const",
                "spoa::Graph::Subgraph(unsigned int, unsigned int, std::vector<spoa::Graph::Node const*",
                "spoa::Graph::UpdateAlignment(std::vector<spoa::Graph::Node const*"]:
        assert sym in out, sym
    assert out.count("spoa::Graph::AddAlignment(") == 6


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_cereal_archives_compile_against_the_header():
    """With SPOA_USE_CEREAL, `archive(graph)` compiles as with the reference
    (the library's save/load hooks put its own bytes into the archive)."""
    src = os.path.join(os.path.dirname(__file__), "cpp", "cereal_compile_check.cpp")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run(["g++", "-std=c++11", "-fsyntax-only", "-DSPOA_USE_CEREAL",
                        "-I", os.path.join(root, "include"),
                        "-I", os.path.join(root, "oracle", "ref_shim"), src],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.skipif(sg.lib().spoa_gb300_device_count() > 0, reason="a GPU is visible")
def test_cpp_api_fails_loudly_without_a_gpu(tmp_path, sample_reads, spoa_test_cases):
    r = _run(tmp_path, sample_reads[:3], spoa_test_cases[:1])
    assert r.returncode != 0
    assert "CUDA error" in r.stdout


@pytest.mark.gpu
def test_cpp_api_known_answers(tmp_path, sample_reads, spoa_test_cases, spoa_test_outputs,
                               slice_windows):
    r = _run(tmp_path, sample_reads, spoa_test_cases, slice_windows)
    lines = r.stdout.splitlines()
    assert lines and lines[-1] == "DONE 0", "\n".join(ln for ln in lines if ln.startswith("FAIL"))
    assert r.returncode == 0
    by = {}
    for ln in lines:
        tag, _, rest = ln.partition(" ")
        name, _, val = rest.partition(" ")
        by.setdefault((tag, name), []).append(val)
    for case in spoa_test_cases:
        name, want = case["name"], spoa_test_outputs[case["name"]]
        assert by[("CONS", name)] == [case["consensus"]], name
        assert sha("\n".join(by[("MSA", name)])) == want["msa_sha"], name
        assert [int(x) for x in by[("SUMMARY", name)][0].split(",")] == want["summary"], name
        assert sha(by[("VSUMMARY", name)][0]) == want["summary_verbose_sha"], name
        assert by[("CLEAR", name)] == ["ok"], name
    # spoa_test.cpp:86-118 and graph.cpp:162-166
    assert by[("ERR", "TypeError")] == ["[spoa::AlignmentEngine::Create] error: invalid alignment type!"]
    assert by[("ERR", "EmptyInput")] == ["empty"]
    assert by[("ERR", "LargeInput1")] == ["AlignmentEngine::Prealloc] error: too large sequence!"]
    assert by[("ERR", "LargeInput2")] == ["no-throw"]
    # graph.cpp:518-605 through Graph::Subgraph / UpdateAlignment
    assert by[("ERR", "Persist")] == ["ok"]
    assert by[("ERR", "SubgraphNullMap")] == [
        "[spoa::Graph::Subgraph] error: invalid ptr to subgraph_to_graph"]
    for w, rec in enumerate(slice_windows):
        rows = [v for (tag, name), vals in by.items() if tag == "SLICE" and name == str(w)
                for v in vals]
        reads = [x for x in rows if x.startswith("R ")]
        assert [int(x.split(" ")[2]) for x in reads] == rec["expect"]["scores"]
        assert [sha(" ".join(x.split(" ")[3:])) for x in reads] == rec["expect"]["aln_sha"]
        assert [x[2:] for x in rows if x.startswith("C ")] == [rec["expect"]["consensus"]]
    assert by[("ERR", "UnequalWeights")] == [
        "[spoa::Graph::AddAlignment] error: sequence and weights are of unequal size!"]
