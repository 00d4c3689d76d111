"""The `spoa` command-line program (spoa_gb300/spoa) against what the
reference CLI (its own src/main.cpp, compiled by oracle/Makefile) printed
for the same files and options (tests/golden/cli_outputs.json): exit code,
stdout byte for byte, and the DOT file."""
import json
import os
import subprocess
import sys

import pytest

from conftest import GOLDEN, sha
from spoa_gb300 import build as sgb

sys.path.insert(0, GOLDEN)
import cli_inputs  # noqa: E402

CLI = sgb.CLI


@pytest.fixture(scope="module")
def cli_outputs():
    with open(os.path.join(GOLDEN, "cli_outputs.json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="module")
def inputs(tmp_path_factory, sample_reads, cli_outputs):
    d = tmp_path_factory.mktemp("cli")
    return cli_inputs.write_inputs(str(d), sample_reads, cli_outputs["sample_names"]), str(d)


def _run(argv, paths, d):
    if not os.path.exists(CLI):
        pytest.skip("spoa CLI not built (python -m spoa_gb300.build)")
    dot = os.path.join(d, "graph.dot")
    if os.path.exists(dot):
        os.remove(dot)
    key, args = argv
    cmd = [CLI] + [dot if a == "{dot}" else a for a in args] + [paths[key]]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
    return r, dot


def test_argument_errors_match_the_reference(inputs, cli_outputs):
    """Checks made before any alignment: the reference's messages and exit
    codes (alignment_engine.cpp:40-55, main.cpp:25-59, 225-229)."""
    paths, d = inputs
    for rec in cli_outputs["errors"]:
        r, _ = _run((rec["input"], rec["args"]), paths, d)
        assert r.returncode == rec["rc"]
        assert r.stderr == rec["stderr"]
        assert r.stdout == ""
    r, _ = _run(("x", []), {"x": os.path.join(d, "reads.txt")}, d)
    assert r.returncode == 1 and "has unsupported format extension" in r.stderr
    r, _ = _run(("x", []), {"x": os.path.join(d, "missing.fastq")}, d)
    assert r.returncode == 1 and "unable to open file" in r.stderr
    r = subprocess.run([CLI], capture_output=True, text=True)
    assert r.returncode == 1 and r.stderr == "[spoa::] error: missing input file!\n"
    r = subprocess.run([CLI, "--version"], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout == "4.0.8\n"


@pytest.mark.gpu
def test_outputs_match_the_reference(inputs, cli_outputs):
    """Consensus, MSA (with and without the consensus row) and GFA (with and
    without the consensus path) on FASTQ, gzip FASTQ, wrapped gzip FASTA,
    every alignment type, linear/affine/convex gaps, strand-ambiguous runs
    with qualities, and the DOT file."""
    paths, d = inputs
    for rec in cli_outputs["cases"]:
        r, dot = _run((rec["input"], rec["args"]), paths, d)
        assert r.returncode == rec["rc"], (rec["args"], r.stderr)
        if "stdout" in rec:
            assert r.stdout == rec["stdout"], rec["args"]
        assert len(r.stdout) == rec["stdout_len"], rec["args"]
        assert sha(r.stdout) == rec["stdout_sha"], rec["args"]
        if "dot_sha" in rec:
            assert sha(open(dot).read()) == rec["dot_sha"], rec["args"]
