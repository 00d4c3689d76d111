"""Regenerates the golden fixtures in this directory.

Run here, where the reference tree and its compiled driver exist:
    python tests/golden/make_golden.py [--reference <reference tree>]

It writes
  sample_reads.tsv.gz      the 55 reads of test/data/sample.fastq.gz
                           (sequence <TAB> quality), decompressed verbatim;
  spoa_test_cases.json     the 18 known-answer consensus tests of
                           test/spoa_test.cpp (type, penalties, quality
                           flag, golden consensus), parsed from the file;
  spoa_test_outputs.json   what the compiled reference prints for those 18
                           runs (per-read scores, sha256 of alignments, MSA
                           and GFA, the consensus summary of
                           GenerateConsensus(summary) and the sha256 of its
                           verbose form);
  ref_windows.json.gz      seeded synthetic windows (inputs verbatim) with the
                           reference's outputs: scores, strand flags,
                           consensus, and sha256 of alignments, MSA and GFA;
  slice_windows.json.gz    backbone windows run through Graph::Subgraph and
                           UpdateAlignment (inputs and slice ranges verbatim)
                           with the reference's outputs: every subgraph's
                           driver lines (sha256 of each; the first three
                           subgraphs also verbatim), scores, alignments
                           (sha256), consensus and MSA (sha256).
  cli_outputs.json         what the reference CLI (its src/main.cpp, built
                           by oracle/Makefile) prints for the cases of
                           cli_inputs.py: exit code, stdout (sha256 and
                           size; verbatim when short), stderr, DOT file
                           (sha256); plus the names of the sample reads.
  persist_windows.json.gz  windows saved after some reads and loaded again
                           with the reference's own Graph::save/load (through
                           the archive stand-ins of oracle/ref_shim/cereal),
                           then given the remaining reads: the graph as
                           loaded (driver lines, sha256; verbatim for the
                           first windows), scores, alignments, consensus, MSA
                           and GFA after.
With --only slices, --only cli or --only persist only that file is
rewritten.
"""
from __future__ import annotations

import argparse
import gzip
import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import pyoracle as po  # noqa: E402
from spoa_gb300 import synth  # noqa: E402

TYPE_MAP = {"kSW": 0, "kNW": 1, "kOV": 2}


def sha(text: str) -> str:
    return hashlib.sha256(text.encode()).hexdigest()


def canon_alignment(arr) -> str:
    return " ".join(f"{int(a)},{int(b)}" for a, b in arr)


def canon_outputs(win: dict) -> dict:
    return {
        "scores": win["scores"],
        "reversed": win["reversed"],
        "consensus": win["consensus"],
        "aln_sha": [sha(canon_alignment(a)) for a in win["alignments"]],
        "msa_sha": sha("\n".join(win["msa"])),
        "gfa_sha": sha("\n".join(win["gfa"])),
        "n_pairs": [int(len(a)) for a in win["alignments"]],
    }


def parse_fastq_gz(path: str):
    reads = []
    with gzip.open(path, "rt") as fh:
        lines = [ln.rstrip("\n") for ln in fh]
    for k in range(0, len(lines) - 3, 4):
        reads.append((lines[k + 1], lines[k + 3]))
    return reads


def parse_test_cases(path: str):
    src = open(path).read()
    cases = []
    pat = re.compile(
        r"TEST_F\(SpoaTest,\s*(\w+)\)\s*\{\s*Setup\(AlignmentType::(\w+),\s*"
        r"(-?\d+),\s*(-?\d+),\s*(-?\d+),\s*(-?\d+),\s*(-?\d+),\s*(-?\d+),\s*(\w+)\);"
        r"\s*Align\(\);\s*std::string c\s*=\s*((?:\s*\"[ACGT]*\")+)\s*;\s*Check\(c\);")
    for mt in pat.finditer(src):
        name, typ = mt.group(1), mt.group(2)
        vals = [int(mt.group(k)) for k in range(3, 9)]
        quality = mt.group(9) == "true"
        cons = "".join(re.findall(r"\"([ACGT]*)\"", mt.group(10)))
        cases.append({"name": name, "type": TYPE_MAP[typ], "params": vals,
                      "quality": quality, "consensus": cons})
    return cases


def synthetic_specs():
    """(name, type, params, reads, quals, strand) of the golden windows."""
    rng = np.random.default_rng(20261203)
    params = [(5, -4, -8, -8, -8, -8), (5, -4, -8, -6, -8, -6), (5, -4, -8, -6, -10, -2),
              (5, -4, -8, -6, -10, -4), (2, -5, -2, -2, -2, -2), (3, -3, -5, -1, -9, 0),
              (1, -1, -1, -1, -1, -1)]
    specs = []
    for k in range(150):  # adversarial small windows, every L mod 16
        typ = int(rng.integers(0, 3))
        par = params[k % len(params)]
        ln = 1 + (k % 48) + int(rng.integers(0, 40))
        depth = int(rng.integers(1, 10))
        alpha = b"ACGTN" if k % 5 == 0 else b"ACGT"
        reads = synth.random_window(rng, ln, depth, err=float(rng.uniform(0.02, 0.4)),
                                    alphabet=alpha)
        quals = ([bytes(rng.integers(33, 75, size=len(r)).astype(np.uint8)) for r in reads]
                 if k % 3 == 0 else None)
        specs.append((f"adv{k}", typ, par, reads, quals, k % 4 == 1))
    A = np.frombuffer(b"ACGT", np.uint8)
    for k in range(48):  # long insertions: convex lane-boundary E behaviour
        base = A[rng.integers(0, 4, size=int(rng.integers(40, 120)))]
        ins = A[rng.integers(0, 4, size=int(rng.integers(10, 60)))]
        pos = int(rng.integers(5, base.size - 5))
        r2 = np.concatenate([base[:pos], ins, base[pos:]])
        reads = [base.tobytes(), r2.tobytes(), base.tobytes()[::-1], r2.tobytes()]
        par = (5, -4, -8, -6, -10, -2) if k % 2 == 0 else (2, -5, -6, -4, -20, -1)
        specs.append((f"ins{k}", k % 3, par, reads, None, False))
    w = synth.single_500(1)
    specs.append(("single_500", w.type, synth.SCORING["single_500"][1], w.reads, None, False))
    for k in range(3):
        w = synth.batch_window(k)
        specs.append((f"batch{k}", w.type, synth.SCORING["batch_10k"][1], w.reads, None, False))
    for k in range(4):
        w = synth.uneven_window(k)
        specs.append((f"uneven{k}", w.type, synth.SCORING["uneven_2k"][1], w.reads[:10], None,
                      True))
    w = synth.long_10k(7, n_reads=3, tpl_len=3200, min_len=2800)  # int32 width
    for typ in (0, 1, 2):
        specs.append((f"int32_{typ}", typ, (5, -4, -8, -6, -10, -4), w.reads, None, False))
    return specs


SLICE_PARAMS = [(5, -4, -8, -8, -8, -8), (5, -4, -8, -6, -8, -6), (5, -4, -8, -6, -10, -4)]


def write_slices():
    """12 backbone windows: every type x gap model, plus three more."""
    specs = []
    for k in range(12):
        reads, sl = synth.slice_window(k)
        specs.append((f"slice{k}", k % 3, SLICE_PARAMS[(k // 3) % 3], reads, sl))
    outs = po.parse_reference_output(po.run_reference(po.format_slices(
        [(t, p, r, sl) for _, t, p, r, sl in specs])))
    recs = []
    for (name, t, p, r, sl), o in zip(specs, outs):
        assert o["error"] is None, (name, o["error"])
        subs = o.get("slices", [])
        recs.append({"name": name, "type": t, "params": list(p),
                     "reads": [x.decode() for x in r], "slices": [list(x) for x in sl],
                     "expect": {"scores": o["scores"],
                                "aln_sha": [sha(canon_alignment(a)) for a in o["alignments"]],
                                "consensus": o["consensus"], "msa_sha": sha("\n".join(o["msa"])),
                                "subgraph_sha": [{k: sha(v) for k, v in x.items()} for x in subs],
                                "subgraph_first": subs[:3]}})
    with gzip.open(os.path.join(HERE, "slice_windows.json.gz"), "wt") as fh:
        json.dump(recs, fh)
    print(f"wrote {len(recs)} slice windows")


def write_persist():
    """Windows of every type and gap model, with and without qualities,
    saved after 0, 1, some or all of their reads."""
    specs = []
    rng = np.random.default_rng(4242)
    for k in range(12):
        w = synth.batch_window(100 + k)
        reads = w.reads[:12]
        quals = ([bytes(rng.integers(33, 75, size=len(r)).astype(np.uint8)) for r in reads]
                 if k % 2 else None)
        split = [0, 1, 5, len(reads)][k % 4]
        specs.append((f"persist{k}", k % 3, SLICE_PARAMS[(k // 3) % 3], reads, quals, split))
    outs = po.parse_reference_output(po.run_reference(po.format_persist(
        [(t, p, r, q, sp) for _, t, p, r, q, sp in specs])))
    recs = []
    for (name, t, p, r, q, sp), o in zip(specs, outs):
        assert o["error"] is None, (name, o["error"])
        recs.append({"name": name, "type": t, "params": list(p),
                     "reads": [x.decode() for x in r],
                     "quals": [x.decode() for x in q] if q is not None else None, "split": sp,
                     "expect": {"loaded_sha": {k: sha(v) for k, v in o["loaded"].items()},
                                "loaded": o["loaded"] if len(recs) < 2 else None,
                                "scores": o["scores"],
                                "aln_sha": [sha(canon_alignment(a)) for a in o["alignments"]],
                                "consensus": o["consensus"], "msa_sha": sha("\n".join(o["msa"])),
                                "gfa_sha": sha("\n".join(o["gfa"]))}})
    with gzip.open(os.path.join(HERE, "persist_windows.json.gz"), "wt") as fh:
        json.dump(recs, fh)
    print(f"wrote {len(recs)} persisted windows")


def write_cli(reference: str):
    """Runs the reference CLI on the inputs of cli_inputs.py."""
    import subprocess
    import tempfile
    import cli_inputs
    cli = os.path.join(ROOT, "oracle", "_ref", "spoa_ref_cli")
    with gzip.open(os.path.join(reference, "test/data/sample.fastq.gz"), "rt") as fh:
        lines = [ln.rstrip("\n") for ln in fh]
    names = [lines[k][1:].split()[0] for k in range(0, len(lines) - 3, 4)]
    with gzip.open(os.path.join(HERE, "sample_reads.tsv.gz"), "rt") as fh:
        sample = [tuple(x.encode() for x in ln.rstrip("\n").split("\t")) for ln in fh if ln.strip()]
    out = {"sample_names": names, "cases": [], "errors": []}
    with tempfile.TemporaryDirectory() as d:
        paths = cli_inputs.write_inputs(d, sample, names)
        dot = os.path.join(d, "graph.dot")
        for key, argv in cli_inputs.CASES + cli_inputs.ERROR_CASES:
            if os.path.exists(dot):
                os.remove(dot)
            cmd = [cli] + [dot if a == "{dot}" else a for a in argv] + [paths[key]]
            r = subprocess.run(cmd, capture_output=True, text=True)
            rec = {"input": key, "args": argv, "rc": r.returncode, "stdout_sha": sha(r.stdout),
                   "stdout_len": len(r.stdout), "stderr": r.stderr}
            if len(r.stdout) < 4096:
                rec["stdout"] = r.stdout
            if "{dot}" in argv:
                rec["dot_sha"] = sha(open(dot).read())
            out["errors" if (key, argv) in cli_inputs.ERROR_CASES else "cases"].append(rec)
            assert (r.returncode == 0) == ((key, argv) in cli_inputs.CASES), (argv, r.stderr)
    with open(os.path.join(HERE, "cli_outputs.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    print(f"wrote {len(out['cases'])} CLI cases and {len(out['errors'])} error cases")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=po.reference_tree())
    ap.add_argument("--only", choices=["slices", "cli", "persist"], default=None)
    args = ap.parse_args()
    os.environ["SPOA_REFERENCE_TREE"] = args.reference
    if po.build_reference() is None:
        raise SystemExit("reference driver could not be built")
    if args.only == "slices":
        write_slices()
        return
    if args.only == "cli":
        write_cli(args.reference)
        return
    if args.only == "persist":
        write_persist()
        return

    reads = parse_fastq_gz(os.path.join(args.reference, "test/data/sample.fastq.gz"))
    assert len(reads) == 55, len(reads)
    with gzip.open(os.path.join(HERE, "sample_reads.tsv.gz"), "wt") as fh:
        for s, q in reads:
            fh.write(f"{s}\t{q}\n")

    cases = parse_test_cases(os.path.join(args.reference, "test/spoa_test.cpp"))
    assert len(cases) == 18, len(cases)
    with open(os.path.join(HERE, "spoa_test_cases.json"), "w") as fh:
        json.dump(cases, fh, indent=1)

    specs = []
    for cs in cases:
        rd = [s.encode() for s, _ in reads]
        ql = [q.encode() for _, q in reads] if cs["quality"] else None
        specs.append((cs["type"], tuple(cs["params"]), rd, ql, False))
    outs = po.parse_reference_output(po.run_reference(po.format_windows(specs)))
    test_out = {}
    for cs, o in zip(cases, outs):
        assert o["error"] is None
        assert o["consensus"] == cs["consensus"], cs["name"]
        test_out[cs["name"]] = canon_outputs(o)
        # GenerateConsensus(summary, verbose) of the reference, both forms
        test_out[cs["name"]]["summary"] = o["summary"]
        test_out[cs["name"]]["summary_verbose_sha"] = sha(
            ",".join(str(x) for x in o["summary_verbose"]))
    with open(os.path.join(HERE, "spoa_test_outputs.json"), "w") as fh:
        json.dump(test_out, fh, indent=1)

    syn = synthetic_specs()
    outs = po.parse_reference_output(po.run_reference(po.format_windows(
        [(t, p, r, q, s) for _, t, p, r, q, s in syn])))
    recs = []
    for (name, t, p, r, q, s), o in zip(syn, outs):
        assert o["error"] is None, (name, o["error"])
        recs.append({"name": name, "type": t, "params": list(p),
                     "reads": [x.decode() for x in r],
                     "quals": [x.decode() for x in q] if q is not None else None,
                     "strand_ambiguous": s, "expect": canon_outputs(o)})
    with gzip.open(os.path.join(HERE, "ref_windows.json.gz"), "wt") as fh:
        json.dump(recs, fh)
    print(f"wrote {len(cases)} known-answer cases and {len(recs)} reference windows")
    write_slices()
    write_cli(args.reference)
    write_persist()


if __name__ == "__main__":
    main()
