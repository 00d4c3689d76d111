"""Input files of the command-line parity cases (tests/test_cli.py), written
the same way by the fixture script and by the tests: the reference's
sample reads as FASTQ (plain and gzip) and two seeded synthetic windows, a
FASTA with wrapped lines and described headers (gzip) and a FASTQ."""
from __future__ import annotations

import gzip
import os

import numpy as np

from spoa_gb300 import synth


def _fasta(reads, names, width=60):
    out = []
    for name, r in zip(names, reads):
        out.append(f">{name} len={len(r)} synthetic\n")
        s = r.decode()
        out.extend(s[k:k + width] + "\n" for k in range(0, len(s), width))
    return "".join(out)


def _fastq(reads, quals, names):
    return "".join(f"@{n} window=7\n{r.decode()}\n+\n{q.decode()}\n"
                   for n, r, q in zip(names, reads, quals))


def write_inputs(directory: str, sample_reads, sample_names) -> dict:
    """Writes the inputs into `directory`; returns {key: path}."""
    os.makedirs(directory, exist_ok=True)
    paths = {}
    text = "".join(f"@{n}\n{s.decode()}\n+\n{q.decode()}\n"
                   for n, (s, q) in zip(sample_names, sample_reads))
    paths["sample_fastq"] = os.path.join(directory, "sample.fastq")
    with open(paths["sample_fastq"], "w") as fh:
        fh.write(text)
    paths["sample_fastq_gz"] = os.path.join(directory, "sample.fastq.gz")
    with gzip.open(paths["sample_fastq_gz"], "wt") as fh:
        fh.write(text)
    w = synth.batch_window(17)
    names = [f"read{k}" for k in range(len(w.reads))]
    paths["synth_fasta_gz"] = os.path.join(directory, "synth.fasta.gz")
    with gzip.open(paths["synth_fasta_gz"], "wt") as fh:
        fh.write(_fasta(w.reads, names))
    u = synth.uneven_window(3)
    reads = [r[:900] for r in u.reads[:20]]
    rng = np.random.Generator(np.random.PCG64(77))
    quals = [bytes(rng.integers(35, 74, size=len(r)).astype(np.uint8)) for r in reads]
    paths["synth_fq"] = os.path.join(directory, "synth.fq")
    with open(paths["synth_fq"], "w") as fh:
        fh.write(_fastq(reads, quals, [f"u{k}" for k in range(len(reads))]))
    return paths


# (input key, arguments); "{dot}" is replaced by a DOT output path
CASES = [
    ("sample_fastq_gz", []),
    ("sample_fastq", ["-l", "1"]),
    ("sample_fastq", ["-l", "2", "-r", "0", "-r", "1"]),
    ("sample_fastq_gz", ["-l", "1", "-r", "2"]),
    ("sample_fastq", ["-l", "2", "-r", "3"]),
    ("sample_fastq", ["-r", "4", "-d", "{dot}"]),
    ("sample_fastq", ["-l", "1", "-m", "2", "-n", "-5", "-g", "-2", "-e", "-2", "-r", "2"]),
    ("sample_fastq_gz", ["-l", "2", "-g", "-8", "-e", "-6", "-q", "-8", "-c", "-6", "-s",
                         "-r", "4"]),
    ("synth_fasta_gz", ["-l", "2", "-r", "2", "-d", "{dot}"]),
    ("synth_fasta_gz", ["-s", "-r", "3"]),
    ("synth_fq", ["-l", "1", "-s", "-r", "4"]),
    ("synth_fq", ["--algorithm", "2", "--result", "1", "--strand-ambiguous"]),
]

# argument errors the reference reports before any alignment
ERROR_CASES = [
    ("sample_fastq", ["-l", "5"]),
    ("sample_fastq", ["-g", "3"]),
    ("sample_fastq", ["-c", "2", "-q", "-3"]),
]
