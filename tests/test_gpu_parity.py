"""GPU path against the reference's golden vectors, recorded reference outputs
and the oracle (bit-exact: scores, alignments, consensus, MSA, GFA)."""
import numpy as np
import pytest

from conftest import check_against_expect

pytestmark = pytest.mark.gpu

sg = pytest.importorskip("spoa_gb300")
from oracle import pyoracle as po  # noqa: E402
from spoa_gb300 import synth  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if sg.lib().spoa_gb300_device_count() <= 0:
        pytest.fail("no CUDA device visible to the GPU library")


def run_per_call(type_, params, reads, quals=None):
    """spoa's CLI loop through the drop-in per-call API (Align, AddAlignment)."""
    engine = sg.AlignmentEngine.create(type_, *params)
    graph = sg.Graph()
    engine.prealloc(max(len(r) for r in reads), 4)
    scores, alns = [], []
    for k, r in enumerate(reads):
        aln, score = engine.align(r, graph)
        scores.append(0 if score is None else score)
        alns.append(aln)
        graph.add_alignment(aln, r, quals[k] if quals is not None else 1)
    cons = graph.generate_consensus()
    msa = graph.generate_multiple_sequence_alignment()
    return scores, alns, cons, msa, graph


def test_known_answers_per_call(sample_reads, spoa_test_cases, spoa_test_outputs):
    """test/spoa_test.cpp:154-440 through Align/AddAlignment, plus the
    reference's own per-read alignments, MSA and GFA of the same runs."""
    reads = [s for s, _ in sample_reads]
    quals = [q for _, q in sample_reads]
    for case in spoa_test_cases:
        scores, alns, cons, msa, graph = run_per_call(
            case["type"], case["params"], reads, quals if case["quality"] else None)
        assert cons == case["consensus"], case["name"]
        gfa = graph.gfa()
        check_against_expect(spoa_test_outputs[case["name"]], scores, [0] * len(reads), alns,
                             cons, msa, gfa)


def test_known_answers_fused(sample_reads, spoa_test_cases):
    """Align + AddAlignment fused on the device (no host round trip)."""
    reads = [s for s, _ in sample_reads]
    quals = [q for _, q in sample_reads]
    for case in spoa_test_cases[::3]:
        engine = sg.AlignmentEngine.create(case["type"], *case["params"])
        graph = sg.Graph()
        for k, r in enumerate(reads):
            sg.align_add(engine, graph, r, quals[k] if case["quality"] else None)
        assert graph.generate_consensus() == case["consensus"], case["name"]


def _group_ref_windows(ref_windows):
    groups = {}
    for rec in ref_windows:
        key = (tuple(rec["params"]), rec["quals"] is not None)
        groups.setdefault(key, []).append(rec)
    return groups


def test_reference_windows_batched(ref_windows):
    """209 recorded reference windows through the persistent kernel, with
    per-read alignments and MSA returned."""
    for (params, has_q), recs in _group_ref_windows(ref_windows).items():
        windows = [[r.encode() for r in rec["reads"]] for rec in recs]
        quals = [[q.encode() for q in rec["quals"]] for rec in recs] if has_q else None
        res = sg.batch_poa(windows, recs[0]["type"], *params,
                           window_types=[rec["type"] for rec in recs],
                           window_strand=[1 if rec["strand_ambiguous"] else 0 for rec in recs],
                           quals=quals, want_alignments=True, want_msa=True)
        assert (res.status == 0).all(), res.status
        r0 = 0
        for w, rec in enumerate(recs):
            nr = len(rec["reads"])
            check_against_expect(rec["expect"], res.scores[r0:r0 + nr].tolist(),
                                 res.reversed[r0:r0 + nr].tolist(), res.alignments[r0:r0 + nr],
                                 res.consensus[w], res.msa[w], None)
            r0 += nr


def test_reference_windows_fused_with_gfa(ref_windows):
    """The same windows read by read through the fused per-read call, GFA
    included."""
    for rec in ref_windows[::7]:
        engine = sg.AlignmentEngine.create(rec["type"], *rec["params"])
        graph = sg.Graph()
        scores, rev = [], []
        for k, r in enumerate(rec["reads"]):
            q = rec["quals"][k] if rec["quals"] else None
            s, rv = sg.align_add(engine, graph, r, q, rec["strand_ambiguous"])
            scores.append(s)
            rev.append(int(rv))
        assert scores == rec["expect"]["scores"], rec["name"]
        assert rev == rec["expect"]["reversed"], rec["name"]
        cons = graph.generate_consensus()
        assert cons == rec["expect"]["consensus"], rec["name"]
        from conftest import sha
        assert sha("\n".join(graph.generate_multiple_sequence_alignment())) == \
            rec["expect"]["msa_sha"]
        assert sha("\n".join(graph.gfa(rev))) == rec["expect"]["gfa_sha"], rec["name"]


def test_polishing_windows_vs_oracle():
    """Polishing-shaped windows (450-550 nt, depth 10-60, OV convex)."""
    wins = synth.batch_windows(24)
    params = synth.SCORING["batch_10k"][1]
    res = sg.batch_poa([w.reads for w in wins], 2, *params, want_alignments=True)
    assert (res.status == 0).all()
    r0 = 0
    for k, w in enumerate(wins):
        ref = po.run_window(2, *params, w.reads, with_msa=False)
        n = len(w.reads)
        assert res.scores[r0:r0 + n].tolist() == ref.scores, k
        for a, b in zip(res.alignments[r0:r0 + n], ref.alignments):
            assert np.array_equal(a, b), k
        assert res.consensus[k] == ref.consensus, k
        r0 += n


def test_uneven_windows_vs_oracle():
    """Uneven windows: per-window NW/OV, strand-ambiguous, mixed widths."""
    wins = [synth.uneven_window(k) for k in range(12)]
    wins = [synth.Window(reads=w.reads[:20], type=w.type, strand_ambiguous=True) for w in wins]
    params = synth.SCORING["uneven_2k"][1]
    res = sg.batch_poa([w.reads for w in wins], 1, *params, window_types=[w.type for w in wins],
                       window_strand=[1] * len(wins))
    assert (res.status == 0).all()
    r0 = 0
    for k, w in enumerate(wins):
        ref = po.run_window(w.type, *params, w.reads, strand_ambiguous=True, with_msa=False)
        n = len(w.reads)
        assert res.scores[r0:r0 + n].tolist() == ref.scores, k
        assert res.reversed[r0:r0 + n].tolist() == ref.reversed, k
        assert res.consensus[k] == ref.consensus, k
        r0 += n


def test_plain_and_batched_forms_agree():
    wins = synth.batch_windows(10, start=100)
    params = synth.SCORING["batch_10k"][1]
    b = sg.Batch([w.reads for w in wins], 2, *params)
    b.launch()
    r1 = b.fetch()
    b.launch_plain()
    r2 = b.fetch()
    assert r2.launches == len(wins)
    assert r1.consensus == r2.consensus
    assert np.array_equal(r1.scores, r2.scores)


def test_errors_match_reference_messages():
    with pytest.raises(sg.SpoaError, match="invalid alignment type"):
        sg.AlignmentEngine.create(4, 1, -1, -1)
    with pytest.raises(sg.SpoaError, match="gap opening penalty must be non-positive"):
        sg.AlignmentEngine.create(0, 1, -1, 1)
    engine = sg.AlignmentEngine.create(0, 1, -1, -1)
    graph = sg.Graph()
    aln, score = engine.align(b"", graph)  # EmptyInput (spoa_test.cpp:96-101)
    assert aln.shape == (0, 2) and score is None
    graph.add_alignment(aln, b"ACGT")
    with pytest.raises(sg.SpoaError, match="invalid alignment"):
        graph.add_alignment(np.array([[0, 9]], np.int32), b"ACGT")
    with pytest.raises(sg.SpoaError, match="unequal size"):
        graph.add_alignment(aln, b"ACGT", [1, 2])


def test_clear_reproduces_consensus(sample_reads):
    """spoa_test.cpp:121-129."""
    reads = [s for s, _ in sample_reads]
    engine = sg.AlignmentEngine.create(0, 5, -4, -8, -8, -8, -8)
    graph = sg.Graph()
    for r in reads:
        sg.align_add(engine, graph, r)
    c1 = graph.generate_consensus()
    graph.clear()
    for r in reads:
        sg.align_add(engine, graph, r)
    assert graph.generate_consensus() == c1


def test_autotuned_tiles_give_the_same_results():
    """The tile tuner (timed candidates per length class) changes only speed."""
    wins = synth.batch_windows(300, start=500) + [synth.uneven_window(k) for k in range(6)]
    reads = [w.reads for w in wins]
    params = synth.SCORING["batch_10k"][1]
    kw = dict(window_types=[2] * 300 + [w.type for w in wins[300:]],
              window_strand=[0] * 300 + [1] * 6)
    a = sg.batch_poa(reads, 2, *params, **kw)
    b = sg.batch_poa(reads, 2, *params, autotune=True, **kw)
    assert (a.status == 0).all() and (b.status == 0).all()
    assert a.consensus == b.consensus
    assert np.array_equal(a.scores, b.scores)


def test_per_read_loop_recorded_in_a_cuda_graph(ref_windows):
    """align_add_reads (one launch per read, recorded into a CUDA graph)
    gives the reference's per-read scores, strands and consensus."""
    for rec in ref_windows[:40]:
        engine = sg.AlignmentEngine.create(rec["type"], *rec["params"])
        graph = sg.Graph()
        reads = [r.encode() for r in rec["reads"]]
        quals = [q.encode() for q in rec["quals"]] if rec["quals"] else None
        scores, rev = sg.align_add_reads(engine, graph, reads, quals,
                                         strand_ambiguous=rec["strand_ambiguous"])
        assert scores == rec["expect"]["scores"], rec["name"]
        assert [int(x) for x in rev] == rec["expect"]["reversed"], rec["name"]
        assert graph.generate_consensus() == rec["expect"]["consensus"], rec["name"]


def test_windows_that_outgrow_their_arena_and_the_int16_width():
    """20-letter noisy windows grow to ~10k nodes: more than the first arena
    (4,096 nodes, 4 aligned nodes per node) and past the int16 rule, which
    the width estimate did not foresee; they rerun with twice the capacity
    and the int32 kernel, in the batch and in the server."""
    rng = np.random.Generator(np.random.PCG64(79))
    wins = [synth.random_window(rng, 300, 40, err=0.6, alphabet=b"ACDEFGHIKLMNPQRSTVWY")
            for _ in range(3)] + [w.reads for w in synth.batch_windows(3, start=900)]
    params = synth.SCORING["batch_10k"][1]
    res = sg.batch_poa(wins, 2, *params)
    assert (res.status == 0).all()
    assert res.launches > 1  # the reruns
    r0 = 0
    for k, w in enumerate(wins):
        ref = po.run_window(2, *params, w, with_msa=False)
        assert res.scores[r0:r0 + len(w)].tolist() == ref.scores, k
        assert res.consensus[k] == ref.consensus, k
        r0 += len(w)
    with sg.Server(2, *params) as sv:
        tickets = [sv.submit(w) for w in wins]
        got = [sv.wait(t, timeout=600) for t in tickets]
    assert [g[0] for g in got] == [0] * len(wins)
    assert [g[1] for g in got] == res.consensus


def run_slices_gpu(type_, params, reads, slices):
    """The slice protocol (read 0 whole; each later read aligned to
    Graph::Subgraph(begin, end) and mapped back by UpdateAlignment) through
    the device graph and the per-call engine."""
    engine = sg.AlignmentEngine.create(type_, *params)
    graph = sg.Graph()
    graph.add_alignment(np.zeros((0, 2), np.int32), reads[0])
    scores, alns, subs = [], [], []
    for r, (b, e) in enumerate(slices, start=1):
        if b >= 0:
            sub, m = graph.subgraph(b, e)
            assert (m[sub.num_nodes:] == sg.NO_NODE).all()
            ex = sub.export()
            cons = sub.generate_consensus()
            subs.append(po.slice_lines(r, m, ex["chars"], ex["rank_to_node"], ex["edge_tail"],
                                       ex["edge_head"], ex["edge_weight"], ex["aligned_off"],
                                       ex["aligned"], cons))
            aln, score = engine.align(reads[r], sub)
            aln = graph.update_alignment(m, aln)
        else:
            aln, score = engine.align(reads[r], graph)
        scores.append(0 if score is None else score)
        alns.append(aln)
        graph.add_alignment(aln, reads[r])
    return scores, alns, subs, graph.generate_consensus(), \
        graph.generate_multiple_sequence_alignment()


def test_subgraph_update_alignment(slice_windows):
    """Graph::Subgraph + UpdateAlignment (graph.cpp:518-605) on the device
    against recorded reference runs: every subgraph's nodes, order, edges,
    aligned lists and consensus, each score and mapped alignment, the final
    consensus and MSA; includes whole-graph, empty and single-node slices."""
    from conftest import check_slices
    for rec in slice_windows:
        got = run_slices_gpu(rec["type"], tuple(rec["params"]),
                             [r.encode() for r in rec["reads"]], rec["slices"])
        check_slices(rec["expect"], *got)


def test_subgraph_rejects_bad_node_ids():
    graph = sg.Graph()
    graph.add_alignment(np.zeros((0, 2), np.int32), b"ACGTACGT")
    for b, e in ((8, 2), (0, 8)):
        with pytest.raises(sg.SpoaError) as ex:
            graph.subgraph(b, e)
        assert ex.value.status == 1
    sub, m = graph.subgraph(7, 0)  # inverted range: an empty subgraph
    assert sub.num_nodes == 0 and (m == sg.NO_NODE).all()


def _loaded_lines(graph):
    ex = graph.export()
    return po.loaded_lines(ex["chars"], ex["rank_to_node"], ex["seq_begin"], ex["consensus"],
                           ex["edge_tail"], ex["edge_head"], ex["edge_weight"], ex["label_off"],
                           ex["labels"], ex["aligned_off"], ex["aligned"])


def test_save_load_matches_the_reference(persist_windows):
    """Graph persistence: a window saved after 0, 1, some or all reads and
    loaded again holds what the reference's own Graph::load rebuilds
    (nodes, edges with labels and weights, aligned lists in the order load
    gives them, rank order, sequence starts, consensus), and the remaining
    reads then give the reference's scores, alignments, consensus, MSA and
    GFA."""
    from conftest import canon_alignment, sha
    for rec in persist_windows:
        reads = [r.encode() for r in rec["reads"]]
        quals = [q.encode() for q in rec["quals"]] if rec["quals"] else None
        engine = sg.AlignmentEngine.create(rec["type"], *rec["params"])
        first = sg.Graph()
        for k in range(rec["split"]):
            aln, _ = engine.align(reads[k], first)
            first.add_alignment(aln, reads[k], quals[k] if quals else 1)
        if rec["split"]:
            first.generate_consensus()
        blob = first.save()
        graph = sg.Graph().load(blob)
        got = _loaded_lines(graph)
        exp = rec["expect"]
        if exp["loaded"]:
            assert got == exp["loaded"], rec["name"]
        assert {k: sha(v) for k, v in got.items()} == exp["loaded_sha"], rec["name"]
        assert graph.save() == blob  # a loaded graph saves to the same bytes
        scores, alns = [], []
        for k in range(rec["split"], len(reads)):
            aln, score = engine.align(reads[k], graph)
            scores.append(0 if score is None else score)
            alns.append(aln)
            graph.add_alignment(aln, reads[k], quals[k] if quals else 1)
        assert scores == exp["scores"], rec["name"]
        assert [sha(canon_alignment(a)) for a in alns] == exp["aln_sha"], rec["name"]
        assert graph.generate_consensus() == exp["consensus"], rec["name"]
        assert sha("\n".join(graph.generate_multiple_sequence_alignment())) == exp["msa_sha"]
        assert sha("\n".join(graph.gfa())) == exp["gfa_sha"], rec["name"]


def test_load_rejects_malformed_bytes():
    graph = sg.Graph()
    graph.add_alignment(np.zeros((0, 2), np.int32), b"ACGTACGT")
    graph.generate_consensus()
    blob = graph.save()
    for bad in (b"", b"XXXXXXXX" + blob[8:], blob[:-1], blob + b"\0"):
        with pytest.raises(sg.SpoaError) as ex:
            sg.Graph().load(bad)
        assert ex.value.status == 1
    assert sg.Graph().load(blob).generate_consensus() == "ACGTACGT"


def test_library_gfa_text(ref_windows):
    """spoa_gb300_graph_gfa (GFA written by the library into a caller buffer)
    equals the GFA pinned by the recorded reference runs."""
    from conftest import sha
    for rec in ref_windows[::21]:
        engine = sg.AlignmentEngine.create(rec["type"], *rec["params"])
        graph = sg.Graph()
        rev = []
        for k, r in enumerate(rec["reads"]):
            q = rec["quals"][k] if rec["quals"] else None
            _, rv = sg.align_add(engine, graph, r, q, rec["strand_ambiguous"])
            rev.append(int(rv))
        graph.generate_consensus()
        text = graph.gfa_text(rev if rec["strand_ambiguous"] else None)
        assert sha(text[:-1]) == rec["expect"]["gfa_sha"], rec["name"]
        assert text == "\n".join(graph.gfa(rev if rec["strand_ambiguous"] else None)) + "\n"
