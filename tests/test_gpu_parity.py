"""GPU parity: the CUDA path, called through the C ABI, against WFA2-lib's goldens, the real
WFA2-lib's recorded outputs, and the oracle — bit-exact scores and CIGARs."""
import numpy as np
import pytest

import biwfa_gpu_pii2025_gb300 as pkg
from biwfa_gpu_pii2025_gb300 import _capi
from golden_data import printed_line, ref_cases, utest
from oracle import binding

pytestmark = pytest.mark.gpu


def gpu_printed_line(res, i, score_only):
    """The GPU result in align_benchmark's `score\\tCIGAR` form."""
    if score_only:
        return printed_line(int(res.scores[i]), "")
    cig = res.cigar(i)
    return printed_line(int(res.scores[i]) if cig else -1, cig)


@pytest.mark.parametrize("name", sorted(utest()["sets"].keys()))
def test_gpu_matches_wfa2_utest_goldens(batch_aligner, name):
    data = utest()
    s = data["sets"][name]
    b = pkg.PairBatch.from_lists([p for p, _ in data["pairs"]], [t for _, t in data["pairs"]])
    res = batch_aligner.align(b, penalties=tuple(s["penalties"]), score_only=s["score_only"],
                              metric=s.get("metric", 0))
    assert (res.status == 0).all()
    bad = [i for i in range(b.n) if gpu_printed_line(res, i, s["score_only"]) != s["lines"][i]]
    assert not bad, f"{name}: {len(bad)} pairs differ, first {bad[:5]}"


@pytest.mark.parametrize("case", ref_cases(), ids=lambda c: c["tag"])
def test_gpu_matches_wfa2_reference_outputs(batch_aligner, case):
    pairs = case["pairs"]
    b = pkg.PairBatch.from_lists([r[0] for r in pairs], [r[1] for r in pairs])
    res = batch_aligner.align(b, penalties=tuple(case["penalties"]), score_only=case["score_only"],
                              metric=case.get("metric", 0))
    for i, (_, _, st, score, cig) in enumerate(pairs):
        assert res.status[i] == st, i
        assert gpu_printed_line(res, i, case["score_only"]) == printed_line(score, "" if case["score_only"] else
                                                                           (cig if cig != "-" else "")), i


@pytest.mark.parametrize("workload,n,seed", [(1, 300, 11), (2, 2000, 12), (3, 60, 13), (5, 400, 15)])
def test_gpu_matches_oracle_on_generated(batch_aligner, workload, n, seed):
    b = pkg.PairBatch.generate(workload, n, seed)
    res = batch_aligner.align(b)
    _, scores, status, ops = binding.oracle_batch_time(b.seq, b.p_off, b.plen, b.t_off, b.tlen, threads=8,
                                                       return_ops=True)
    assert (status == 0).all() and (res.status == 0).all()
    bad = [i for i in range(b.n) if pkg.runs_to_ops(res.runs_of(i)) != ops[i] or
           res.scores[i] != (scores[i] if ops[i] else 0)]
    assert not bad, f"{len(bad)} pairs differ, first {bad[:5]}"


OTHER_METRICS = [(_capi.METRIC_EDIT, (0, 0, 0, 0)), (_capi.METRIC_INDEL, (0, 0, 0, 0)),
                 (_capi.METRIC_GAP_LINEAR, (0, 4, 2, 0)), (_capi.METRIC_GAP_LINEAR, (-3, 2, 3, 0)),
                 (_capi.METRIC_GAP_AFFINE_2P, (0, 4, 6, 2, 24, 1)), (_capi.METRIC_GAP_AFFINE_2P, (-2, 3, 1, 2, 8, 1)),
                 (_capi.METRIC_GAP_AFFINE_2P, (0, 4, 12, 1, 3, 4)), (_capi.METRIC_GAP_AFFINE_2P, (-1, 4, 6, 2, 24, 1))]
OTHER_IDS = ["edit", "indel", "gap_linear_0_4_2", "gap_linear_m3_2_3", "affine2p_0_4_6_2_24_1",
             "affine2p_m2_3_1_2_8_1", "affine2p_0_4_12_1_3_4", "affine2p_m1_4_6_2_24_1_scope52"]


@pytest.mark.parametrize("metric,pen", OTHER_METRICS, ids=OTHER_IDS)
@pytest.mark.parametrize("workload,n,seed", [(1, 200, 31), (3, 120, 33), (5, 2000, 35)])
def test_gpu_other_distances_match_oracle(batch_aligner, metric, pen, workload, n, seed):
    """Edit, indel, gap-linear and two-piece gap-affine BiWFA (WFA2-lib's edit-wfa / indel-wfa /
    gap-linear-wfa / gap-affine2p-wfa with ultralow memory) against the oracle, full CIGARs and
    score-only."""
    b = pkg.PairBatch.generate(workload, n, seed)
    res = batch_aligner.align(b, penalties=pen, metric=metric)
    res_so = batch_aligner.align(b, penalties=pen, metric=metric, score_only=True)
    _, scores, status, ops = binding.oracle_batch_time(b.seq, b.p_off, b.plen, b.t_off, b.tlen, pen, threads=8,
                                                       return_ops=True, metric=metric)
    _, scores_so, _ = binding.oracle_batch_time(b.seq, b.p_off, b.plen, b.t_off, b.tlen, pen, threads=8,
                                                score_only=True, metric=metric)
    assert (status == 0).all() and (res.status == 0).all() and (res_so.status == 0).all()
    bad = [i for i in range(b.n) if pkg.runs_to_ops(res.runs_of(i)) != ops[i] or
           res.scores[i] != (scores[i] if ops[i] else 0) or res_so.scores[i] != scores_so[i]]
    assert not bad, f"{len(bad)} pairs differ, first {bad[:5]}"


@pytest.mark.parametrize("metric,pen", [OTHER_METRICS[i] for i in (0, 1, 2, 4)],
                         ids=[OTHER_IDS[i] for i in (0, 1, 2, 4)])
def test_gpu_other_distances_through_retry_passes_and_shapes(batch_aligner, metric, pen):
    """Long pairs of very different lengths (edit's exact pruning), the retry passes of every
    shape and the multi-warp shapes give the single-warp results."""
    rng = np.random.default_rng(5)
    pats, txts = [], []
    for a, c in ((6000, 1500), (1200, 7000), (3000, 3000), (4000, 100)):
        pats.append(bytes(rng.choice(list(b"ACGT"), a).astype(np.uint8)))
        txts.append(bytes(rng.choice(list(b"ACGT"), c).astype(np.uint8)))
    long_b = pkg.PairBatch.from_lists(pats, txts)
    mix = pkg.PairBatch.generate(5, 200, seed=36)
    for b in (long_b, mix):
        ref = batch_aligner.align(b, penalties=pen, metric=metric)
        for i in range(b.n):
            st, score, ops, _ = binding.oracle_align(b.pattern(i), b.text(i), pen, metric=metric)
            assert ref.status[i] == 0 and pkg.runs_to_ops(ref.runs_of(i)) == ops, i
        outs = []
        try:
            batch_aligner.set_arena_limits(ring_w=16, leaf_words=64)
            for rw in (8, 4, 1):
                batch_aligner.set_retry_shape(rw)
                outs.append(batch_aligner.align(b, penalties=pen, metric=metric))
            batch_aligner.set_arena_limits(0, 0)
            for gw, smem in ((4, False), (8, False), (8, True)):
                batch_aligner.set_exec_shape(gw, smem)
                outs.append(batch_aligner.align(b, penalties=pen, metric=metric, sched=_capi.SCHED_PLAIN))
        finally:
            batch_aligner.set_arena_limits(0, 0)
            batch_aligner.set_retry_shape(8)
            batch_aligner.set_exec_shape(1, False)
        for r in outs:
            assert np.array_equal(r.status, ref.status) and np.array_equal(r.scores, ref.scores)
            for i in range(b.n):
                assert np.array_equal(r.runs_of(i), ref.runs_of(i))


def test_gpu_long_noisy_pair_matches_oracle(batch_aligner):
    """Two 50-100 kbp pairs at 12 % error beside short pairs: the sorted schedule sends the long
    ones straight to the multi-warp launch with full-width rings (no retry pass), concurrently
    with the single-warp launch of the rest."""
    long_b = pkg.PairBatch.generate(4, 2, seed=404)
    short = pkg.PairBatch.generate(2, 300, seed=405)
    b = pkg.PairBatch.from_lists([long_b.pattern(i) for i in range(2)] + [short.pattern(i) for i in range(300)],
                                 [long_b.text(i) for i in range(2)] + [short.text(i) for i in range(300)])
    res = batch_aligner.align(b)
    assert batch_aligner.stats().retried_pairs == 0
    _, scores, status, ops = binding.oracle_batch_time(short.seq, short.p_off, short.plen, short.t_off, short.tlen,
                                                       threads=8, return_ops=True)
    for j in range(300):
        assert res.status[2 + j] == 0 and res.scores[2 + j] == scores[j]
        assert pkg.runs_to_ops(res.runs_of(2 + j)) == ops[j]
    for i in range(2):
        st, score, ops, _ = binding.oracle_align(b.pattern(i), b.text(i))
        assert res.status[i] == 0
        assert res.scores[i] == score
        assert pkg.runs_to_ops(res.runs_of(i)) == ops


def test_gpu_score_only_matches_oracle(batch_aligner):
    b = pkg.PairBatch.generate(5, 300, seed=21)
    res = batch_aligner.align(b, score_only=True)
    assert (res.status == 0).all()
    assert (res.run_len == 0).all()
    for i in range(b.n):
        assert res.scores[i] == binding.oracle_align(b.pattern(i), b.text(i), score_only=True)[1]


@pytest.mark.parametrize("retry_warps", [8, 4, 1])
def test_overflow_retry_passes_keep_results_exact(batch_aligner, retry_warps):
    """Tiny first-pass arenas push most pairs into the retry passes (of each shape); results
    must not move."""
    b = pkg.PairBatch.generate(5, 200, seed=31)
    ref = batch_aligner.align(b)
    try:
        batch_aligner.set_arena_limits(ring_w=16, leaf_words=64)
        batch_aligner.set_retry_shape(retry_warps)
        res = batch_aligner.align(b)
        st = batch_aligner.stats()
    finally:
        batch_aligner.set_arena_limits(0, 0)
        batch_aligner.set_retry_shape(8)
    assert st.retried_pairs > 0
    assert (res.status == 0).all()
    assert np.array_equal(res.scores, ref.scores)
    for i in range(b.n):
        assert np.array_equal(res.runs_of(i), ref.runs_of(i))


def test_given_order_and_predictions_do_not_change_results(batch_aligner):
    b = pkg.PairBatch.generate(5, 300, seed=41)
    ref = batch_aligner.align(b)
    batch_aligner.upload(b)
    batch_aligner.set_order(np.random.default_rng(0).permutation(b.n))
    batch_aligner.run(sched=_capi.SCHED_GIVEN)
    r2 = batch_aligner.fetch()
    batch_aligner.upload(b)
    batch_aligner.set_predictions(np.random.default_rng(1).uniform(0, 3000, b.n))
    batch_aligner.run(sched=_capi.SCHED_LEARNED)
    r3 = batch_aligner.fetch()
    for r in (r2, r3):
        assert np.array_equal(r.scores, ref.scores) and np.array_equal(r.status, ref.status)
        for i in range(b.n):
            assert np.array_equal(r.runs_of(i), ref.runs_of(i))


def test_graph_and_direct_launches_agree(batch_aligner):
    """wfg_run's device work as a captured CUDA graph (updated in place across batches of
    different sizes and schedules) gives the results of direct launches."""
    outs = {}
    for graph in (True, False):
        batch_aligner.set_graph(graph)
        try:
            for n, seed in ((120, 5), (37, 6), (120, 7)):
                b = pkg.PairBatch.generate(5, n, seed=seed)
                for sched in (_capi.SCHED_PLAIN, _capi.SCHED_LEARNED):
                    batch_aligner.upload(b)
                    if sched == _capi.SCHED_LEARNED:
                        batch_aligner.set_predictions(np.asarray(b.plen, np.float32) * 0.3)
                    batch_aligner.run(sched=sched)
                    st = batch_aligner.stats()
                    assert st.used_graph == int(graph)
                    outs[(graph, n, seed, sched)] = batch_aligner.fetch()
        finally:
            batch_aligner.set_graph(True)
    for (graph, n, seed, sched), r in outs.items():
        d = outs[(False, n, seed, sched)]
        assert (r.status == 0).all()
        assert np.array_equal(r.scores, d.scores)
        for i in range(n):
            assert np.array_equal(r.runs_of(i), d.runs_of(i))


def _mutate(rng, seq: bytes, n_edits: int) -> bytes:
    s = bytearray(seq)
    for _ in range(n_edits):
        i = int(rng.integers(0, len(s)))
        kind = int(rng.integers(0, 3))
        if kind == 0:
            s[i] = b"ACGT"[(b"ACGT".index(s[i]) + 1 + int(rng.integers(0, 3))) % 4]
        elif kind == 1:
            s.insert(i, b"ACGT"[int(rng.integers(0, 4))])
        else:
            del s[i]
    return bytes(s)


def test_long_low_error_pairs_match_oracle(batch_aligner):
    """Long pairs (up to 32 kbp) with long exact runs between edits: deep LCP loops, three
    recursion levels, and the same results through the tiny-arena retry passes."""
    rng = np.random.default_rng(77)
    pats, txts = [], []
    for L in (32766, 32000, 20000, 8000):
        p = bytes(rng.choice(list(b"ACGT"), L).astype(np.uint8))
        pats.append(p)
        txts.append(_mutate(rng, p, L // 200)[:32766])
    b = pkg.PairBatch.from_lists(pats, txts)
    res = batch_aligner.align(b)
    try:
        batch_aligner.set_arena_limits(ring_w=32, leaf_words=256)
        small = batch_aligner.align(b)
    finally:
        batch_aligner.set_arena_limits(0, 0)
    for i in range(b.n):
        st, score, ops, _ = binding.oracle_align(pats[i], txts[i])
        assert st == 0 and res.status[i] == 0 and small.status[i] == 0
        assert res.scores[i] == score and small.scores[i] == score
        assert pkg.runs_to_ops(res.runs_of(i)) == ops
        assert np.array_equal(small.runs_of(i), res.runs_of(i))


def test_wfa2_single_pair_api():
    data = utest()
    s = data["sets"]["test.biwfa.affine.alg"]
    al = pkg.WavefrontAligner(0, 4, 6, 2)
    try:
        for i in (0, 5, 77, 150, 304):
            p, t = data["pairs"][i]
            assert al.align(p, t) == _capi.WF_STATUS_ALG_COMPLETED
            assert al.status == 0
            line = printed_line(al.cigar_score(), al.cigar_str())
            assert line == s["lines"][i]
            assert al.score == al.cigar_score()
            sam = al.sam_cigar(True)
            assert sum(x >> 4 for x in sam) == len(al.cigar_ops())
        # empty inputs
        assert al.align("", "") == 0 and al.cigar_str() == ""
        assert al.align("ACGT", "") == 0 and al.cigar_str() == "4D" and al.score == -(6 + 2 * 4)
        st, out = al.align_batch(["GATTACA", "ACGT"], ["GATCACA", "ACGT"])
        assert st == 0 and out[0] == (0, -4, "3M1X3M") and out[1] == (0, 0, "4M")
    finally:
        al.close()


def test_wfa2_api_refuses_unsupported_configurations():
    for kw in (dict(memory_mode=_capi.WAVEFRONT_MEMORY_HIGH), dict(heuristic=_capi.WF_HEURISTIC_WFADAPTIVE),
               dict(match=1), dict(mismatch=0)):
        al = pkg.WavefrontAligner(**kw)
        try:
            assert al.align("ACGT", "ACGT") == _capi.WF_STATUS_UNSUPPORTED
        finally:
            al.close()


def _check_properties(b, res, penalties=(0, 4, 6, 2)):
    """Size-independent checks of every pair: status, consumed lengths, score = rescore(CIGAR)."""
    m, x, o, e = penalties
    assert (res.status == 0).all()
    runs = res.runs.astype(np.int64)
    op = runs & 15
    ln = runs >> 4
    pair_of = np.repeat(np.arange(b.n), res.run_len)
    order = np.argsort(res.run_off, kind="stable")
    # runs are contiguous per pair: rebuild pair ids in run-buffer order
    pair_of = np.empty(runs.shape[0], np.int64)
    for_pos = np.repeat(order, res.run_len[order])
    pair_of[:] = for_pos
    cons_p = np.bincount(pair_of, weights=ln * np.isin(op, [7, 8, 2]), minlength=b.n)
    cons_t = np.bincount(pair_of, weights=ln * np.isin(op, [7, 8, 1]), minlength=b.n)
    assert np.array_equal(cons_p.astype(np.int64), b.plen.astype(np.int64))
    assert np.array_equal(cons_t.astype(np.int64), b.tlen.astype(np.int64))
    pen = np.where(op == 7, -m * ln, np.where(op == 8, -x * ln, -(o + e * ln)))
    sc = np.bincount(pair_of, weights=pen, minlength=b.n).astype(np.int64)
    assert np.array_equal(sc, res.scores.astype(np.int64))
    # adjacent runs of one pair never share an op (maximal runs)
    same = (pair_of[1:] == pair_of[:-1]) & (op[1:] == op[:-1])
    assert not same.any()


@pytest.mark.parametrize("workload,n,checked", [(1, 10_000, 10_000), (2, 1_000_000, 1_000_000),
                                                (3, 200_000, 200_000), (4, 2_000, 200), (5, 1_000_000, 1_000_000)])
def test_full_size_workloads(batch_aligner, workload, n, checked):
    """Full-size workloads: every pair checked by properties, and every pair (the long noisy
    workload: a seeded 200 of its 2,000) bit-exact against the oracle on all host threads —
    status, score and the whole operation string."""
    b = pkg.PairBatch.generate(workload, n, seed=5000 + workload)
    res = batch_aligner.align(b)
    _check_properties(b, res)
    idx = None if checked == n else np.sort(np.random.default_rng(workload).choice(n, size=checked, replace=False))
    r = binding.check_batch(b.seq, b.p_off, b.plen, b.t_off, b.tlen, res.scores, res.status, res.runs, res.run_off,
                            res.run_len, idx=idx)
    print(f"workload {workload}: {r['checked']} pairs checked against the oracle, {r['mismatches']} mismatches")
    assert r["checked"] == checked
    assert r["mismatches"] == 0, f"{r['mismatches']} of {checked} pairs differ, first {r['first_bad']}"


def test_scope_above_64_is_refused(batch_aligner):
    """Penalties whose score scope exceeds every kernel instantiation's cap are refused with a
    status and a message, not run with a wrong ring."""
    b = pkg.PairBatch.from_lists(["ACGTACGT"], ["ACGAACGT"])
    batch_aligner.upload(b)
    with pytest.raises(RuntimeError, match="max_score_scope"):
        batch_aligner.run((0, 4, 60, 10))
    res = batch_aligner.align(b, penalties=(0, 20, 30, 10))  # scope 41: the scope-64 kernel
    st, score, ops, _ = binding.oracle_align(b.pattern(0), b.text(0), (0, 20, 30, 10))
    assert res.status[0] == 0 and pkg.runs_to_ops(res.runs_of(0)) == ops and res.scores[0] == score


def test_gpu_matches_oracle_on_random_penalties(batch_aligner):
    """Random penalty sets for every distance (gap-open 0 and match < 0 included, score scope
    within 64) on mutated pairs: the GPU path against the oracle, full CIGAR and score-only."""
    rng = np.random.default_rng(4242)
    metrics = {0: _capi.METRIC_GAP_AFFINE, 1: _capi.METRIC_EDIT, 2: _capi.METRIC_INDEL, 3: _capi.METRIC_GAP_LINEAR,
               4: _capi.METRIC_GAP_AFFINE_2P}
    b = pkg.PairBatch.generate(5, 40, seed=43)
    for trial in range(24):
        m = -int(rng.integers(0, 3))
        x, o, e = int(rng.integers(1, 7)), int(rng.integers(0, 9)), int(rng.integers(1, 4))
        cands = [(0, (m, x, o, e)), (3, (m, x, int(rng.integers(1, 7)), 0)),
                 (4, (m, x, o, e, int(rng.integers(0, 16)), int(rng.integers(1, 4)))), (1, (0, 0, 0, 0)),
                 (2, (0, 0, 0, 0))]
        om, pen = cands[trial % len(cands)]
        for score_only in (False, True):
            res = batch_aligner.align(b, penalties=pen, metric=metrics[om], score_only=score_only)
            for i in range(b.n):
                st, score, ops, _ = binding.oracle_align(b.pattern(i), b.text(i), pen, score_only, metric=om)
                assert res.status[i] == st, (pen, om, i)
                if score_only:
                    assert res.scores[i] == score, (pen, om, i)
                else:
                    assert pkg.runs_to_ops(res.runs_of(i)) == ops and res.scores[i] == (score if ops else 0), (pen, om, i)


@pytest.mark.parametrize("distance,pen,golden", [
    (_capi.GAP_AFFINE_2P, (0, 4, 6, 2, 24, 1), "test.biwfa.affine2p.alg"),
    (_capi.GAP_LINEAR, (0, 4, 2, 0), None),
    (_capi.EDIT, (0, 0, 0, 0), "test.biwfa.edit.alg"),
    (_capi.INDEL, (0, 0, 0, 0), "test.biwfa.indel.alg")], ids=["affine2p", "gap_linear", "edit", "indel"])
def test_wfa2_single_pair_api_other_distances(distance, pen, golden):
    """WFA2-lib's aligner API with the other distances: the operations and cigar_score() of
    each pair equal the oracle's, and the printed `score\\tCIGAR` line equals WFA2-lib's own
    golden line where WFA2-lib ships one."""
    metric = {_capi.GAP_AFFINE_2P: binding.METRIC_AFFINE2P, _capi.GAP_LINEAR: binding.METRIC_LINEAR,
              _capi.EDIT: binding.METRIC_EDIT, _capi.INDEL: binding.METRIC_INDEL}[distance]
    data = utest()
    o2, e2 = (pen[4], pen[5]) if len(pen) == 6 else (24, 1)
    al = pkg.WavefrontAligner(*pen[:4], distance=distance, gap_opening2=o2, gap_extension2=e2)
    try:
        for i in (0, 3, 41, 150, 222, 304):
            p, t = data["pairs"][i]
            assert al.align(p, t) == _capi.WF_STATUS_ALG_COMPLETED
            st, score, ops, _ = binding.oracle_align(p, t, pen, metric=metric)
            assert st == 0 and al.cigar_ops() == ops, i
            assert al.cigar_score() == score, i
            if golden:
                assert printed_line(al.cigar_score(), al.cigar_str()) == data["sets"][golden]["lines"][i], i
    finally:
        al.close()
