"""The CPU oracle (oracle/biwfa_oracle.c) pinned against WFA2-lib's golden files and
against the real WFA2-lib built from the reference sources."""
import numpy as np
import pytest

from golden_data import printed_line, ref_cases, utest
from oracle import binding

UTEST_NAMES = sorted(utest()["sets"].keys())


@pytest.mark.parametrize("name", UTEST_NAMES)
def test_oracle_matches_wfa2_utest_goldens(name):
    data = utest()
    s = data["sets"][name]
    pen, score_only, metric = tuple(s["penalties"]), s["score_only"], s.get("metric", 0)
    bad = []
    for i, (p, t) in enumerate(data["pairs"]):
        st, score, ops, _ = binding.oracle_align(p, t, pen, score_only, metric=metric)
        line = printed_line(score, "" if score_only else binding.rle(ops))
        if st != 0 or line != s["lines"][i]:
            bad.append(i)
    assert not bad, f"{name}: {len(bad)} of {len(data['pairs'])} pairs differ, first {bad[:5]}"


@pytest.mark.parametrize("case", ref_cases(), ids=lambda c: c["tag"])
def test_oracle_matches_wfa2_reference_cases(case):
    pen, score_only, metric = tuple(case["penalties"]), case["score_only"], case.get("metric", 0)
    for p, t, st_ref, score_ref, cig_ref in case["pairs"]:
        st, score, ops, _ = binding.oracle_align(p, t, pen, score_only, metric=metric)
        assert st == st_ref
        assert score == score_ref
        if not score_only:
            assert (binding.rle(ops) if ops else "-") == cig_ref


def test_oracle_matches_live_reference_on_random_pairs():
    if binding.build_ref() is None:
        pytest.skip("WFA2-lib reference sources not mounted here")
    rng = np.random.default_rng(77)
    for trial in range(120):
        n = int(rng.integers(0, 400))
        p = "".join(rng.choice(list("ACGT"), n))
        t = list(p)
        for _ in range(int(rng.integers(0, 40))):
            if not t:
                break
            pos = int(rng.integers(0, len(t)))
            r = rng.random()
            if r < 0.4:
                t[pos] = str(rng.choice(list("ACGT")))
            elif r < 0.7:
                t.insert(pos, str(rng.choice(list("ACGT"))) * int(rng.integers(1, 6)))
            else:
                del t[pos:pos + int(rng.integers(1, 6))]
        t = "".join(t)
        pen = [(0, 4, 6, 2), (0, 1, 2, 1), (0, 5, 3, 2), (-3, 5, 3, 2)][trial % 4]
        for metric in (binding.METRIC_AFFINE, binding.METRIC_EDIT, binding.METRIC_INDEL, binding.METRIC_LINEAR,
                       binding.METRIC_AFFINE2P):
            # gap-linear reads (match, mismatch, indel) from the first three penalties; the
            # two-piece distance adds a second gap piece (o2, e2) = (4*o1, max(e1 - 1, 1))
            mpen = (pen[0], pen[1], pen[3] + 1, 0) if metric == binding.METRIC_LINEAR else pen
            if metric == binding.METRIC_AFFINE2P:
                mpen = tuple(pen) + (4 * pen[2], max(pen[3] - 1, 1))
            ref = binding.ref_align(p, t, mpen, metric=metric)
            st, score, ops, _ = binding.oracle_align(p, t, mpen, metric=metric)
            assert (st, score, ops) == (ref[0], ref[1], ref[2]), (p, t, mpen, metric)


def test_oracle_batch_threads_agree_with_single():
    import biwfa_gpu_pii2025_gb300 as pkg
    b = pkg.PairBatch.generate(3, 40, seed=9)
    secs1, s1, st1 = binding.oracle_batch_time(b.seq, b.p_off, b.plen, b.t_off, b.tlen, threads=1)
    secs4, s4, st4 = binding.oracle_batch_time(b.seq, b.p_off, b.plen, b.t_off, b.tlen, threads=4)
    assert (st1 == 0).all() and (st4 == 0).all()
    assert (s1 == s4).all()
    for i in range(0, b.n, 7):
        assert binding.oracle_align(b.pattern(i), b.text(i))[1] == s1[i]


def test_oracle_matches_live_reference_on_random_penalties():
    """Random penalty sets for every distance (match <= 0 included, two-piece openings on either
    side of the first piece's), a few mutated pairs each, full CIGAR and score-only."""
    if binding.build_ref() is None:
        pytest.skip("WFA2-lib reference sources not mounted here")
    rng = np.random.default_rng(2026)
    for trial in range(300):
        m = -int(rng.integers(0, 4))
        x, o, e = int(rng.integers(1, 9)), int(rng.integers(0, 11)), int(rng.integers(1, 6))
        sets = [(binding.METRIC_AFFINE, (m, x, o, e)),
                (binding.METRIC_LINEAR, (m, x, int(rng.integers(1, 9)), 0)),
                (binding.METRIC_AFFINE2P, (m, x, o, e, int(rng.integers(0, 30)), int(rng.integers(1, 6)))),
                (binding.METRIC_EDIT, (0, 0, 0, 0)), (binding.METRIC_INDEL, (0, 0, 0, 0))]
        n = int(rng.integers(1, 260 if trial % 10 else 1500))
        p = "".join(rng.choice(list("ACGT"), n))
        t = list(p)
        for _ in range(int(rng.integers(0, 25))):
            if not t:
                break
            pos = int(rng.integers(0, len(t)))
            r = rng.random()
            if r < 0.4:
                t[pos] = str(rng.choice(list("ACGT")))
            elif r < 0.7:
                t.insert(pos, "".join(rng.choice(list("ACGT"), int(rng.integers(1, 12)))))
            else:
                del t[pos:pos + int(rng.integers(1, 12))]
        t = "".join(t)
        for metric, pen in sets:
            for score_only in (False, True):
                ref = binding.ref_align(p, t, pen, score_only, metric=metric)
                st, score, ops, _ = binding.oracle_align(p, t, pen, score_only, metric=metric)
                assert (st, score, ops) == (ref[0], ref[1], ref[2]), (p, t, pen, metric, score_only)


def _runs_of_ops(ops: bytes):
    code = {ord("M"): 7, ord("X"): 8, ord("I"): 1, ord("D"): 2}
    runs, j = [], 0
    while j < len(ops):
        e = j
        while e < len(ops) and ops[e] == ops[j]:
            e += 1
        runs.append(((e - j) << 4) | code[ops[j]])
        j = e
    return runs


def test_batch_checker_finds_a_planted_difference():
    """The whole-batch checker the full-size GPU tests and the bench use: results rebuilt from
    the oracle's own operations pass; one planted change (in a copy of those results, on the
    CPU) is found and named."""
    import biwfa_gpu_pii2025_gb300 as pkg
    b = pkg.PairBatch.generate(5, 240, 3)
    _, sc, st, (ops, off, ln) = binding.oracle_batch_time(b.seq, b.p_off, b.plen, b.t_off, b.tlen, threads=4,
                                                          return_ops="raw")
    runs, roff, rlen = [], [], []
    for i in range(b.n):
        r = _runs_of_ops(ops[off[i]:off[i] + ln[i]].tobytes())
        roff.append(len(runs)); rlen.append(len(r)); runs += r
    runs = np.array(runs, np.uint32); roff = np.array(roff, np.int64); rlen = np.array(rlen, np.int32)
    scores = np.where(ln > 0, sc, 0)
    ok = binding.check_batch(b.seq, b.p_off, b.plen, b.t_off, b.tlen, scores, st, runs, roff, rlen, chunk=64)
    assert ok["checked"] == b.n and ok["mismatches"] == 0
    planted = runs.copy()
    planted[roff[17]] += 16  # one more base in pair 17's first run
    bad = binding.check_batch(b.seq, b.p_off, b.plen, b.t_off, b.tlen, scores, st, planted, roff, rlen)
    assert bad["mismatches"] == 1 and bad["first_bad"] == [17]
    s2 = scores.copy(); s2[5] -= 2
    assert binding.check_batch(b.seq, b.p_off, b.plen, b.t_off, b.tlen, s2, st, runs, roff, rlen)["first_bad"] == [5]


def test_wfa2_threaded_batch_matches_oracle():
    """The timed CPU baseline (the real WFA2-lib, one aligner per thread) gives the oracle's
    status, score and operations on every pair."""
    if binding.ref_lib() is None:
        pytest.skip("WFA2-lib not built here")
    import biwfa_gpu_pii2025_gb300 as pkg
    b = pkg.PairBatch.generate(5, 600, 8)
    _, s1, t1, (o1, f1, l1) = binding.oracle_batch_time(b.seq, b.p_off, b.plen, b.t_off, b.tlen, threads=4,
                                                        return_ops="raw")
    _, s2, t2, (o2, f2, l2) = binding.ref_batch_time(b.seq, b.p_off, b.plen, b.t_off, b.tlen, threads=4,
                                                     return_ops=True)
    assert np.array_equal(s1, s2) and np.array_equal(t1, t2) and np.array_equal(l1, l2)
    assert all(o1[f1[i]:f1[i] + l1[i]].tobytes() == o2[f2[i]:f2[i] + l2[i]].tobytes() for i in range(b.n))
