"""Every execution shape (warps per pair, rings in shared or global memory) gives the same
bit-exact results as the oracle and WFA2-lib's goldens."""
import numpy as np
import pytest

import biwfa_gpu_pii2025_gb300 as pkg
from golden_data import printed_line, utest
from oracle import binding

pytestmark = pytest.mark.gpu

SHAPES = [(1, False), (4, False), (4, True), (8, False), (8, True)]


@pytest.mark.parametrize("gw,smem", SHAPES)
def test_shape_matches_oracle(batch_aligner, gw, smem):
    b = pkg.PairBatch.generate(5, 240, seed=300 + gw)
    long_pairs = pkg.PairBatch.generate(3, 12, seed=301)
    try:
        batch_aligner.set_exec_shape(gw, smem)
        for batch in (b, long_pairs):
            res = batch_aligner.align(batch)
            _, scores, status, ops = binding.oracle_batch_time(batch.seq, batch.p_off, batch.plen, batch.t_off,
                                                               batch.tlen, threads=8, return_ops=True)
            assert (res.status == 0).all()
            bad = [i for i in range(batch.n) if pkg.runs_to_ops(res.runs_of(i)) != ops[i] or
                   res.scores[i] != (scores[i] if ops[i] else 0)]
            assert not bad, (gw, smem, bad[:5])
    finally:
        batch_aligner.set_exec_shape(1, False)


@pytest.mark.parametrize("gw,smem", SHAPES[1:])
def test_shape_matches_wfa2_goldens(batch_aligner, gw, smem):
    data = utest()
    b = pkg.PairBatch.from_lists([p for p, _ in data["pairs"]], [t for _, t in data["pairs"]])
    try:
        batch_aligner.set_exec_shape(gw, smem)
        for name in ("test.biwfa.affine.alg", "test.biwfa.affine.p1.alg", "test.biwfa.score.affine.alg"):
            s = data["sets"][name]
            res = batch_aligner.align(b, penalties=tuple(s["penalties"]), score_only=s["score_only"])
            for i in range(b.n):
                if s["score_only"]:
                    line = printed_line(int(res.scores[i]), "")
                else:
                    cig = res.cigar(i)
                    line = printed_line(int(res.scores[i]) if cig else -1, cig)
                assert line == s["lines"][i], (name, i)
    finally:
        batch_aligner.set_exec_shape(1, False)


def test_learned_policy_with_wide_shapes_keeps_results(batch_aligner):
    b = pkg.PairBatch.generate(5, 600, seed=333)
    ref = batch_aligner.align(b)
    # synthetic predictions: the true scores scaled, so some pairs take the wide shapes
    pred = (-ref.scores).astype(np.float32) * np.random.default_rng(2).uniform(0.5, 1.5, b.n).astype(np.float32)
    for thr, gw, smem in [(300.0, 8, True), (300.0, 4, False), (50.0, 8, False)]:
        batch_aligner.set_learned_policy(thr, gw, smem, 1.2)
        batch_aligner.upload(b)
        batch_aligner.set_predictions(pred)
        batch_aligner.run(sched=pkg._capi.SCHED_LEARNED)
        got = batch_aligner.fetch()
        assert np.array_equal(got.scores, ref.scores) and (got.status == 0).all()
        for i in range(b.n):
            assert np.array_equal(got.runs_of(i), ref.runs_of(i)), (thr, gw, smem, i)
    batch_aligner.set_learned_policy()
