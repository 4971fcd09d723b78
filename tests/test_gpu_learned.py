"""Learned scheduling on the GPU: features and gradients against the float64 CPU oracle
(oracle/mlp_oracle.py), training on plain-method scores, and results that never depend on
the model."""
import time

import numpy as np
import pytest

import biwfa_gpu_pii2025_gb300 as pkg
from biwfa_gpu_pii2025_gb300 import _capi
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def aligner():
    al = pkg.BatchAligner(0)
    yield al
    al.close()


def test_features_match_oracle(aligner):
    b = pkg.PairBatch.generate(5, 300, seed=61)
    extra = pkg.PairBatch.from_lists(["", "ACG", "ACGTNNACGT" * 20], ["ACGT", "", "ACGTACGT" * 25])
    for batch in (b, extra):
        aligner.upload(batch)
        pred = pkg.ScorePredictor(aligner, seed=3)
        got = mo.bf16_bits_to_float(pred.features())
        pred.close()
        ref = np.stack([mo.features(batch.pattern(i), batch.text(i)) for i in range(batch.n)])
        # equal after bf16 rounding, up to one bf16 ulp where float32 and float64 round apart
        np.testing.assert_allclose(got, mo.bf16_round(ref), rtol=2 ** -7, atol=1e-6)


def test_gradient_matches_float64_oracle(aligner):
    b = pkg.PairBatch.generate(5, 500, seed=62)
    aligner.upload(b)
    pred = pkg.ScorePredictor(aligner, seed=11)
    try:
        rng = np.random.default_rng(5)
        params = (rng.standard_normal(mo.N_PARAMS) * 0.2).astype(np.float32)
        pred.set_params(params)
        X = mo.bf16_bits_to_float(pred.features())
        t = rng.uniform(0, 8, b.n).astype(np.float32)
        loss_gpu, g_gpu = pred.gradient(t)
        loss_ref, g_ref = mo.loss_and_grad(params.astype(np.float64), X, t.astype(np.float64))
        assert abs(loss_gpu - loss_ref) <= 1e-3 * max(1.0, abs(loss_ref))
        # fp32 accumulation on the device vs float64 here: relative error of the whole gradient
        err = np.linalg.norm(g_gpu - g_ref) / np.linalg.norm(g_ref)
        assert err < 1e-3, err
        for name, a, z in [("W1", mo.OFF_W1, mo.OFF_B1), ("W2", mo.OFF_W2, mo.OFF_B2), ("w3", mo.OFF_W3, mo.OFF_B3)]:
            e = np.linalg.norm(g_gpu[a:z] - g_ref[a:z]) / max(np.linalg.norm(g_ref[a:z]), 1e-12)
            assert e < 5e-3, (name, e)
    finally:
        pred.close()


def test_training_learns_scores_and_schedule_keeps_results(aligner):
    train = pkg.PairBatch.generate(5, 6000, seed=9001)       # held-out seed for training
    res = aligner.align(train, score_only=True)
    assert (res.status == 0).all()
    pred = pkg.ScorePredictor(aligner, seed=5)
    try:
        losses = pred.train(-res.scores, epochs=25, batch_rows=1024, lr=3e-3)
        assert losses[-1] < 0.5 * losses[0], losses
        test = pkg.PairBatch.generate(5, 3000, seed=77)
        ref = aligner.align(test)
        aligner.upload(test)
        p = pred.predict()
        truth = np.log1p(-ref.scores.astype(np.float64))
        rank_corr = np.corrcoef(np.argsort(np.argsort(p)), np.argsort(np.argsort(truth)))[0, 1]
        assert rank_corr > 0.85, rank_corr
        # learned schedule on the device: results identical to the plain path
        pred.attach()
        aligner.run(sched=_capi.SCHED_LEARNED)
        got = aligner.fetch()
        assert np.array_equal(got.scores, ref.scores) and np.array_equal(got.status, ref.status)
        for i in range(test.n):
            assert np.array_equal(got.runs_of(i), ref.runs_of(i))
    finally:
        pred.close()


def test_trained_network_gains_over_the_method_without_it(aligner):
    """What the trained network adds: (1) it ranks pairs by alignment cost better than pair
    length (the plain path's only signal), since error rates vary 10x at equal length; (2) the
    learned-binned persistent schedule aligns a mixture batch faster than the plain length-
    sorted batched path, with identical results (the speed-up is measured, with a wide margin
    so that it holds on any GB300)."""
    train = pkg.PairBatch.generate(5, 20000, seed=9101)
    res = aligner.align(train, score_only=True)
    pred = pkg.ScorePredictor(aligner, seed=5)
    try:
        pred.train(-res.scores, epochs=20, batch_rows=1024, lr=3e-3)
        test = pkg.PairBatch.generate(5, 200000, seed=9102)  # large enough that no single pair sets the time
        ref = aligner.align(test, sched=_capi.SCHED_PLAIN)
        aligner.upload(test)
        p = pred.predict()
        cost = -ref.scores.astype(np.float64)
        rank = lambda v: np.argsort(np.argsort(v, kind="stable"), kind="stable")
        corr_net = np.corrcoef(rank(p), rank(cost))[0, 1]
        corr_len = np.corrcoef(rank(test.plen + test.tlen), rank(cost))[0, 1]
        assert corr_net > corr_len + 0.02, (corr_net, corr_len)
        # among pairs of similar length, only the network separates cheap from costly ones
        heavy = test.plen > 3000
        c_net = np.corrcoef(rank(p[heavy]), rank(cost[heavy]))[0, 1]
        c_len = np.corrcoef(rank((test.plen + test.tlen)[heavy]), rank(cost[heavy]))[0, 1]
        assert c_net > c_len + 0.1, (c_net, c_len)
        pred.attach()
        times = {}
        for sched in (_capi.SCHED_PLAIN, _capi.SCHED_LEARNED):
            best = None
            for _ in range(3):
                aligner.synchronize()
                t0 = time.perf_counter()
                aligner.run(sched=sched)  # learned: features, MLP, binning and alignment
                aligner.synchronize()
                ms = 1e3 * (time.perf_counter() - t0)
                best = ms if best is None else min(best, ms)
            times[sched] = best
            got = aligner.fetch()
            assert np.array_equal(got.scores, ref.scores) and np.array_equal(got.status, ref.status)
        assert times[_capi.SCHED_LEARNED] < 0.8 * times[_capi.SCHED_PLAIN], times
    finally:
        aligner.lib.wfg_set_model(aligner.ctx, None)
        pred.close()
