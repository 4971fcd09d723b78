"""The end-to-end call (wfg_align_host) overlaps its input copy with the alignment on large
batches: chunked uploads, per-chunk packing, prediction and ordering, per-chunk first passes,
one set of retry passes. Results must equal the upload-then-run path's, pair for pair."""
import numpy as np
import pytest

import biwfa_gpu_pii2025_gb300 as pkg
from biwfa_gpu_pii2025_gb300 import _capi

pytestmark = pytest.mark.gpu

N = 160_000  # above the 131,072-pair threshold: three chunks


def _align_into(al, hb, n, sched):
    pin = pkg.PinnedHost()
    try:
        cap = int(hb.plen.astype(np.int64).sum() + hb.tlen.astype(np.int64).sum() + n)
        out = pkg.BatchResult(pin.empty(n, np.int32), pin.empty(n, np.int32), pin.empty(n, np.int64),
                              pin.empty(n, np.int32), pin.empty(cap, np.uint32))
        total = al.align_into(hb, out, sched=sched)
        st = al.stats()
        res = pkg.BatchResult(out.scores.copy(), out.status.copy(), out.run_off.copy(), out.run_len.copy(),
                              out.runs[:total].copy())
    finally:
        pin.close()
    return res, st


def _same(a, b, n):
    assert np.array_equal(a.status, b.status) and np.array_equal(a.scores, b.scores)
    assert np.array_equal(a.run_len, b.run_len)
    for i in range(0, n, 997):
        assert np.array_equal(a.runs_of(i), b.runs_of(i)), i


@pytest.mark.parametrize("sched", [_capi.SCHED_SORTED, _capi.SCHED_LEARNED], ids=["sorted", "learned"])
def test_pipelined_end_to_end_matches_upload_then_run(batch_aligner, sched):
    b = pkg.PairBatch.generate(5, N, seed=606)
    al = batch_aligner
    pred = None
    if sched == _capi.SCHED_LEARNED:
        al.upload(b)
        pred = pkg.ScorePredictor(al, seed=4)
        pred.train(-((b.plen.astype(np.int64) + b.tlen) // 8).astype(np.int32), epochs=1, batch_rows=4096, lr=1e-3)
        pred.attach()
        al.set_learned_policy(wide_threshold=3.4e38, wide_warps=8, wide_smem=False, ring_margin=1.4)
    pin = pkg.PinnedHost()
    try:
        hb = pin.batch(b)
        al.set_pipeline(True)
        piped, st_p = _align_into(al, hb, N, sched)
        al.set_pipeline(False)
        plain, st_u = _align_into(al, hb, N, sched)
    finally:
        al.set_pipeline(True)
        al.set_learned_policy()
        if pred is not None:
            pred.close()
        pin.close()
    assert st_p.pipeline_chunks >= 2 and st_u.pipeline_chunks == 0
    assert (piped.status == 0).all()
    _same(piped, plain, N)
    # and the resident-batch path
    ref = al.align(b, sched=_capi.SCHED_SORTED)
    _same(piped, ref, N)
