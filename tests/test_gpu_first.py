"""First GPU parity check: generated workloads vs the oracle, bit-exact score + CIGAR."""
import pytest

import biwfa_gpu_pii2025_gb300 as pkg
from oracle import binding

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("workload,n", [(1, 64), (2, 256), (3, 24)])
def test_generated_vs_oracle(batch_aligner, workload, n):
    b = pkg.PairBatch.generate(workload, n, seed=1234 + workload)
    res = batch_aligner.align(b)
    bad = []
    for i in range(b.n):
        st, score, ops, _ = binding.oracle_align(b.pattern(i), b.text(i))
        got = pkg.runs_to_ops(res.runs_of(i))
        if res.status[i] != 0 or got != ops or res.scores[i] != (score if ops else 0):
            bad.append(i)
    assert not bad, f"{len(bad)} mismatching pairs, first {bad[:5]}"
