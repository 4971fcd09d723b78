"""Test infrastructure: the algorithmic work of the BiWFA path per config, counted in the
oracle on seeded samples of each workload:
  N_cells = sum over every compute step (both directions, every recursion level, leaves) of
            components x (hi - lo + 1);
  N_ext   = sum over every extended diagonal of (matched characters + 1);
  steps   = compute steps.
Prints per-pair means (and the sample size) for the gap-affine penalties (0,4,6,2).

    python oracle/work_counts.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import biwfa_gpu_pii2025_gb300 as pkg  # noqa: E402
from oracle import binding  # noqa: E402

# (workload, generated pairs, sampled pairs)
CONFIGS = ((1, 10_000, 200), (2, 200_000, 5_000), (3, 200_000, 400), (4, 2_000, 4), (5, 200_000, 1_200))


def main() -> int:
    for wl, n_gen, n in CONFIGS:
        b = pkg.PairBatch.generate(wl, n_gen, 20251203)
        idx = np.random.default_rng(99).permutation(b.n)[:n]
        cells = ext = steps = 0
        for i in idx:
            _, _, _, r = binding.oracle_align(b.pattern(int(i)), b.text(int(i)))
            cells += r.n_cells
            ext += r.n_ext
            steps += r.n_steps
        print(f"workload {wl}: {n} pairs sampled; per pair N_cells {cells / n:.4g}, N_ext {ext / n:.4g}, "
              f"steps {steps / n:.4g}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
