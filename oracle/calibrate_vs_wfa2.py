"""Test infrastructure: times the oracle (oracle/biwfa_oracle.c) against the real WFA2-lib
(oracle/_ref/libwfa2_ref.so, built from the reference sources by `make -C oracle ref`) on the
same seeded pairs, one thread each, one aligner reused across pairs (as align_benchmark does
per thread), full CIGAR, penalties (0,4,6,2); checks that the scores are identical.

It calibrates the CPU baseline that bench.py reports: on the GPU machine the WFA2-lib sources
are absent, so the baseline there is the oracle port. Runs only where the reference is mounted.

    python oracle/calibrate_vs_wfa2.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import biwfa_gpu_pii2025_gb300 as pkg  # noqa: E402
from oracle import binding  # noqa: E402

# (workload, pairs generated, pairs sampled)
CASES = ((5, 200_000, 3000), (1, 10_000, 300), (2, 200_000, 20_000), (3, 200_000, 400))
REPEATS = 5


def main() -> int:
    if binding.build_ref() is None:
        print("WFA2-lib sources not found; nothing to calibrate")
        return 0
    ref = binding.ref_lib()
    ref.ref_biwfa_batch_time.restype = C.c_double
    i64p, ip = C.POINTER(C.c_longlong), C.POINTER(C.c_int)
    for wl, n_gen, n in CASES:
        b = pkg.PairBatch.generate(wl, n_gen, 20251203)
        sub = b.subset(np.random.default_rng(99).permutation(b.n)[:n])
        scores = np.empty(sub.n, np.int32)
        po = np.ascontiguousarray(sub.p_off, np.int64)
        to = np.ascontiguousarray(sub.t_off, np.int64)
        pl = np.ascontiguousarray(sub.plen, np.int32)
        tl = np.ascontiguousarray(sub.tlen, np.int32)
        ratios, same = [], True
        for _ in range(REPEATS):  # alternating, so that host noise hits both sides alike
            secs_o, sc_o, _ = binding.oracle_batch_time(sub.seq, sub.p_off, sub.plen, sub.t_off, sub.tlen, threads=1)
            secs_r = ref.ref_biwfa_batch_time(C.c_int(sub.n), sub.seq.ctypes.data_as(C.c_char_p),
                                              po.ctypes.data_as(i64p), pl.ctypes.data_as(ip), to.ctypes.data_as(i64p),
                                              tl.ctypes.data_as(ip), 0, 4, 6, 2, scores.ctypes.data_as(ip))
            ratios.append(secs_r / secs_o)
            same = same and bool(np.array_equal(scores, sc_o))
        print(f"workload {wl}, {sub.n} pairs: oracle speed / WFA2-lib speed median {np.median(ratios):.2f} "
              f"(range {min(ratios):.2f}-{max(ratios):.2f}, {REPEATS} alternating runs), scores identical {same}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
