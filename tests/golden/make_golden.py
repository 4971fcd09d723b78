"""Regenerates the golden fixtures in this folder (run where the reference project is present;
WFA2_SRC names its WFA2-lib folder).

1. wfa2_utest.json.gz — WFA2-lib's own test vectors for this path, read as text from
   WFA2-lib/tests/: the 305 input pairs (wfa.utest.seq) and the expected `score\\tCIGAR`
   lines of the BiWFA gap-affine runs (test.biwfa.affine{,.p0..p5}.alg), the BiWFA
   score-only runs (test.biwfa.score.affine{,.p0..p5}.alg) and the BiWFA edit and indel
   runs (test.biwfa{,.score}.{edit,indel}.alg) and the BiWFA two-piece gap-affine runs
   (test.biwfa{,.score}.affine2p.alg, align_benchmark's default penalties 0,4,6,2,24,1).
   Penalties per file follow WFA2-lib/tests/wfa.utest.sh:45-59; "metric" is 0 gap-affine,
   1 edit, 2 indel, 4 two-piece gap-affine.
2. wfa2_ref_cases.json.gz — outputs of the real WFA2-lib v2.3 (oracle/_ref/libwfa2_ref.so,
   compiled from the reference sources by oracle/Makefile) on seeded synthetic pairs of
   every workload and on edge cases, for the gap-affine, edit, indel, gap-linear and two-piece
   gap-affine distances ("metric" 0, 1, 2, 3, 4), so the GPU tests can pin parity on the GPU machine where the
   reference is absent.
3. wfa2_abi_layout.txt — sizeof / offsetof of the structures a drop-in must match byte for byte
   (tests/cpp/abi_layout.c compiled against WFA2-lib's own headers), so the layout test runs
   where those headers are absent.

Usage:  WFA2_SRC=<reference>/WFA2-lib python tests/golden/make_golden.py
"""
from __future__ import annotations

import gzip
import json
import os
import random
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

WFA2_DIR = Path(os.environ.get("WFA2_SRC", ""))
WFA2_TESTS = WFA2_DIR / "tests"

UTEST_SETS = {
    # name: (penalties (match, mismatch, gap_open, gap_ext), score_only)
    "test.biwfa.affine.alg": ((0, 4, 6, 2), False),
    "test.biwfa.affine.p0.alg": ((0, 1, 2, 1), False),
    "test.biwfa.affine.p1.alg": ((0, 3, 1, 4), False),
    "test.biwfa.affine.p2.alg": ((0, 5, 3, 2), False),
    "test.biwfa.affine.p3.alg": ((-5, 1, 2, 1), False),
    "test.biwfa.affine.p4.alg": ((-2, 3, 1, 4), False),
    "test.biwfa.affine.p5.alg": ((-3, 5, 3, 2), False),
    "test.biwfa.score.affine.alg": ((0, 4, 6, 2), True),
    "test.biwfa.score.affine.p0.alg": ((0, 1, 2, 1), True),
    "test.biwfa.score.affine.p1.alg": ((0, 3, 1, 4), True),
    "test.biwfa.score.affine.p2.alg": ((0, 5, 3, 2), True),
    "test.biwfa.score.affine.p3.alg": ((-5, 1, 2, 1), True),
    "test.biwfa.score.affine.p4.alg": ((-2, 3, 1, 4), True),
    "test.biwfa.score.affine.p5.alg": ((-3, 5, 3, 2), True),
}
LINEAR_SETS = {
    # name: (metric, score_only)
    "test.biwfa.edit.alg": (1, False),
    "test.biwfa.indel.alg": (2, False),
    "test.biwfa.score.edit.alg": (1, True),
    "test.biwfa.score.indel.alg": (2, True),
}
AFFINE2P_SETS = {
    # name: (penalties (match, mismatch, o1, e1, o2, e2), score_only)
    "test.biwfa.affine2p.alg": ((0, 4, 6, 2, 24, 1), False),
    "test.biwfa.score.affine2p.alg": ((0, 4, 6, 2, 24, 1), True),
}


def read_seq_file(path: Path):
    lines = path.read_text().split("\n")
    pairs = []
    for i in range(0, len(lines) - 1, 2):
        if lines[i].startswith(">") and lines[i + 1].startswith("<"):
            pairs.append((lines[i][1:], lines[i + 1][1:]))
    return pairs


def make_utest():
    pairs = read_seq_file(WFA2_TESTS / "wfa.utest.seq")
    sets = {}
    for name, (pen, score_only) in UTEST_SETS.items():
        lines = (WFA2_TESTS / "wfa.utest.check" / name).read_text().split("\n")[: len(pairs)]
        sets[name] = {"penalties": list(pen), "score_only": score_only, "metric": 0, "lines": lines}
    for name, (metric, score_only) in LINEAR_SETS.items():
        lines = (WFA2_TESTS / "wfa.utest.check" / name).read_text().split("\n")[: len(pairs)]
        sets[name] = {"penalties": [0, 0, 0, 0], "score_only": score_only, "metric": metric, "lines": lines}
    for name, (pen, score_only) in AFFINE2P_SETS.items():
        lines = (WFA2_TESTS / "wfa.utest.check" / name).read_text().split("\n")[: len(pairs)]
        sets[name] = {"penalties": list(pen), "score_only": score_only, "metric": 4, "lines": lines}
    out = {"source": "WFA2-lib/tests (v2.3)", "pairs": pairs, "sets": sets}
    with gzip.open(HERE / "wfa2_utest.json.gz", "wt") as f:
        json.dump(out, f)
    print(f"wfa2_utest.json.gz: {len(pairs)} pairs x {len(sets)} sets")


def edge_pairs():
    rnd = random.Random(2024)

    def rs(n, alphabet="ACGT"):
        return "".join(rnd.choice(alphabet) for _ in range(n))

    a150, b150 = rs(150), rs(150)
    a100, b100 = rs(100), rs(100)
    a101, b101 = rs(101), rs(101)
    rep = "ACGTTG" * 60
    return [
        ("", ""), ("", "ACGT"), ("ACGT", ""), ("A", "A"), ("A", "C"), ("A", ""), ("", "G"),
        ("ACGT" * 50, "ACGT" * 50), (a150, b150), (a100, b100), (a101, b101),
        (rs(10), rs(1000)), (rs(1000), rs(10)), (rs(300), rs(300)),
        ("ACGTNNNNACGTACGTNACGT" * 6, "ACGTNNACGTACGTTNACGT" * 6),
        ("acgtACGTacgt" * 12, "ACGTACGTacgt" * 12),
        ("A" * 400, "A" * 380 + "C" * 20), ("A" * 200, "A" * 230),
        (rep, rep[:150] + "TTTT" + rep[150:]), (rep, rep[:100] + rep[130:]),
        ("GATTACA" * 30, "GATCACA" * 30), (rs(5000, "AC"), rs(5000, "AC")),
    ]


def make_ref_cases():
    import biwfa_gpu_pii2025_gb300 as pkg
    from oracle import binding
    if binding.build_ref() is None:
        raise SystemExit("oracle/_ref cannot be built: WFA2-lib sources not found")
    cases = []

    def add(tag, pen, score_only, pairs, metric=0):
        rows = []
        for p, t in pairs:
            st, score, ops, cs = binding.ref_align(p, t, pen, score_only, metric=metric)
            rows.append([p, t, st, score, binding.rle(ops) if ops else "-"])
        cases.append({"tag": tag, "penalties": list(pen), "score_only": score_only, "metric": metric,
                      "pairs": rows})
        print(f"  {tag}: {len(rows)} pairs")

    def gen(workload, n, seed):
        b = pkg.PairBatch.generate(workload, n, seed)
        return [(b.pattern(i).decode(), b.text(i).decode()) for i in range(b.n)]

    add("w1_1kbp_5pct", (0, 4, 6, 2), False, gen(1, 24, 101))
    add("w2_150bp_2pct", (0, 4, 6, 2), False, gen(2, 96, 102))
    add("w3_uneven", (0, 4, 6, 2), False, gen(3, 24, 103))
    add("w4_long_noisy", (0, 4, 6, 2), False, gen(4, 1, 104))
    add("w5_mixture_score_only", (0, 4, 6, 2), True, gen(5, 48, 105))
    edges = edge_pairs()
    for pen in [(0, 4, 6, 2), (0, 1, 2, 1), (0, 3, 1, 4), (0, 5, 3, 2), (-5, 1, 2, 1), (-2, 3, 1, 4)]:
        add(f"edge_{'_'.join(map(str, pen))}", pen, False, edges)
    add("edge_score_only", (0, 4, 6, 2), True, edges)
    # penalties whose score scope exceeds 32 (41 for both: plain, and match < 0 after the
    # transform), run by the scope-64 kernel instantiation
    for pen in ((0, 20, 30, 10), (-4, 8, 12, 6)):
        tag = "affine_scope41_" + "_".join(map(str, pen))
        add(f"{tag}_generated", pen, False, gen(1, 8, 501) + gen(3, 12, 503) + gen(2, 24, 502))
        add(f"{tag}_edges", pen, False, edges)
        add(f"{tag}_score_only", pen, True, gen(5, 24, 505))
    # edit and indel distances: generated pairs, edge cases, and pairs of very different
    # lengths whose wavefronts exceed 1,000 diagonals (edit's exact pruning)
    rnd = random.Random(77)
    far = [("".join(rnd.choice("ACGT") for _ in range(a)), "".join(rnd.choice("ACGT") for _ in range(b)))
           for a, b in ((6000, 1500), (1200, 7000), (4000, 100), (50, 3000))]
    for metric, name in ((1, "edit"), (2, "indel")):
        add(f"{name}_w1_1kbp", (0, 0, 0, 0), False, gen(1, 12, 201), metric)
        add(f"{name}_w3_uneven", (0, 0, 0, 0), False, gen(3, 16, 203), metric)
        add(f"{name}_edges", (0, 0, 0, 0), False, edges + far, metric)
        add(f"{name}_score_only", (0, 0, 0, 0), True, gen(5, 32, 205) + far, metric)
    # gap-linear (penalties match, mismatch, indel, -), including match < 0 (Eizenga)
    for pen in ((0, 4, 2, 0), (0, 1, 1, 0), (-3, 2, 3, 0)):
        tag = "linear_" + "_".join(map(str, pen[:3]))
        add(f"{tag}_generated", pen, False, gen(1, 8, 301) + gen(3, 12, 303), 3)
        add(f"{tag}_edges", pen, False, edges + far[:2], 3)
        add(f"{tag}_score_only", pen, True, gen(5, 24, 305), 3)
    # two-piece gap-affine (match, mismatch, o1, e1, o2, e2), including match < 0 and a second
    # piece cheaper to open than the first
    # (the last two: score scopes of 52 and 42, above the three-component kernels' cap of 32)
    for pen in ((0, 4, 6, 2, 24, 1), (0, 3, 4, 2, 12, 1), (-2, 3, 1, 2, 8, 1), (0, 4, 12, 1, 3, 4),
                (-1, 4, 6, 2, 24, 1), (0, 4, 6, 2, 40, 1)):
        tag = "affine2p_" + "_".join(map(str, pen))
        add(f"{tag}_generated", pen, False, gen(1, 8, 401) + gen(3, 12, 403) + gen(2, 24, 402), 4)
        add(f"{tag}_edges", pen, False, edges + far[:2], 4)
        add(f"{tag}_score_only", pen, True, gen(5, 24, 405), 4)
    with gzip.open(HERE / "wfa2_ref_cases.json.gz", "wt") as f:
        json.dump({"source": "WFA2-lib v2.3 built from the reference sources (oracle/Makefile ref)",
                   "cases": cases}, f)


def make_abi_layout():
    """tests/cpp/abi_layout.c against WFA2-lib's headers -> wfa2_abi_layout.txt."""
    with tempfile.TemporaryDirectory() as td:
        exe = Path(td) / "abi_layout"
        subprocess.run(["gcc", "-std=gnu11", "-DWITH_WFA2", "-I", str(WFA2_DIR), str(HERE.parent / "cpp" / "abi_layout.c"),
                        "-o", str(exe)], check=True)
        out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    (HERE / "wfa2_abi_layout.txt").write_text(out)


if __name__ == "__main__":
    if not (WFA2_TESTS / "wfa.utest.seq").exists():
        sys.exit("set WFA2_SRC to the reference's WFA2-lib folder")
    make_utest()
    make_ref_cases()
    make_abi_layout()
