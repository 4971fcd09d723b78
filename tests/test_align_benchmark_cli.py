"""The align_benchmark-compatible CLI (biwfa_gpu_pii2025_gb300/align_benchmark, built from
csrc/align_benchmark.cpp): option handling on CPU; on the GPU its output files reproduce
WFA2-lib's own unit-test outputs line for line."""
import subprocess

import pytest

from biwfa_gpu_pii2025_gb300 import build as B
from golden_data import utest
from oracle import binding


def _cli():
    if not B.CLI.exists():
        pytest.skip("align_benchmark not built")
    return str(B.CLI)


def _write_seq(path, pairs):
    with open(path, "w") as f:
        for p, t in pairs:
            f.write(f">{p}\n<{t}\n")


def test_cli_options():
    exe = _cli()
    assert subprocess.run([exe, "--help"], capture_output=True).returncode == 0
    for bad in (["-i", "x.seq", "--wfa-memory", "high"], ["-i", "x.seq", "--wfa-heuristic", "wfa-adaptive"],
                ["-i", "x.seq", "-a", "gap-affine2p-dp"], ["-i", "x.seq", "--affine2p-penalties", "0,4,6,2"],
                ["-i", "x.seq", "--wfa-span", "extension"],
                ["-i", "x.seq", "--bogus"], ["-g", "0,4,6"]):
        r = subprocess.run([exe, *bad], capture_output=True, text=True)
        assert r.returncode == 1 and r.stderr, bad


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["test.biwfa.affine.alg", "test.biwfa.score.affine.alg",
                                  "test.biwfa.affine.p1.alg", "test.biwfa.affine.p4.alg",
                                  "test.biwfa.edit.alg", "test.biwfa.indel.alg", "test.biwfa.score.edit.alg",
                                  "test.biwfa.affine2p.alg", "test.biwfa.score.affine2p.alg"])
def test_cli_reproduces_wfa2_utest_outputs(tmp_path, name):
    exe = _cli()
    data = utest()
    s = data["sets"][name]
    seq = tmp_path / "in.seq"
    out = tmp_path / "out.alg"
    _write_seq(seq, data["pairs"])
    algo = {0: "gap-affine-wfa", 1: "edit-wfa", 2: "indel-wfa", 4: "gap-affine2p-wfa"}[s.get("metric", 0)]
    args = [exe, "-a", algo, "-i", str(seq), "-o", str(out), "--wfa-memory", "ultralow",
            "--wfa-heuristic", "none", "--batch-size", "97", "-q"]
    if algo == "gap-affine-wfa":
        args += ["-g", ",".join(map(str, s["penalties"]))]
    if algo == "gap-affine2p-wfa":
        args += ["--affine2p-penalties", ",".join(map(str, s["penalties"]))]
    if s["score_only"]:
        args.append("--wfa-score-only")
    subprocess.run(args, check=True)
    lines = out.read_text().splitlines()
    assert lines == s["lines"]


@pytest.mark.gpu
def test_cli_output_full(tmp_path):
    exe = _cli()
    pairs = [("ACGTACGTAC", "ACGTTACGTAC"), ("", "ACG"), ("GATTACA", "GATTACA")]
    seq, out = tmp_path / "in.seq", tmp_path / "out.alg"
    _write_seq(seq, pairs)
    subprocess.run([exe, "-i", str(seq), "--output-full", str(out), "--wfa-memory", "ultralow", "--wfa-heuristic",
                    "none", "-q"], check=True)
    rows = [line.split("\t") for line in out.read_text().splitlines()]
    _, score, ops, _ = binding.oracle_align(b"ACGTACGTAC", b"ACGTTACGTAC")
    rle = "".join(f"{len(r)}{r[0]}" for r in __import__("re").findall(r"(M+|X+|I+|D+)", ops))
    assert rows[0] == ["10", "11", str(score), "ACGTACGTAC", "ACGTTACGTAC", rle] and score == -8
    assert rows[1] == ["0", "3", "-12", "", "ACG", "3I"]
    assert rows[2] == ["7", "7", "0", "GATTACA", "GATTACA", "7M"]


@pytest.mark.gpu
def test_cli_gap_linear_matches_oracle(tmp_path):
    """gap-linear-wfa with --linear-penalties: every line equals the oracle's (the real WFA2-lib
    pins the oracle for gap-linear in tests/test_oracle.py)."""
    exe = _cli()
    pairs = utest()["pairs"][:150]
    seq, out = tmp_path / "in.seq", tmp_path / "out.alg"
    _write_seq(seq, pairs)
    subprocess.run([exe, "-a", "gap-linear-wfa", "-p", "0,4,2", "-i", str(seq), "-o", str(out), "--wfa-memory",
                    "ultralow", "--wfa-heuristic", "none", "-q"], check=True)
    lines = out.read_text().splitlines()
    for i, (p, t) in enumerate(pairs):
        st, score, ops, _ = binding.oracle_align(p, t, (0, 4, 2, 0), metric=binding.METRIC_LINEAR)
        assert lines[i] == (f"{score}\t{binding.rle(ops)}" if ops else "-1\t-"), i
