"""The C++ binding (include/WFAligner.hpp, WFA2-lib's wfa::WFAligner surface over the C ABI):
compiled with g++ against libbiwfa_gb300.so and driven by tests/cpp/wfaligner_pairs.cpp."""
import shutil
import subprocess
from pathlib import Path

import pytest

import biwfa_gpu_pii2025_gb300 as pkg
from biwfa_gpu_pii2025_gb300 import _capi
from golden_data import utest
from oracle import binding

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "wfaligner_pairs.cpp"


def _build(tmp_path) -> Path:
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    lib_dir = _capi.LIB_PATH.parent
    exe = tmp_path / "wfaligner_pairs"
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(SRC),
                    f"-L{lib_dir}", "-lbiwfa_gb300", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    return exe


def _sam(ops: str) -> str:
    out, i = [], 0
    while i < len(ops):
        j = i
        while j < len(ops) and ops[j] == ops[i]:
            j += 1
        out.append(f"{j - i}{'=' if ops[i] == 'M' else ops[i]}")
        i = j
    return "".join(out)


def test_cpp_binding_reports_unsupported_configurations(tmp_path):
    _capi.load()
    exe = _build(tmp_path)
    out = subprocess.run([str(exe), "--config-only"], capture_output=True, text=True, check=True).stdout
    rows = dict(line.split("\t", 1) for line in out.strip().splitlines())
    unsupported = str(_capi.WF_STATUS_UNSUPPORTED)
    # MemoryHigh (the binding's default, for gap-affine and two-piece affine), WFA2-lib's
    # default heuristic, an explicit heuristic and ends-free all refuse with a status instead
    # of exiting
    for key in ("default_heuristic", "high", "affine2p", "heuristic", "endsfree"):
        assert rows[key] == unsupported, (key, rows[key])
    assert rows["no_device"] in ("0", str(_capi.WF_STATUS_DEVICE_ERROR))
    assert "not supported" in rows["status_text"]
    assert rows["cigar_after_refusal"] == "[]"


@pytest.mark.gpu
@pytest.mark.parametrize("two_piece", [False, True])
def test_cpp_binding_matches_oracle(tmp_path, two_piece):
    exe = _build(tmp_path)
    pairs = [(p, t) for p, t in utest()["pairs"][:120]]
    b = pkg.PairBatch.generate(1, 40, seed=8)
    pairs += [(b.pattern(i).decode(), b.text(i).decode()) for i in range(b.n)]
    pairs += [("", ""), ("ACGT", ""), ("", "ACGT")]
    stdin = "".join(f"{p}\t{t}\n" for p, t in pairs)
    args = [str(exe)] + (["--affine2p"] if two_piece else [])
    pen, metric = ((0, 4, 6, 2, 24, 1), binding.METRIC_AFFINE2P) if two_piece else ((0, 4, 6, 2), binding.METRIC_AFFINE)
    out = subprocess.run(args, input=stdin, capture_output=True, text=True, check=True).stdout.splitlines()
    single = [line.split("\t") for line in out if not line.startswith("batch\t")]
    batch = [line.split("\t")[1:] for line in out if line.startswith("batch\t")]
    assert len(single) == len(pairs) and len(batch) == len(pairs)
    for i, (p, t) in enumerate(pairs):
        st, score, ops, _ = binding.oracle_align(p.encode(), t.encode(), pen, metric=metric)
        assert int(single[i][0]) == 0 and int(batch[i][0]) == 0, i
        if ops:
            assert int(single[i][1]) == score and int(batch[i][1]) == score, i
        assert single[i][3] == ops, i
        assert single[i][2] == _sam(ops) and batch[i][2] == _sam(ops), i
