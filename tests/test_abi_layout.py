"""The drop-in boundary is layout-compatible: wavefront_aligner_attr_t, cigar_t,
wavefront_align_status_t and the public members of wavefront_aligner_t have WFA2-lib's sizes
and field offsets, so object code compiled against WFA2-lib's headers can pass its attribute
structure to this library and read wf_aligner->cigar, ->align_status and ->system."""
import shutil
import subprocess
from pathlib import Path

import pytest

from oracle import binding

ROOT = Path(__file__).resolve().parent.parent
PROBE = ROOT / "tests" / "cpp" / "abi_layout.c"
RECORDED = ROOT / "tests" / "golden" / "wfa2_abi_layout.txt"


def _probe(tmp_path, compiler, *flags) -> str:
    exe = tmp_path / f"abi_{compiler}_{len(flags)}"
    src = PROBE
    if compiler == "g++":
        src = tmp_path / "abi_layout.cpp"
        src.write_text(PROBE.read_text())
    subprocess.run([compiler, *flags, str(src), "-o", str(exe)], check=True)
    return subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_layout_matches_recorded_wfa2_layout(tmp_path):
    ours = _probe(tmp_path, "gcc", "-std=gnu11", "-I", str(ROOT / "include"))
    assert ours == RECORDED.read_text()


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_layout_is_the_same_from_cpp(tmp_path):
    ours = _probe(tmp_path, "g++", "-std=c++17", "-I", str(ROOT / "include"))
    assert ours == RECORDED.read_text()


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_layout_matches_live_wfa2_headers(tmp_path):
    if not (binding.WFA2_SRC / "wavefront" / "wavefront_align.h").exists():
        pytest.skip("WFA2-lib headers not present here")
    ours = _probe(tmp_path, "gcc", "-std=gnu11", "-I", str(ROOT / "include"))
    theirs = _probe(tmp_path, "gcc", "-std=gnu11", "-DWITH_WFA2", "-I", str(binding.WFA2_SRC))
    assert ours == theirs
