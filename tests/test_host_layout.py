"""Host-side sizing and ABI facts (no GPU): ring buffer counts per distance, the five-component
arena layout, and the wfg_config_t layout against the ctypes mirror. Compiled with g++ from
tests/cpp/layout_check.cpp against include/ and the package's internal header."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

from biwfa_gpu_pii2025_gb300 import _capi

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def facts(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("layout") / "layout_check"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", str(ROOT / "include"), "-I",
                    str(ROOT / "biwfa_gpu_pii2025_gb300" / "csrc"), str(ROOT / "tests" / "cpp" / "layout_check.cpp"),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    return {k: v.split("\t") for k, v in (line.split("\t", 1) for line in out.strip().splitlines())}


def test_ring_buffer_counts(facts):
    # ceil(scope / g): scores that hold a wavefront are multiples of g (the gcd of the step costs)
    assert int(facts["ring_buffers_4_6_2"][0]) == 5          # scope 9, g 2
    assert int(facts["ring_buffers_1_2_1"][0]) == 4          # scope 4, g 1
    assert int(facts["ring_buffers_linear_4_2"][0]) == 3     # gap-linear: scope 5, g 2
    assert int(facts["ring_buffers_2p_4_6_2_24_1"][0]) == 26  # scope 26, g 1
    assert int(facts["ring_buffers_2p_4_6_2_24_2"][0]) == 14  # scope 27, g 2
    assert int(facts["ring_buffers_2p_4_12_4_24_4"][0]) == 8  # scope 29, g 4


def test_five_component_arena(facts):
    r3, r5 = int(facts["arena3_ring"][0]), int(facts["arena5_ring"][0])
    assert r3 == 2 * 5 * 3 * 4096 * 4 and r5 == 2 * 5 * 5 * 4096 * 4
    align = lambda v: (v + 255) // 256 * 256  # every region starts on a 256-byte boundary
    assert int(facts["arena5_ldesc"][0]) == align(529 * 5 * 16)
    assert int(facts["arena3_rdesc2"][0]) == 0
    max2p = int(facts["max_scope"][1])
    assert int(facts["arena5_rdesc2"][0]) == align(2 * max2p * 2 * 8)
    assert int(facts["arena5_end"][0]) <= int(facts["arena5_total"][0])
    assert int(facts["arena3_total"][0]) < int(facts["arena5_total"][0])


def test_config_abi_matches_ctypes(facts):
    assert int(facts["sizeof_wfg_config_t"][0]) == C.sizeof(_capi.Config)
    assert int(facts["offsetof_metric"][0]) == _capi.Config.metric.offset
    assert int(facts["offsetof_gap_opening2"][0]) == _capi.Config.gap_opening2.offset
    assert int(facts["offsetof_gap_extension2"][0]) == _capi.Config.gap_extension2.offset
