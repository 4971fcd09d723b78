"""CPU-side checks of the C ABI library: it loads without a GPU, exports every entry point
declared in include/wfa_gpu.h, and its host-only parts behave."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import biwfa_gpu_pii2025_gb300 as pkg
from biwfa_gpu_pii2025_gb300 import _capi

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "wfa_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    # function declarations only: `name(args);`, not function-pointer members `ret (*name)(args);`
    names = set(re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\((?!\s*\*)[^;{]*\)\s*;", text))
    return sorted(n for n in names if n not in {"if", "while", "for", "return", "sizeof"})


def test_library_loads_and_exports_every_declared_symbol():
    lib = pkg.load_library()
    names = declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), f"{n} declared in wfa_gpu.h but not exported"
        assert n in _capi.SIGNATURES, f"{n} has no ctypes signature"
    # the attribute defaults are exported as data, like WFA2-lib's
    d = _capi.attr_default()
    assert d.affine_penalties.mismatch == 4 and d.affine_penalties.gap_opening == 6
    assert d.memory_mode == _capi.WAVEFRONT_MEMORY_HIGH
    assert d.heuristic.strategy == _capi.WF_HEURISTIC_WFADAPTIVE


def test_strerror_matches_wfa2_messages():
    lib = pkg.load_library()
    assert lib.wavefront_align_strerror(0) == b"[WFA] Alignment completed successfully"
    assert lib.wavefront_align_strerror_short(-100) == b"FAILED.MaxWFASteps"
    assert lib.wavefront_align_strerror_short(-400) == b"FAILED.Unsupported"


def test_generator_is_deterministic_and_matches_spec():
    a = pkg.PairBatch.generate(1, 50, seed=11)
    b = pkg.PairBatch.generate(1, 50, seed=11)
    c = pkg.PairBatch.generate(1, 50, seed=12)
    assert np.array_equal(a.seq, b.seq) and not np.array_equal(a.seq, c.seq)
    assert (a.plen == 1000).all()
    assert set(np.unique(a.seq[: a.plen[0]]).tolist()) <= set(b"ACGT")
    w2 = pkg.PairBatch.generate(2, 200, seed=3)
    assert (w2.plen == 150).all() and (np.abs(w2.tlen - 150) <= 3).all()
    w3 = pkg.PairBatch.generate(3, 400, seed=3)
    assert w3.plen.min() >= 100 and w3.plen.max() <= 10000
    # log-uniform: about half of the lengths below sqrt(100*10000) = 1000
    frac = float((w3.plen < 1000).mean())
    assert 0.4 < frac < 0.6
    w5 = pkg.PairBatch.generate(5, 300, seed=3)
    kinds = {1000: 0, 150: 0}
    for L in w5.plen:
        if int(L) in kinds:
            kinds[int(L)] += 1
    assert kinds[1000] > 60 and kinds[150] > 60
    # fixed checksum: the generator must produce the same bytes on every platform
    assert int(a.seq.astype(np.uint64).sum()) == int(b.seq.astype(np.uint64).sum())


def test_generator_checksum_pinned():
    b = pkg.PairBatch.generate(3, 20, seed=2024)
    h = int(np.frombuffer(b.seq.tobytes(), np.uint8).astype(np.uint64).dot(
        np.arange(1, b.seq.size + 1, dtype=np.uint64) % np.uint64(1000003)))
    assert (int(b.seq.size), h) == GEN_PIN, (int(b.seq.size), h)


GEN_PIN = (98556, 348394859071)  # same bytes on x86-64 and aarch64


def test_runs_to_cigar_format():
    runs = np.array([(14 << 4) | 7, (1 << 4) | 1, (86 << 4) | 7], np.uint32)
    assert pkg.runs_to_cigar(runs) == "14M1I86M"
    assert pkg.runs_to_ops(runs) == "M" * 14 + "I" + "M" * 86


def test_context_create_without_gpu_returns_null_or_works():
    lib = pkg.load_library()
    ctx = lib.wfg_context_create(0)
    if ctx:
        lib.wfg_context_destroy(ctx)
    assert lib.wfg_context_create(99) is None


def _cigar_of(ops: str) -> "_capi.Cigar":
    buf = C.create_string_buffer(ops.encode(), len(ops) + 1)
    cg = _capi.Cigar()
    cg.operations = C.cast(buf, C.POINTER(C.c_char))
    cg.max_operations = len(ops) + 1
    cg.begin_offset, cg.end_offset = 0, len(ops)
    cg._buf = buf  # keep the buffer alive with the struct
    return cg


@pytest.mark.parametrize("metric,pen", [(0, (0, 4, 6, 2)), (0, (-3, 5, 3, 2)), (1, (0, 0, 0, 0)), (2, (0, 0, 0, 0)),
                                        (3, (0, 4, 2, 0)), (4, (0, 4, 6, 2, 24, 1)), (4, (-2, 3, 1, 2, 8, 1))])
def test_cigar_scorers_match_oracle_rescoring(metric, pen):
    """cigar_score_gap_affine / _edit / _gap_linear / _gap_affine2p (host functions of the C
    ABI) give the score align_benchmark prints for the oracle's CIGARs."""
    from oracle import binding
    lib = pkg.load_library()
    rng = np.random.default_rng(metric * 10 + len(pen))
    for _ in range(40):
        n = int(rng.integers(1, 300))
        p = bytes(rng.choice(list(b"ACGT"), n).astype(np.uint8))
        t = bytearray(p)
        for _ in range(int(rng.integers(0, 25))):
            pos = int(rng.integers(0, max(len(t), 1)))
            r = rng.random()
            if r < 0.4 and t:
                t[min(pos, len(t) - 1)] = int(rng.choice(list(b"ACGT")))
            elif r < 0.7:
                t[pos:pos] = bytes(rng.choice(list(b"ACGT"), int(rng.integers(1, 30))).astype(np.uint8))
            else:
                del t[pos:pos + int(rng.integers(1, 30))]
        st, score, ops, _ = binding.oracle_align(p, bytes(t), pen, metric=metric)
        if not ops:
            continue
        cg = _cigar_of(ops)
        if metric == 0:
            got = lib.cigar_score_gap_affine(C.byref(cg), C.byref(_capi.AffinePenalties(*pen)))
        elif metric in (1, 2):
            got = lib.cigar_score_edit(C.byref(cg))
        elif metric == 3:
            got = lib.cigar_score_gap_linear(C.byref(cg), C.byref(_capi.LinearPenalties(*pen[:3])))
        else:
            got = lib.cigar_score_gap_affine2p(C.byref(cg), C.byref(_capi.Affine2pPenalties(*pen)))
        assert got == score, (metric, pen, ops)


def _refusal_status(mutate) -> int:
    """wavefront_align's status for a default BiWFA configuration changed by `mutate`; an
    unsupported configuration answers before any device is touched."""
    lib = pkg.load_library()
    attr = _capi.AlignerAttr.from_buffer_copy(_capi.attr_default())
    attr.memory_mode = _capi.WAVEFRONT_MEMORY_ULTRALOW
    attr.heuristic.strategy = _capi.WF_HEURISTIC_NONE
    mutate(attr)
    wf = lib.wavefront_aligner_new(C.byref(attr))
    assert wf
    try:
        return lib.wavefront_align(wf, b"ACGTACGT", 8, b"ACGAACGT", 8)
    finally:
        lib.wavefront_aligner_delete(wf)


@pytest.mark.parametrize("case", ["affine_mismatch0", "affine_match_pos", "affine2p_e2_0", "affine2p_o2_neg",
                                  "linear_indel0", "heuristic", "memory_high", "endsfree", "metric_unknown"])
def test_wfa2_api_refuses_bad_configurations_without_a_gpu(case):
    def mutate(a):
        if case == "affine_mismatch0":
            a.affine_penalties = _capi.AffinePenalties(0, 0, 6, 2)
        elif case == "affine_match_pos":
            a.affine_penalties = _capi.AffinePenalties(1, 4, 6, 2)
        elif case == "affine2p_e2_0":
            a.distance_metric = _capi.GAP_AFFINE_2P
            a.affine2p_penalties = _capi.Affine2pPenalties(0, 4, 6, 2, 24, 0)
        elif case == "affine2p_o2_neg":
            a.distance_metric = _capi.GAP_AFFINE_2P
            a.affine2p_penalties = _capi.Affine2pPenalties(0, 4, 6, 2, -1, 1)
        elif case == "linear_indel0":
            a.distance_metric = _capi.GAP_LINEAR
            a.linear_penalties = _capi.LinearPenalties(0, 4, 0)
        elif case == "heuristic":
            a.heuristic.strategy = _capi.WF_HEURISTIC_WFADAPTIVE
        elif case == "memory_high":
            a.memory_mode = _capi.WAVEFRONT_MEMORY_HIGH
        elif case == "endsfree":
            a.alignment_form.span = _capi.ALIGNMENT_ENDSFREE
            a.alignment_form.text_end_free = 2
        else:
            a.distance_metric = 9
    assert _refusal_status(mutate) == _capi.WF_STATUS_UNSUPPORTED


@pytest.mark.parametrize("distance", ["GAP_AFFINE", "GAP_AFFINE_2P", "GAP_LINEAR", "EDIT", "INDEL"])
def test_python_wavefront_aligner_builds_every_distance(distance):
    """The Python mirror of WFA2-lib's aligner accepts every distance; without a GPU a valid
    configuration reaches the device check, an invalid one is refused first."""
    al = pkg.WavefrontAligner(distance=getattr(_capi, distance))
    try:
        st = al.align("ACGTACGT", "ACGAACGT")
        assert st in (0, _capi.WF_STATUS_DEVICE_ERROR)
    finally:
        al.close()
    bad = pkg.WavefrontAligner(distance=getattr(_capi, distance), mismatch=0)
    try:
        st = bad.align("ACGT", "ACGA")
        if distance in ("EDIT", "INDEL"):  # they ignore the penalties
            assert st in (0, _capi.WF_STATUS_DEVICE_ERROR)
        else:
            assert st == _capi.WF_STATUS_UNSUPPORTED
    finally:
        bad.close()
