"""ctypes access to the oracle builds (test infrastructure, never the product).

  * libbiwfa_oracle.so  — the C restatement in biwfa_oracle.c (builds anywhere with gcc);
  * libwfa2_ref.so      — the real WFA2-lib v2.3 compiled from its unmodified sources (the
                          copy stage_wfa2.py puts in the git-ignored baseline/_ref/, or
                          the folder WFA2_SRC names; see Makefile).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "_build" / "libbiwfa_oracle.so"
REF_SO = HERE / "_ref" / "libwfa2_ref.so"
WFA2_SRC = Path(os.environ.get("WFA2_SRC", str(HERE.parent / "baseline" / "_ref" / "WFA2-lib")))


class OrcResult(C.Structure):
    _fields_ = [("status", C.c_int), ("score", C.c_int), ("cigar_score", C.c_int), ("ops_len", C.c_int),
                ("n_cells", C.c_int64), ("n_ext", C.c_int64), ("n_steps", C.c_int64),
                ("max_leaf_score", C.c_int), ("max_depth", C.c_int)]


def build_oracle() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "oracle"], check=True)
    return ORACLE_SO


def build_ref() -> Path | None:
    """Builds the WFA2-lib reference library when its sources are present; else None."""
    if not (WFA2_SRC / "wavefront" / "wavefront_align.c").exists():
        return REF_SO if REF_SO.exists() else None
    subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"WFA2={WFA2_SRC}"], check=True)
    return REF_SO


_orc = None
_ref = None

# distances (oracle/biwfa_oracle.h ORC_METRIC_*)
METRIC_AFFINE, METRIC_EDIT, METRIC_INDEL, METRIC_LINEAR, METRIC_AFFINE2P = 0, 1, 2, 3, 4


def pen6(penalties) -> tuple:
    """(match, mismatch, o1, e1[, o2, e2]) -> the six-entry set; o2/e2 default to (0, 1)."""
    p = tuple(int(v) for v in penalties)
    return p + (0, 1)[len(p) - 4:] if len(p) < 6 else p[:6]


def oracle_lib() -> C.CDLL:
    global _orc
    if _orc is None:
        if not ORACLE_SO.exists():
            build_oracle()
        lib = C.CDLL(str(ORACLE_SO))
        lib.orc_biwfa_align.restype = C.c_int
        lib.orc_biwfa_align.argtypes = [C.c_char_p, C.c_int, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.c_int, C.c_int, C.c_char_p, C.c_int, C.POINTER(OrcResult)]
        lib.orc_biwfa_align_batch.restype = C.c_double
        lib.orc_wfa_align.restype = C.c_int
        lib.orc_wfa_align.argtypes = [C.c_int] + lib.orc_biwfa_align.argtypes
        lib.orc_wfa_align_batch.restype = C.c_double
        lib.orc_wfa_align_pen.restype = C.c_int
        lib.orc_wfa_align_batch_pen.restype = C.c_double
        _orc = lib
    return _orc


def ref_lib() -> C.CDLL | None:
    global _ref
    if _ref is None:
        if not REF_SO.exists():
            return None
        lib = C.CDLL(str(REF_SO))
        lib.ref_biwfa_align.restype = C.c_int
        lib.ref_wfa_align_linear.restype = C.c_int
        lib.ref_wfa_align_affine2p.restype = C.c_int
        _ref = lib
    return _ref


def _b(x) -> bytes:
    return x.encode() if isinstance(x, str) else bytes(x)


def rle(ops: str) -> str:
    out, i = [], 0
    while i < len(ops):
        j = i
        while j < len(ops) and ops[j] == ops[i]:
            j += 1
        out.append(f"{j - i}{ops[i]}")
        i = j
    return "".join(out)


def oracle_align(pattern, text, penalties=(0, 4, 6, 2), score_only=False, metric=METRIC_AFFINE):
    """Returns (status, score, ops, OrcResult). score follows align_benchmark's printing:
    the rescored CIGAR (full mode, -1 when the CIGAR is empty) or cigar->score (score-only);
    for the edit and indel distances the rescoring counts the edits."""
    p, t = _b(pattern), _b(text)
    cap = len(p) + len(t) + 8
    buf = C.create_string_buffer(cap)
    r = OrcResult()
    pen = (C.c_int * 6)(*pen6(penalties))
    st = oracle_lib().orc_wfa_align_pen(C.c_int(metric), p, C.c_int(len(p)), t, C.c_int(len(t)), pen,
                                        C.c_int(1 if score_only else 0), buf, C.c_int(cap), C.byref(r))
    return st, r.score, buf.raw[:r.ops_len].decode(), r


def ref_align(pattern, text, penalties=(0, 4, 6, 2), score_only=False, metric=METRIC_AFFINE):
    """The real WFA2-lib. Returns (status, printed score, ops, cigar->score) or None if unavailable."""
    lib = ref_lib()
    if lib is None:
        return None
    m, x, o, e = penalties[:4]
    p, t = _b(pattern), _b(text)
    cap = len(p) + len(t) + 8
    buf = C.create_string_buffer(cap)
    cs, rs, ol = C.c_int(), C.c_int(), C.c_int()
    if metric == METRIC_AFFINE:
        st = lib.ref_biwfa_align(p, len(p), t, len(t), m, x, o, e, 1 if score_only else 0, C.byref(cs),
                                 C.byref(rs), buf, cap, C.byref(ol))
    elif metric == METRIC_AFFINE2P:
        pen = (C.c_int * 6)(*pen6(penalties))
        st = lib.ref_wfa_align_affine2p(p, C.c_int(len(p)), t, C.c_int(len(t)), pen, C.c_int(1 if score_only else 0),
                                        C.byref(cs), C.byref(rs), buf, C.c_int(cap), C.byref(ol))
    elif metric == METRIC_LINEAR:  # penalties (match, mismatch, indel, -)
        st = lib.ref_wfa_align_gap_linear(p, len(p), t, len(t), m, x, o, 1 if score_only else 0, C.byref(cs),
                                          C.byref(rs), buf, cap, C.byref(ol))
    else:
        st = lib.ref_wfa_align_linear(metric, p, len(p), t, len(t), 1 if score_only else 0, C.byref(cs),
                                      C.byref(rs), buf, cap, C.byref(ol))
    ops = buf.raw[:ol.value].decode()
    score = cs.value if score_only else (rs.value if ops else -1)
    return st, score, ops, cs.value


def oracle_batch_time(seq: np.ndarray, p_off, plen, t_off, tlen, penalties=(0, 4, 6, 2), score_only=False,
                      threads: int = 1, return_ops: bool = False, metric: int = METRIC_AFFINE):
    """Aligns a batch with the oracle on `threads` POSIX threads; returns (seconds, scores, status[, ops])."""
    lib = oracle_lib()
    n = int(len(plen))
    p_off = np.ascontiguousarray(p_off, np.int64); t_off = np.ascontiguousarray(t_off, np.int64)
    plen = np.ascontiguousarray(plen, np.int32); tlen = np.ascontiguousarray(tlen, np.int32)
    ops_off = np.zeros(n, np.int64)
    if n > 1:
        ops_off[1:] = np.cumsum((plen.astype(np.int64) + tlen + 1))[:-1]
    ops = np.empty(int((plen.astype(np.int64) + tlen + 1).sum()) + 1, np.uint8)
    scores = np.empty(n, np.int32); status = np.empty(n, np.int32); ops_len = np.empty(n, np.int32)
    i64p, ip = C.POINTER(C.c_int64), C.POINTER(C.c_int)
    pen = (C.c_int * 6)(*pen6(penalties))
    secs = lib.orc_wfa_align_batch_pen(
        C.c_int(metric), C.c_int(n), seq.ctypes.data_as(C.c_char_p), p_off.ctypes.data_as(i64p), plen.ctypes.data_as(ip),
        seq.ctypes.data_as(C.c_char_p), t_off.ctypes.data_as(i64p), tlen.ctypes.data_as(ip), pen,
        C.c_int(1 if score_only else 0), ops.ctypes.data_as(C.c_char_p), ops_off.ctypes.data_as(i64p),
        scores.ctypes.data_as(ip), status.ctypes.data_as(ip), ops_len.ctypes.data_as(ip), C.c_int(threads))
    if return_ops == "raw":
        return float(secs), scores, status, (ops, ops_off, ops_len)
    if return_ops:
        cig = [ops[ops_off[i]:ops_off[i] + ops_len[i]].tobytes().decode() for i in range(n)]
        return float(secs), scores, status, cig
    return float(secs), scores, status


def ref_batch_time(seq: np.ndarray, p_off, plen, t_off, tlen, penalties=(0, 4, 6, 2), threads: int = 1,
                   return_ops=False):
    """The real WFA2-lib (gap-affine BiWFA, full CIGAR) on `threads` POSIX threads, one aligner
    per thread; returns (seconds, printed scores, status[, raw ops]) like oracle_batch_time, or
    None when the library is not built here."""
    lib = ref_lib()
    if lib is None:
        return None
    n = int(len(plen))
    p_off = np.ascontiguousarray(p_off, np.int64); t_off = np.ascontiguousarray(t_off, np.int64)
    plen = np.ascontiguousarray(plen, np.int32); tlen = np.ascontiguousarray(tlen, np.int32)
    scores = np.empty(n, np.int32); status = np.empty(n, np.int32); ops_len = np.zeros(n, np.int32)
    ops, ops_off = None, None
    if return_ops:
        ops_off = np.zeros(n, np.int64)
        if n > 1:
            ops_off[1:] = np.cumsum((plen.astype(np.int64) + tlen + 1))[:-1]
        ops = np.empty(int((plen.astype(np.int64) + tlen + 1).sum()) + 1, np.uint8)
    i64p, ip = C.POINTER(C.c_int64), C.POINTER(C.c_int)
    pen = (C.c_int * 4)(*[int(v) for v in penalties[:4]])
    fn = lib.ref_biwfa_align_batch_mt
    fn.restype = C.c_double
    secs = fn(C.c_int(n), seq.ctypes.data_as(C.c_char_p), p_off.ctypes.data_as(i64p), plen.ctypes.data_as(ip),
              t_off.ctypes.data_as(i64p), tlen.ctypes.data_as(ip), pen, C.c_int(threads),
              ops.ctypes.data_as(C.c_char_p) if ops is not None else None,
              ops_off.ctypes.data_as(i64p) if ops_off is not None else None,
              scores.ctypes.data_as(ip), status.ctypes.data_as(ip), ops_len.ctypes.data_as(ip))
    if return_ops:
        return float(secs), scores, status, (ops, ops_off, ops_len)
    return float(secs), scores, status


def compare_runs(raw_ops, runs: np.ndarray, run_off: np.ndarray, run_len: np.ndarray) -> np.ndarray:
    """Per-pair flag (1 = differs) of the oracle's raw operations (oracle_batch_time(...,
    return_ops="raw")) against run-length lists (uint32 len << 4 | SAM op, the GPU's form)."""
    ops, ops_off, ops_len = raw_ops
    n = int(ops_len.shape[0])
    lib = oracle_lib()
    lib.orc_compare_runs.restype = C.c_int64
    runs = np.ascontiguousarray(runs, np.uint32)
    run_off = np.ascontiguousarray(run_off, np.int64)
    run_len = np.ascontiguousarray(run_len, np.int32)
    ops_len = np.ascontiguousarray(ops_len, np.int32)
    bad = np.zeros(n, np.uint8)
    i64p, ip = C.POINTER(C.c_int64), C.POINTER(C.c_int)
    lib.orc_compare_runs(C.c_int(n), ops.ctypes.data_as(C.c_char_p), ops_off.ctypes.data_as(i64p),
                         ops_len.ctypes.data_as(ip), runs.ctypes.data_as(C.POINTER(C.c_uint32)),
                         run_off.ctypes.data_as(i64p), run_len.ctypes.data_as(ip),
                         bad.ctypes.data_as(C.POINTER(C.c_uint8)))
    return bad


def check_batch(seq, p_off, plen, t_off, tlen, scores, status, runs, run_off, run_len, penalties=(0, 4, 6, 2),
                metric: int = METRIC_AFFINE, threads: int | None = None, chunk: int = 100_000,
                idx: np.ndarray | None = None, against: str = "oracle") -> dict:
    """Every pair (or the pairs idx) of a batch aligned by the oracle (against="wfa2": the real
    WFA2-lib, gap-affine only) on `threads` threads and compared bit-exactly with given results:
    status, score (full-CIGAR mode) and the whole operation string. Returns {"checked",
    "mismatches", "first_bad", "oracle_s"}."""
    threads = threads or os.cpu_count() or 1
    n_all = int(len(plen))
    idx = np.arange(n_all) if idx is None else np.asarray(idx, np.int64)
    bad_all, secs_all = [], 0.0
    for c0 in range(0, len(idx), chunk):
        sel = idx[c0:c0 + chunk]
        if against == "wfa2":
            secs, sc, st, raw = ref_batch_time(seq, np.asarray(p_off)[sel], np.asarray(plen)[sel],
                                               np.asarray(t_off)[sel], np.asarray(tlen)[sel], penalties,
                                               threads=threads, return_ops=True)
        else:
            secs, sc, st, raw = oracle_batch_time(seq, np.asarray(p_off)[sel], np.asarray(plen)[sel],
                                                  np.asarray(t_off)[sel], np.asarray(tlen)[sel], penalties,
                                                  threads=threads, return_ops="raw", metric=metric)
        secs_all += secs
        flag = compare_runs(raw, runs, np.asarray(run_off)[sel], np.asarray(run_len)[sel]).astype(bool)
        # align_benchmark prints -1 for an empty CIGAR; the GPU reports the score 0 there
        exp_scores = np.where(raw[2] > 0, sc, 0)
        flag |= (np.asarray(status)[sel] != st) | (np.asarray(scores)[sel] != exp_scores)
        bad_all.append(sel[flag])
    bad = np.concatenate(bad_all) if bad_all else np.zeros(0, np.int64)
    return {"checked": int(len(idx)), "mismatches": int(bad.shape[0]), "first_bad": [int(i) for i in bad[:5]],
            "oracle_s": secs_all}
