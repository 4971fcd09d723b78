"""ctypes binding of include/wfa_gpu.h (libbiwfa_gb300.so).

The library is the product; this module only declares its C signatures. Loading fails
loudly when the library has not been built (there is no Python or CPU fallback).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libbiwfa_gb300.so"

# Status codes (WFA2-lib wavefront/wfa.h:46-55 plus this library's two additions).
WF_STATUS_ALG_COMPLETED = 0
WF_STATUS_ALG_PARTIAL = 1
WF_STATUS_MAX_STEPS_REACHED = -100
WF_STATUS_OOM = -200
WF_STATUS_UNATTAINABLE = -300
WF_STATUS_UNSUPPORTED = -400
WF_STATUS_DEVICE_ERROR = -500

# enums (distance_metric_t of wavefront/wavefront_penalties.h)
INDEL, EDIT, GAP_LINEAR, GAP_AFFINE, GAP_AFFINE_2P = 0, 1, 2, 3, 4
COMPUTE_SCORE, COMPUTE_ALIGNMENT = 0, 1
ALIGNMENT_END2END, ALIGNMENT_ENDSFREE = 0, 1
WF_HEURISTIC_NONE, WF_HEURISTIC_WFADAPTIVE = 0, 4
WAVEFRONT_MEMORY_HIGH, WAVEFRONT_MEMORY_ULTRALOW = 0, 3
SCHED_PLAIN, SCHED_LEARNED, SCHED_GIVEN, SCHED_SORTED = 0, 1, 2, 3
METRIC_GAP_AFFINE, METRIC_EDIT, METRIC_INDEL, METRIC_GAP_LINEAR, METRIC_GAP_AFFINE_2P = 0, 1, 2, 3, 4

# SAM op codes of the output runs
OP_INS, OP_DEL, OP_EQ, OP_X = 1, 2, 7, 8
OP_CHAR = {OP_EQ: "M", OP_X: "X", OP_INS: "I", OP_DEL: "D"}


class AlignmentForm(C.Structure):
    _fields_ = [("span", C.c_int), ("extension", C.c_bool), ("pattern_begin_free", C.c_int),
                ("pattern_end_free", C.c_int), ("text_begin_free", C.c_int), ("text_end_free", C.c_int)]


class LinearPenalties(C.Structure):
    _fields_ = [("match", C.c_int), ("mismatch", C.c_int), ("indel", C.c_int)]


class AffinePenalties(C.Structure):
    _fields_ = [("match", C.c_int), ("mismatch", C.c_int), ("gap_opening", C.c_int), ("gap_extension", C.c_int)]


class Affine2pPenalties(C.Structure):
    _fields_ = [("match", C.c_int), ("mismatch", C.c_int), ("gap_opening1", C.c_int), ("gap_extension1", C.c_int),
                ("gap_opening2", C.c_int), ("gap_extension2", C.c_int)]


class Heuristic(C.Structure):
    _fields_ = [("strategy", C.c_int), ("steps_between_cutoffs", C.c_int), ("min_k", C.c_int), ("max_k", C.c_int),
                ("min_wavefront_length", C.c_int), ("max_distance_threshold", C.c_int), ("xdrop", C.c_int),
                ("zdrop", C.c_int), ("steps_wait", C.c_int), ("max_sw_score", C.c_int), ("max_wf_score", C.c_int),
                ("max_sw_score_offset", C.c_int), ("max_sw_score_k", C.c_int)]


class PlotAttr(C.Structure):
    _fields_ = [("enabled", C.c_bool), ("resolution_points", C.c_int), ("align_level", C.c_int)]


class Timer(C.Structure):  # profiler_timer_t: struct timespec, profiler_counter_t, accumulated
    _fields_ = [("tv_sec", C.c_int64), ("tv_nsec", C.c_long), ("counter", C.c_uint64 * 4), ("moments", C.c_double * 4),
                ("accumulated", C.c_uint64)]


class System(C.Structure):
    _fields_ = [("max_alignment_steps", C.c_int), ("probe_interval_global", C.c_int),
                ("probe_interval_compact", C.c_int), ("max_partial_compacts", C.c_uint64),
                ("max_memory_compact", C.c_uint64), ("max_memory_resident", C.c_uint64),
                ("max_memory_abort", C.c_uint64), ("verbose", C.c_int), ("check_alignment_correct", C.c_bool),
                ("timer", Timer), ("max_num_threads", C.c_int), ("min_offsets_per_thread", C.c_int)]


class AlignerAttr(C.Structure):
    _fields_ = [("distance_metric", C.c_int), ("alignment_scope", C.c_int), ("alignment_form", AlignmentForm),
                ("linear_penalties", LinearPenalties), ("affine_penalties", AffinePenalties),
                ("affine2p_penalties", Affine2pPenalties), ("heuristic", Heuristic), ("memory_mode", C.c_int),
                ("mm_allocator", C.c_void_p), ("plot", PlotAttr), ("system", System)]


class Cigar(C.Structure):
    _fields_ = [("operations", C.POINTER(C.c_char)), ("max_operations", C.c_int), ("begin_offset", C.c_int),
                ("end_offset", C.c_int), ("score", C.c_int), ("end_v", C.c_int), ("end_h", C.c_int),
                ("has_misms", C.c_bool), ("cigar_buffer", C.POINTER(C.c_uint32)), ("cigar_length", C.c_int)]


class AlignStatus(C.Structure):
    _fields_ = [("status", C.c_int), ("score", C.c_int), ("dropped", C.c_bool), ("num_null_steps", C.c_int),
                ("memory_used", C.c_uint64), ("wf_align_compute", C.c_void_p), ("wf_align_extend", C.c_void_p)]


class EndPos(C.Structure):
    _fields_ = [("score", C.c_int), ("k", C.c_int), ("offset", C.c_int32)]


class Aligner(C.Structure):  # wavefront_aligner_t, WFA2-lib's layout
    _fields_ = [("align_mode", C.c_int), ("align_mode_tag", C.c_char_p), ("align_status", AlignStatus),
                ("sequences_", C.c_uint64 * 13), ("alignment_scope", C.c_int), ("alignment_form", AlignmentForm),
                ("penalties_", C.c_int32 * 21), ("heuristic", Heuristic), ("memory_mode", C.c_int),
                ("wf_components_", C.c_uint64 * 12), ("component_begin", C.c_int), ("component_end", C.c_int),
                ("alignment_end_pos", EndPos), ("bialigner", C.c_void_p), ("cigar", C.POINTER(Cigar)),
                ("mm_allocator_own", C.c_bool), ("mm_allocator", C.c_void_p), ("wavefront_slab", C.c_void_p),
                ("plot", C.c_void_p), ("system", System)]


class Config(C.Structure):
    _fields_ = [("match", C.c_int), ("mismatch", C.c_int), ("gap_opening", C.c_int), ("gap_extension", C.c_int),
                ("score_only", C.c_int), ("max_alignment_steps", C.c_int), ("metric", C.c_int),
                ("gap_opening2", C.c_int), ("gap_extension2", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("kernel_ms", C.c_double), ("pack_ms", C.c_double), ("total_ms", C.c_double),
                ("launches", C.c_int), ("retried_pairs", C.c_int), ("num_warps", C.c_int), ("ring_w", C.c_int),
                ("arena_bytes", C.c_int64), ("total_runs", C.c_int64), ("h2d_bytes", C.c_int64),
                ("d2h_bytes", C.c_int64), ("used_graph", C.c_int), ("upload_host_ms", C.c_double),
                ("upload_copy_ms", C.c_double), ("pipeline_chunks", C.c_int)]


P = C.POINTER
_i64p = P(C.c_int64)
_ip = P(C.c_int)
_u32p = P(C.c_uint32)

# name -> (restype, argtypes); every entry point declared in include/wfa_gpu.h
SIGNATURES = {
    "wavefront_aligner_new": (P(Aligner), [P(AlignerAttr)]),
    "wavefront_aligner_delete": (None, [P(Aligner)]),
    "wavefront_align": (C.c_int, [P(Aligner), C.c_char_p, C.c_int, C.c_char_p, C.c_int]),
    "wavefront_align_strerror": (C.c_char_p, [C.c_int]),
    "wavefront_align_strerror_short": (C.c_char_p, [C.c_int]),
    "wavefront_aligner_set_alignment_end_to_end": (None, [P(Aligner)]),
    "wavefront_aligner_set_heuristic_none": (None, [P(Aligner)]),
    "wavefront_aligner_set_max_alignment_steps": (None, [P(Aligner), C.c_int]),
    "cigar_sprint": (C.c_int, [C.c_char_p, P(Cigar), C.c_bool]),
    "cigar_score_gap_affine": (C.c_int, [P(Cigar), P(AffinePenalties)]),
    "cigar_score_edit": (C.c_int, [P(Cigar)]),
    "cigar_score_gap_linear": (C.c_int, [P(Cigar), P(LinearPenalties)]),
    "cigar_score_gap_affine2p": (C.c_int, [P(Cigar), P(Affine2pPenalties)]),
    "cigar_get_CIGAR": (None, [P(Cigar), C.c_bool, P(_u32p), _ip]),
    "wavefront_align_batch": (C.c_int, [P(Aligner), C.c_int, P(C.c_char_p), _ip, P(C.c_char_p), _ip, _ip, _ip]),
    "wavefront_batch_cigar": (C.c_int, [P(Aligner), C.c_int, P(_u32p), _ip]),
    "wfg_context_create": (C.c_void_p, [C.c_int]),
    "wfg_context_destroy": (None, [C.c_void_p]),
    "wfg_last_error": (C.c_char_p, [C.c_void_p]),
    "wfg_upload": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int64, _i64p, _ip, _i64p, _ip]),
    "wfg_set_order": (C.c_int, [C.c_void_p, _ip]),
    "wfg_set_predictions": (C.c_int, [C.c_void_p, P(C.c_float)]),
    "wfg_run": (C.c_int, [C.c_void_p, P(Config), C.c_int]),
    "wfg_fetch": (C.c_int, [C.c_void_p, _ip, _ip, _i64p, _ip, _u32p, C.c_int64, _i64p]),
    "wfg_align_host": (C.c_int, [C.c_void_p, P(Config), C.c_int, C.c_int, C.c_void_p, C.c_int64, _i64p, _ip,
                                 _i64p, _ip, _ip, _ip, _i64p, _ip, _u32p, C.c_int64, _i64p]),
    "wfg_get_stats": (C.c_int, [C.c_void_p, P(Stats)]),
    "wfg_set_arena_limits": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "wfg_set_exec_shape": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "wfg_set_graph": (C.c_int, [C.c_void_p, C.c_int]),
    "wfg_set_pipeline": (C.c_int, [C.c_void_p, C.c_int]),
    "wfg_set_retry_shape": (C.c_int, [C.c_void_p, C.c_int]),
    "wfg_set_learned_policy": (C.c_int, [C.c_void_p, C.c_float, C.c_int, C.c_int, C.c_float]),
    "wfg_autotune_learned_policy": (C.c_int, [C.c_void_p, P(Config), P(C.c_float), P(C.c_float), _ip, _ip]),
    "wfg_flush_l2": (C.c_int, [C.c_void_p, C.c_int64]),
    "wfg_synchronize": (C.c_int, [C.c_void_p]),
    "wfg_host_alloc": (C.c_void_p, [C.c_int64]),
    "wfg_host_free": (None, [C.c_void_p]),
    "wfg_align_noalloc": (C.c_int, [P(Config), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                    C.c_void_p]),
    "wfg_model_param_count": (C.c_int, []),
    "wfg_model_create": (C.c_void_p, [C.c_void_p, C.c_uint64]),
    "wfg_model_destroy": (None, [C.c_void_p]),
    "wfg_model_get_params": (C.c_int, [C.c_void_p, P(C.c_float)]),
    "wfg_model_set_params": (C.c_int, [C.c_void_p, P(C.c_float)]),
    "wfg_features": (C.c_int, [C.c_void_p, P(C.c_uint16)]),
    "wfg_model_train": (C.c_int, [C.c_void_p, C.c_void_p, _ip, C.c_int, C.c_int, C.c_float, C.c_uint64,
                                  P(C.c_float)]),
    "wfg_model_gradient": (C.c_int, [C.c_void_p, C.c_void_p, P(C.c_float), P(C.c_float), P(C.c_float)]),
    "wfg_model_predict": (C.c_int, [C.c_void_p, C.c_void_p, P(C.c_float)]),
    "wfg_set_model": (C.c_int, [C.c_void_p, C.c_void_p]),
    "wfg_generate": (C.c_int, [C.c_int, C.c_int, C.c_uint64, C.c_void_p, _i64p, _i64p, _ip, _i64p, _ip]),
}

_lib = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Load libbiwfa_gb300.so and declare its signatures. Raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def attr_default() -> AlignerAttr:
    lib = load()
    return AlignerAttr.in_dll(lib, "wavefront_aligner_attr_default")
