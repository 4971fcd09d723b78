"""Python mirror of the C ABI (include/wfa_gpu.h) for tests, the benchmark and scripting.

Two classes, matching the library's two surfaces:
  * WavefrontAligner  — WFA2-lib's aligner API (wavefront_aligner_new / wavefront_align /
                        cigar), one pair per call, computed on the GPU;
  * BatchAligner      — the wfg_* batch path (upload / run / fetch, or align end to end).
All computation happens in libbiwfa_gb300.so; nothing here aligns.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _capi

_i64p = C.POINTER(C.c_int64)
_ip = C.POINTER(C.c_int)
_u32p = C.POINTER(C.c_uint32)


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


@dataclass
class PairBatch:
    """Pairs laid out in one byte buffer: pattern i = seq[p_off[i]:p_off[i]+plen[i]], text likewise."""
    seq: np.ndarray    # uint8
    p_off: np.ndarray  # int64
    plen: np.ndarray   # int32
    t_off: np.ndarray  # int64
    tlen: np.ndarray   # int32

    @property
    def n(self) -> int:
        return int(self.plen.shape[0])

    @classmethod
    def from_lists(cls, patterns, texts) -> "PairBatch":
        bufs, p_off, plen, t_off, tlen = [], [], [], [], []
        cur = 0
        for p, t in zip(patterns, texts):
            pb = p.encode() if isinstance(p, str) else bytes(p)
            tb = t.encode() if isinstance(t, str) else bytes(t)
            p_off.append(cur); plen.append(len(pb)); bufs.append(pb); cur += len(pb)
            t_off.append(cur); tlen.append(len(tb)); bufs.append(tb); cur += len(tb)
        seq = np.frombuffer(b"".join(bufs) or b"\0", dtype=np.uint8).copy()
        return cls(seq, np.asarray(p_off, np.int64), np.asarray(plen, np.int32),
                   np.asarray(t_off, np.int64), np.asarray(tlen, np.int32))

    @classmethod
    def generate(cls, workload: int, n: int, seed: int) -> "PairBatch":
        """Seeded synthetic pairs (wfg_generate): workloads 1..5 as documented in wfa_gpu.h."""
        lib = _capi.load()
        total = C.c_int64(0)
        st = lib.wfg_generate(workload, n, seed, None, C.byref(total), None, None, None, None)
        if st != 0:
            raise ValueError(f"wfg_generate({workload}) failed: {st}")
        seq = np.empty(max(total.value, 1), np.uint8)
        p_off = np.empty(n, np.int64); plen = np.empty(n, np.int32)
        t_off = np.empty(n, np.int64); tlen = np.empty(n, np.int32)
        lib.wfg_generate(workload, n, seed, seq.ctypes.data_as(C.c_void_p), C.byref(total),
                         _ptr(p_off, _i64p), _ptr(plen, _ip), _ptr(t_off, _i64p), _ptr(tlen, _ip))
        return cls(seq, p_off, plen, t_off, tlen)

    def pattern(self, i: int) -> bytes:
        return self.seq[self.p_off[i]:self.p_off[i] + self.plen[i]].tobytes()

    def text(self, i: int) -> bytes:
        return self.seq[self.t_off[i]:self.t_off[i] + self.tlen[i]].tobytes()

    def subset(self, idx) -> "PairBatch":
        return PairBatch.from_lists([self.pattern(i) for i in idx], [self.text(i) for i in idx])


class PinnedHost:
    """Page-locked host arrays from wfg_host_alloc (freed on close)."""

    def __init__(self):
        self.lib = _capi.load()
        self._ptrs = []

    def empty(self, n: int, dtype) -> np.ndarray:
        dtype = np.dtype(dtype)
        nbytes = max(int(n) * dtype.itemsize, dtype.itemsize)
        p = self.lib.wfg_host_alloc(nbytes)
        if not p:
            raise MemoryError(f"wfg_host_alloc({nbytes}) failed")
        self._ptrs.append(p)
        return np.frombuffer((C.c_uint8 * nbytes).from_address(p), dtype=dtype)[: int(n)]

    def copy(self, a: np.ndarray) -> np.ndarray:
        out = self.empty(a.size, a.dtype)
        out[...] = a.reshape(-1)
        return out

    def batch(self, b: "PairBatch") -> "PairBatch":
        return PairBatch(self.copy(b.seq), self.copy(b.p_off), self.copy(b.plen), self.copy(b.t_off),
                         self.copy(b.tlen))

    def close(self):
        for p in self._ptrs:
            self.lib.wfg_host_free(p)
        self._ptrs = []


@dataclass
class BatchResult:
    scores: np.ndarray
    status: np.ndarray
    run_off: np.ndarray
    run_len: np.ndarray
    runs: np.ndarray

    def runs_of(self, i: int) -> np.ndarray:
        return self.runs[self.run_off[i]:self.run_off[i] + self.run_len[i]]

    def cigar(self, i: int) -> str:
        return runs_to_cigar(self.runs_of(i))


def runs_to_cigar(runs: np.ndarray) -> str:
    """Run-length CIGAR text as WFA2-lib's cigar_sprint(print_matches=true) prints it."""
    return "".join(f"{int(r) >> 4}{_capi.OP_CHAR[int(r) & 15]}" for r in runs)


def runs_to_ops(runs: np.ndarray) -> str:
    return "".join(_capi.OP_CHAR[int(r) & 15] * (int(r) >> 4) for r in runs)


class BatchAligner:
    """The GB300 batch path (wfg_context_t)."""

    def __init__(self, device: int = 0):
        self.lib = _capi.load()
        self.ctx = self.lib.wfg_context_create(device)
        if not self.ctx:
            raise RuntimeError("wfg_context_create failed: no usable CUDA device")
        self.n = 0

    def close(self):
        if self.ctx:
            self.lib.wfg_context_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int, what: str):
        if st != 0:
            msg = self.lib.wfg_last_error(self.ctx).decode(errors="replace")
            raise RuntimeError(f"{what} failed ({st}): {msg}")

    @staticmethod
    def config(penalties=(0, 4, 6, 2), score_only=False, max_steps=0, metric=0) -> _capi.Config:
        """metric: _capi.METRIC_GAP_AFFINE (default), METRIC_EDIT or METRIC_INDEL (penalties unused),
        METRIC_GAP_LINEAR (match, mismatch, indel, -) or METRIC_GAP_AFFINE_2P (match, mismatch,
        o1, e1, o2, e2)."""
        m, x, o, e = penalties[:4]
        o2, e2 = (penalties[4], penalties[5]) if len(penalties) >= 6 else (0, 0)
        return _capi.Config(m, x, o, e, 1 if score_only else 0, max_steps, metric, o2, e2)

    def upload(self, b: PairBatch):
        self._batch = b  # keep host buffers alive
        st = self.lib.wfg_upload(self.ctx, b.n, b.seq.ctypes.data_as(C.c_void_p), int(b.seq.shape[0]),
                                 _ptr(b.p_off, _i64p), _ptr(b.plen, _ip), _ptr(b.t_off, _i64p), _ptr(b.tlen, _ip))
        self._check(st, "wfg_upload")
        self.n = b.n

    def set_order(self, order: np.ndarray):
        order = np.ascontiguousarray(order, np.int32)
        self._check(self.lib.wfg_set_order(self.ctx, _ptr(order, _ip)), "wfg_set_order")

    def set_arena_limits(self, ring_w: int = 0, leaf_words: int = 0):
        self._check(self.lib.wfg_set_arena_limits(self.ctx, ring_w, leaf_words), "wfg_set_arena_limits")

    def set_exec_shape(self, group_warps: int = 1, ring_in_smem: bool = False):
        self._check(self.lib.wfg_set_exec_shape(self.ctx, group_warps, 1 if ring_in_smem else 0),
                    "wfg_set_exec_shape")

    def set_graph(self, enable: bool = True):
        """Run each wfg_run's device work as one CUDA graph (default) or as direct launches."""
        self._check(self.lib.wfg_set_graph(self.ctx, 1 if enable else 0), "wfg_set_graph")

    def set_pipeline(self, enable: bool = True):
        """Let align_into (wfg_align_host) overlap its input copy with the alignment (default)."""
        self._check(self.lib.wfg_set_pipeline(self.ctx, 1 if enable else 0), "wfg_set_pipeline")

    def set_retry_shape(self, group_warps: int = 8):
        """Warps per pair of the retry passes (default 8)."""
        self._check(self.lib.wfg_set_retry_shape(self.ctx, group_warps), "wfg_set_retry_shape")

    def set_learned_policy(self, wide_threshold=1200.0, wide_warps=8, wide_smem=True, ring_margin=1.4):
        self._check(self.lib.wfg_set_learned_policy(self.ctx, wide_threshold, wide_warps, 1 if wide_smem else 0,
                                                    ring_margin), "wfg_set_learned_policy")

    def autotune_learned_policy(self, penalties=(0, 4, 6, 2)):
        """Measure the learned-schedule policies on the resident batch; keeps and returns the best."""
        cfg = self.config(penalties, False, 0)
        ms, thr = C.c_float(0), C.c_float(0)
        gw, sm = C.c_int(0), C.c_int(0)
        self._check(self.lib.wfg_autotune_learned_policy(self.ctx, C.byref(cfg), C.byref(ms), C.byref(thr),
                                                         C.byref(gw), C.byref(sm)), "wfg_autotune_learned_policy")
        return {"ms": ms.value, "wide_threshold": thr.value, "wide_warps": gw.value, "wide_smem": bool(sm.value)}

    def set_predictions(self, pred: np.ndarray):
        pred = np.ascontiguousarray(pred, np.float32)
        self._check(self.lib.wfg_set_predictions(self.ctx, pred.ctypes.data_as(C.POINTER(C.c_float))),
                    "wfg_set_predictions")

    def run(self, penalties=(0, 4, 6, 2), score_only=False, sched=_capi.SCHED_SORTED, max_steps=0, metric=0):
        cfg = self.config(penalties, score_only, max_steps, metric)
        self._check(self.lib.wfg_run(self.ctx, C.byref(cfg), sched), "wfg_run")

    def fetch(self, runs_cap: int | None = None) -> BatchResult:
        n = self.n
        scores = np.empty(n, np.int32); status = np.empty(n, np.int32)
        run_off = np.empty(n, np.int64); run_len = np.empty(n, np.int32)
        if runs_cap is None:
            b = self._batch
            runs_cap = int(b.plen.astype(np.int64).sum() + b.tlen.astype(np.int64).sum() + n)
        runs = np.empty(max(runs_cap, 1), np.uint32)
        total = C.c_int64(0)
        st = self.lib.wfg_fetch(self.ctx, _ptr(scores, _ip), _ptr(status, _ip), _ptr(run_off, _i64p),
                                _ptr(run_len, _ip), _ptr(runs, _u32p), runs_cap, C.byref(total))
        self._check(st, "wfg_fetch")
        return BatchResult(scores, status, run_off, run_len, runs[:total.value])

    def align_into(self, b: PairBatch, out: BatchResult, penalties=(0, 4, 6, 2), score_only=False,
                   sched=_capi.SCHED_SORTED, metric=0) -> int:
        """End to end through wfg_align_host into caller-owned (e.g. pinned) output arrays.
        Returns the number of CIGAR runs written to out.runs."""
        cfg = self.config(penalties, score_only, 0, metric)
        total = C.c_int64(0)
        st = self.lib.wfg_align_host(
            self.ctx, C.byref(cfg), sched, b.n, b.seq.ctypes.data_as(C.c_void_p), int(b.seq.shape[0]),
            _ptr(b.p_off, _i64p), _ptr(b.plen, _ip), _ptr(b.t_off, _i64p), _ptr(b.tlen, _ip),
            _ptr(out.scores, _ip), _ptr(out.status, _ip), _ptr(out.run_off, _i64p), _ptr(out.run_len, _ip),
            _ptr(out.runs, _u32p), int(out.runs.shape[0]), C.byref(total))
        self._check(st, "wfg_align_host")
        self.n = b.n
        return int(total.value)

    def align(self, b: PairBatch, penalties=(0, 4, 6, 2), score_only=False, sched=_capi.SCHED_SORTED,
              max_steps=0, metric=0) -> BatchResult:
        self.upload(b)
        self.run(penalties, score_only, sched, max_steps, metric)
        return self.fetch()

    def synchronize(self):
        self._check(self.lib.wfg_synchronize(self.ctx), "wfg_synchronize")

    def flush_l2(self, nbytes: int = 512 << 20):
        self._check(self.lib.wfg_flush_l2(self.ctx, nbytes), "wfg_flush_l2")

    def stats(self) -> _capi.Stats:
        s = _capi.Stats()
        self._check(self.lib.wfg_get_stats(self.ctx, C.byref(s)), "wfg_get_stats")
        return s


class ScorePredictor:
    """The learned scheduler's score model (wfg_model_t) on a BatchAligner's device.

    Features, training (forward/backward/Adam kernels, one CUDA-graph per epoch) and
    inference all run in libbiwfa_gb300.so on the batch resident in the aligner."""

    def __init__(self, aligner: BatchAligner, seed: int = 1):
        self.al = aligner
        self.lib = aligner.lib
        self.model = self.lib.wfg_model_create(aligner.ctx, seed)
        if not self.model:
            raise RuntimeError("wfg_model_create failed")
        self.nparams = self.lib.wfg_model_param_count()

    def close(self):
        if self.model:
            self.lib.wfg_set_model(self.al.ctx, None)
            self.lib.wfg_model_destroy(self.model)
            self.model = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        p = np.empty(self.nparams, np.float32)
        self.al._check(self.lib.wfg_model_get_params(self.model, p.ctypes.data_as(C.POINTER(C.c_float))),
                       "wfg_model_get_params")
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        self.al._check(self.lib.wfg_model_set_params(self.model, p.ctypes.data_as(C.POINTER(C.c_float))),
                       "wfg_model_set_params")

    def features(self) -> np.ndarray:
        """bf16 bit patterns of the resident batch's features (n x 32, uint16)."""
        f = np.empty((self.al.n, 32), np.uint16)
        self.al._check(self.lib.wfg_features(self.al.ctx, f.ctypes.data_as(C.POINTER(C.c_uint16))),
                       "wfg_features")
        return f

    def train(self, target_scores: np.ndarray, epochs=20, batch_rows=2048, lr=2e-3, seed=7) -> np.ndarray:
        t = np.ascontiguousarray(target_scores, np.int32)
        losses = np.zeros(max(epochs, 1), np.float32)
        st = self.lib.wfg_model_train(self.model, self.al.ctx, _ptr(t, _ip), epochs, batch_rows, lr, seed,
                                      losses.ctypes.data_as(C.POINTER(C.c_float)))
        self.al._check(st, "wfg_model_train")
        return losses[:epochs]

    def gradient(self, log_targets: np.ndarray):
        t = np.ascontiguousarray(log_targets, np.float32)
        g = np.empty(self.nparams, np.float32)
        loss = C.c_float(0)
        st = self.lib.wfg_model_gradient(self.model, self.al.ctx, t.ctypes.data_as(C.POINTER(C.c_float)),
                                         g.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss))
        self.al._check(st, "wfg_model_gradient")
        return float(loss.value), g

    def predict(self) -> np.ndarray:
        out = np.empty(self.al.n, np.float32)
        self.al._check(self.lib.wfg_model_predict(self.model, self.al.ctx, out.ctypes.data_as(C.POINTER(C.c_float))),
                       "wfg_model_predict")
        return out

    def attach(self):
        """Use this model for SCHED_LEARNED runs of the aligner."""
        self.al._check(self.lib.wfg_set_model(self.al.ctx, self.model), "wfg_set_model")


class WavefrontAligner:
    """WFA2-lib's aligner API (wavefront_aligner_new / wavefront_align), BiWFA on the GPU.

    distance: _capi.GAP_AFFINE (default; match, mismatch, gap_opening, gap_extension),
    _capi.GAP_AFFINE_2P (plus gap_opening2, gap_extension2), _capi.GAP_LINEAR (match, mismatch
    and the indel penalty in gap_opening), _capi.EDIT or _capi.INDEL (penalties unused)."""

    def __init__(self, match=0, mismatch=4, gap_opening=6, gap_extension=2, score_only=False,
                 memory_mode=_capi.WAVEFRONT_MEMORY_ULTRALOW, heuristic=_capi.WF_HEURISTIC_NONE,
                 distance=_capi.GAP_AFFINE, gap_opening2=24, gap_extension2=1):
        self.lib = _capi.load()
        attr = _capi.AlignerAttr.from_buffer_copy(_capi.attr_default())
        attr.distance_metric = distance
        attr.affine_penalties = _capi.AffinePenalties(match, mismatch, gap_opening, gap_extension)
        attr.affine2p_penalties = _capi.Affine2pPenalties(match, mismatch, gap_opening, gap_extension, gap_opening2,
                                                          gap_extension2)
        attr.linear_penalties = _capi.LinearPenalties(match, mismatch, gap_opening)
        attr.memory_mode = memory_mode
        attr.heuristic.strategy = heuristic
        attr.alignment_scope = _capi.COMPUTE_SCORE if score_only else _capi.COMPUTE_ALIGNMENT
        self.attr = attr
        self.distance = distance
        self.penalties = _capi.AffinePenalties(match, mismatch, gap_opening, gap_extension)
        self.wf = self.lib.wavefront_aligner_new(C.byref(attr))
        if not self.wf:
            raise RuntimeError("wavefront_aligner_new failed: no usable CUDA device")

    def close(self):
        if self.wf:
            self.lib.wavefront_aligner_delete(self.wf)
            self.wf = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def align(self, pattern, text) -> int:
        p = pattern.encode() if isinstance(pattern, str) else bytes(pattern)
        t = text.encode() if isinstance(text, str) else bytes(text)
        return self.lib.wavefront_align(self.wf, p, len(p), t, len(t))

    @property
    def status(self) -> int:
        return self.wf.contents.align_status.status

    @property
    def score(self) -> int:
        return self.wf.contents.cigar.contents.score

    def cigar_ops(self) -> str:
        cg = self.wf.contents.cigar.contents
        n = cg.end_offset - cg.begin_offset
        if n <= 0:
            return ""
        return C.string_at(C.addressof(cg.operations.contents) + cg.begin_offset, n).decode()

    def cigar_str(self, print_matches=True) -> str:
        cg = self.wf.contents.cigar
        n = cg.contents.end_offset - cg.contents.begin_offset
        buf = C.create_string_buffer(4 * max(n, 1) + 32)
        self.lib.cigar_sprint(buf, cg, print_matches)
        return buf.value.decode()

    def cigar_score(self) -> int:
        """The CIGAR rescored as align_benchmark prints it for the aligner's distance."""
        cg = self.wf.contents.cigar
        if self.distance == _capi.GAP_AFFINE_2P:
            return self.lib.cigar_score_gap_affine2p(cg, C.byref(self.attr.affine2p_penalties))
        if self.distance == _capi.GAP_LINEAR:
            return self.lib.cigar_score_gap_linear(cg, C.byref(self.attr.linear_penalties))
        if self.distance in (_capi.EDIT, _capi.INDEL):
            return self.lib.cigar_score_edit(cg)
        return self.lib.cigar_score_gap_affine(cg, C.byref(self.penalties))

    def sam_cigar(self, show_mismatches=True) -> list[int]:
        buf = _u32p()
        n = C.c_int(0)
        self.lib.cigar_get_CIGAR(self.wf.contents.cigar, show_mismatches, C.byref(buf), C.byref(n))
        return [buf[i] for i in range(n.value)]

    def align_batch(self, patterns, texts):
        n = len(patterns)
        pb = [p.encode() if isinstance(p, str) else bytes(p) for p in patterns]
        tb = [t.encode() if isinstance(t, str) else bytes(t) for t in texts]
        parr = (C.c_char_p * n)(*pb); tarr = (C.c_char_p * n)(*tb)
        pl = (C.c_int * n)(*[len(x) for x in pb]); tl = (C.c_int * n)(*[len(x) for x in tb])
        scores = (C.c_int * n)(); statuses = (C.c_int * n)()
        st = self.lib.wavefront_align_batch(self.wf, n, parr, pl, tarr, tl, scores, statuses)
        out = []
        for i in range(n):
            runs = _u32p(); nr = C.c_int(0)
            self.lib.wavefront_batch_cigar(self.wf, i, C.byref(runs), C.byref(nr))
            out.append((statuses[i], scores[i], "".join(
                f"{runs[j] >> 4}{_capi.OP_CHAR[runs[j] & 15]}" for j in range(nr.value))))
        return st, out
