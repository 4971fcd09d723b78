"""wfg_align_noalloc: the entry point for callers that cannot allocate device memory.

The caller owns the inputs and outputs (here: torch tensors standing in for a host
framework's own device memory); the library's scratch is its fixed __device__ array.
Results must equal the allocating batch entry point's (wfg_run) exactly, on two calls in
a row (the second call reuses the array the first one left behind), and the golden pairs'
lines must equal WFA2-lib's own expected `score\\tCIGAR` lines."""
import ctypes as C

import numpy as np
import pytest

import biwfa_gpu_pii2025_gb300 as pkg
from biwfa_gpu_pii2025_gb300 import _capi
from golden_data import printed_line, utest
from oracle import binding

NOALLOC_SIG = (C.c_int, [C.POINTER(_capi.Config), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                         C.c_void_p])
MAX_PAIRS = 4096
MAX_PAIR_LEN = 1024
N_SHORT = 600


def _lib():
    lib = pkg.load_library()
    fn = lib.wfg_align_noalloc
    fn.restype, fn.argtypes = NOALLOC_SIG
    return lib


def _batch():
    short = pkg.PairBatch.generate(2, N_SHORT, seed=77)
    data = utest()
    fits = [i for i, (p, t) in enumerate(data["pairs"]) if len(p) + len(t) <= MAX_PAIR_LEN][:120]
    pats = [short.pattern(i) for i in range(short.n)] + [data["pairs"][i][0].encode() for i in fits]
    txts = [short.text(i) for i in range(short.n)] + [data["pairs"][i][1].encode() for i in fits]
    # one pair above the per-pair limit, two empty-sided pairs, and a fully mismatched 100 bp
    # pair (a whole-pair leaf of a high score under the larger penalty sets)
    pats += [b"A" * 700, b"", b"ACGT", b"A" * 100]
    txts += [b"A" * 400, b"ACG", b"", b"C" * 100]
    return pkg.PairBatch.from_lists(pats, txts), fits


class _Buffers:
    """Device inputs and outputs of one batch, allocated by the caller (torch) up front."""

    def __init__(self, torch, b):
        dev = torch.device("cuda:0")
        self.torch = torch
        self.n = b.n
        self.d_seq = torch.from_numpy(b.seq.copy()).to(dev)
        self.d_poff = torch.from_numpy(b.p_off.copy()).to(dev)
        self.d_plen = torch.from_numpy(b.plen.copy()).to(dev)
        self.d_toff = torch.from_numpy(b.t_off.copy()).to(dev)
        self.d_tlen = torch.from_numpy(b.tlen.copy()).to(dev)
        self.runs_cap = int(b.plen.astype(np.int64).sum() + b.tlen.astype(np.int64).sum() + b.n)
        self.d_scores = torch.empty((b.n,), dtype=torch.int32, device=dev)
        self.d_status = torch.empty((b.n,), dtype=torch.int32, device=dev)
        self.d_roff = torch.empty((b.n,), dtype=torch.int64, device=dev)
        self.d_rlen = torch.empty((b.n,), dtype=torch.int32, device=dev)
        self.d_runs = torch.empty((self.runs_cap,), dtype=torch.int32, device=dev)

    def call(self, lib, cfg):
        """One call; returns its status and the device's free bytes just before and after it."""
        t = self.torch
        for a, v in ((self.d_scores, -7), (self.d_status, -7), (self.d_roff, 0), (self.d_rlen, 0), (self.d_runs, 0)):
            a.fill_(v)
        t.cuda.synchronize()
        free0 = t.cuda.mem_get_info()[0]
        st = lib.wfg_align_noalloc(C.byref(cfg), self.n, self.d_seq.data_ptr(), self.d_poff.data_ptr(),
                                   self.d_plen.data_ptr(), self.d_toff.data_ptr(), self.d_tlen.data_ptr(),
                                   self.d_scores.data_ptr(), self.d_status.data_ptr(), self.d_roff.data_ptr(),
                                   self.d_rlen.data_ptr(), self.d_runs.data_ptr(), self.runs_cap, None)
        t.cuda.synchronize()
        free1 = t.cuda.mem_get_info()[0]
        out = (self.d_scores.cpu().numpy(), self.d_status.cpu().numpy(), self.d_roff.cpu().numpy(),
               self.d_rlen.cpu().numpy(), self.d_runs.cpu().numpy().view(np.uint32))
        return st, free0, free1, out


# (penalties, expected refusal): the default set; match < 0 within the scope limit (internal
# x 6, o 8, e 3: scope 12); a score scope of exactly 16; match < 0 beyond it (scope 18, refused)
PENALTY_SETS = [((0, 4, 6, 2), False), ((-1, 2, 4, 1), False), ((0, 4, 13, 2), False), ((-1, 4, 6, 2), True)]


@pytest.mark.gpu
@pytest.mark.parametrize("penalties,refused", PENALTY_SETS, ids=["0_4_6_2", "m1_2_4_1", "0_4_13_2_scope16",
                                                                   "m1_4_6_2_scope18"])
def test_noalloc_matches_allocating_entry_point_twice(penalties, refused):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _lib()
    b, fits = _batch()
    bufs = _Buffers(torch, b)
    too_long = (b.plen.astype(np.int64) + b.tlen) > MAX_PAIR_LEN
    assert too_long.sum() == 1
    ok = ~too_long
    for score_only in (False, True):
        cfg = _capi.Config(*penalties, 1 if score_only else 0, 0)
        if refused:
            st, _, _, _ = bufs.call(lib, cfg)
            assert st == _capi.WF_STATUS_UNSUPPORTED
            continue
        al = pkg.BatchAligner(0)
        ref = al.align(b, penalties=penalties, score_only=score_only)
        al.close()
        for call in range(2):
            st, free0, free1, (scores, status, roff, rlen, runs) = bufs.call(lib, cfg)
            assert st == _capi.WF_STATUS_ALG_COMPLETED
            if call == 1:
                assert free1 == free0, "the second call changed the device's free memory"
            assert (status[too_long] == _capi.WF_STATUS_UNSUPPORTED).all()
            # every in-limit pair: wfg_run's status, score and CIGAR, or WF_STATUS_OOM where the
            # fixed arena is too small (never a different result)
            oom = ok & (status == _capi.WF_STATUS_OOM)
            same = ok & ~oom
            assert (status[same] == ref.status[same]).all(), (call, np.unique(status))
            assert np.array_equal(scores[same], ref.scores[same]), call
            if not score_only:
                for i in np.nonzero(same)[0]:
                    assert np.array_equal(runs[roff[i]:roff[i] + rlen[i]], ref.runs_of(i)), (call, i)
            if penalties == (0, 4, 6, 2):
                assert not oom.any(), np.nonzero(oom)[0]
                # WFA2-lib's own expected lines for the golden pairs (test.biwfa{,.score}.affine.alg)
                s = utest()["sets"]["test.biwfa.score.affine.alg" if score_only else "test.biwfa.affine.alg"]
                for j, gi in enumerate(fits):
                    i = N_SHORT + j
                    cig = "" if score_only else pkg.runs_to_cigar(runs[roff[i]:roff[i] + rlen[i]])
                    got = printed_line(int(scores[i]), "") if score_only else printed_line(
                        int(scores[i]) if cig else -1, cig)
                    assert got == s["lines"][gi], (call, gi)
            # the fully mismatched pair (the last one) against the oracle
            last = b.n - 1
            if status[last] == 0:
                _, oscore, oops, _ = binding.oracle_align(b.pattern(last), b.text(last), penalties, score_only)
                assert scores[last] == oscore
                if not score_only:
                    assert pkg.runs_to_ops(runs[roff[last]:roff[last] + rlen[last]]) == oops
            else:
                assert status[last] == _capi.WF_STATUS_OOM


def test_noalloc_refuses_oversized_calls():
    """Host-side refusals, made before any device work (so this runs without a GPU too)."""
    fn = _lib().wfg_align_noalloc
    cfg = _capi.Config(0, 4, 6, 2, 0, 0)
    # more pairs than the fixed scratch holds
    assert fn(C.byref(cfg), MAX_PAIRS + 1, None, None, None, None, None, None, None, None, None, None, 0,
              None) == _capi.WF_STATUS_UNSUPPORTED
    # penalties whose score scope exceeds the fixed rings
    big = _capi.Config(0, 40, 6, 2, 0, 0)
    assert fn(C.byref(big), 1, None, None, None, None, None, None, None, None, None, None, 0,
              None) == _capi.WF_STATUS_UNSUPPORTED
    # another distance
    lin = _capi.Config(0, 4, 2, 0, 0, 0, _capi.METRIC_GAP_LINEAR)
    assert fn(C.byref(lin), 1, None, None, None, None, None, None, None, None, None, None, 0,
              None) == _capi.WF_STATUS_UNSUPPORTED
