"""wfg_align_noalloc: the entry point for callers that cannot allocate device memory.

The caller owns the inputs and outputs (here: torch tensors standing in for a host
framework's own device memory); the library's scratch is its fixed __device__ array.
Results must equal the allocating batch entry point's (wfg_run) exactly, on two calls in
a row (the second call reuses the array the first one left behind)."""
import ctypes as C

import numpy as np
import pytest

import biwfa_gpu_pii2025_gb300 as pkg
from biwfa_gpu_pii2025_gb300 import _capi
from golden_data import utest

pytestmark = pytest.mark.gpu

NOALLOC_SIG = (C.c_int, [C.POINTER(_capi.Config), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                         C.c_void_p])
MAX_PAIRS = 4096
MAX_PAIR_LEN = 1024


def _batch():
    short = pkg.PairBatch.generate(2, 600, seed=77)
    data = utest()
    fits = [(p, t) for p, t in data["pairs"] if len(p) + len(t) <= MAX_PAIR_LEN][:120]
    pats = [short.pattern(i) for i in range(short.n)] + [p.encode() for p, _ in fits]
    txts = [short.text(i) for i in range(short.n)] + [t.encode() for _, t in fits]
    # one pair above the per-pair limit, and two empty-sided pairs
    pats += [b"A" * 700, b"", b"ACGT"]
    txts += [b"A" * 400, b"ACG", b""]
    return pkg.PairBatch.from_lists(pats, txts)


def _noalloc(lib, torch, b, cfg):
    dev = torch.device("cuda:0")
    d_seq = torch.from_numpy(b.seq.copy()).to(dev)
    d_poff = torch.from_numpy(b.p_off.copy()).to(dev)
    d_plen = torch.from_numpy(b.plen.copy()).to(dev)
    d_toff = torch.from_numpy(b.t_off.copy()).to(dev)
    d_tlen = torch.from_numpy(b.tlen.copy()).to(dev)
    n = b.n
    runs_cap = int(b.plen.astype(np.int64).sum() + b.tlen.astype(np.int64).sum() + n)
    d_scores = torch.full((n,), -7, dtype=torch.int32, device=dev)
    d_status = torch.full((n,), -7, dtype=torch.int32, device=dev)
    d_roff = torch.zeros((n,), dtype=torch.int64, device=dev)
    d_rlen = torch.zeros((n,), dtype=torch.int32, device=dev)
    d_runs = torch.zeros((runs_cap,), dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    st = lib.wfg_align_noalloc(C.byref(cfg), n, d_seq.data_ptr(), d_poff.data_ptr(), d_plen.data_ptr(),
                               d_toff.data_ptr(), d_tlen.data_ptr(), d_scores.data_ptr(), d_status.data_ptr(),
                               d_roff.data_ptr(), d_rlen.data_ptr(), d_runs.data_ptr(), runs_cap, None)
    torch.cuda.synchronize()
    assert st == _capi.WF_STATUS_ALG_COMPLETED
    return (d_scores.cpu().numpy(), d_status.cpu().numpy(), d_roff.cpu().numpy(), d_rlen.cpu().numpy(),
            d_runs.cpu().numpy().view(np.uint32))


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = pkg.load_library()
    fn = lib.wfg_align_noalloc
    fn.restype, fn.argtypes = NOALLOC_SIG
    b = _batch()
    for score_only in (False, True):
        al = pkg.BatchAligner(0)
        ref = al.align(b, score_only=score_only)
        al.close()
        cfg = _capi.Config(0, 4, 6, 2, 1 if score_only else 0, 0)
        for call in range(2):
            scores, status, roff, rlen, runs = _noalloc(lib, torch, b, cfg)
            too_long = (b.plen.astype(np.int64) + b.tlen) > MAX_PAIR_LEN
            assert too_long.sum() == 1
            assert (status[too_long] == _capi.WF_STATUS_UNSUPPORTED).all()
            ok = ~too_long
            assert (status[ok] == 0).all(), (call, np.unique(status))
            assert np.array_equal(scores[ok], ref.scores[ok]), call
            for i in np.nonzero(ok)[0]:
                got = runs[roff[i]:roff[i] + rlen[i]]
                assert np.array_equal(got, ref.runs_of(i)), (call, i)


def test_noalloc_refuses_oversized_calls():
    lib = pkg.load_library()
    fn = lib.wfg_align_noalloc
    fn.restype, fn.argtypes = NOALLOC_SIG
    cfg = _capi.Config(0, 4, 6, 2, 0, 0)
    # more pairs than the fixed scratch holds: refused before any device work
    assert fn(C.byref(cfg), MAX_PAIRS + 1, None, None, None, None, None, None, None, None, None, None, 0,
              None) == _capi.WF_STATUS_UNSUPPORTED
    # penalties whose score scope exceeds the fixed rings
    big = _capi.Config(0, 40, 6, 2, 0, 0)
    assert fn(C.byref(big), 1, None, None, None, None, None, None, None, None, None, None, 0,
              None) == _capi.WF_STATUS_UNSUPPORTED
