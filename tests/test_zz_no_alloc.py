"""mg_grad_sweep_noalloc: the gradient sweep for callers that cannot allocate
device memory (their whole GPU budget is reserved for their own pool, or
allocator calls are forbidden in the loop that needs derivatives).  It takes
its scratch from a fixed array inside the library instead of a workspace.

Called through the C ABI, twice in a row with different fields, its output must
match mg_grad_sweep's (with a caller workspace) within the first-derivative
tolerance of the parity suite.  A low condition threshold sends many rows
through the FP64 re-solve, so the fixed scratch is really exercised.  This file
is collected last on purpose and also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from gpu_util import row_rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

D1_TOL = 1e-5


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _sweep(lib, N, M, hi, lo, nf, order, use_noalloc, cond):
    nq = M.Nmask
    nd2 = {1: 1, 2: 3, 3: 6}[M.dim]
    d1 = torch.full((nq, nf, M.dim), float("nan"), dtype=torch.float32, device=M.device)
    d2 = torch.full((nq, nf, nd2), float("nan"), dtype=torch.float32, device=M.device) if order == 2 else None
    qs = torch.zeros(nq, dtype=torch.int32, device=M.device)
    args = (M._cells, N.ptr(M._queries), nq, N.ptr(M._ngb_slots), M.des_ngb, N.ptr(M._hsml_q), N.ptr(M._hsml_lo_q),
            order, 1,
            N.ptr(hi), N.ptr(lo), nf, N.ptr(M._out_rows), N.ptr(d1), N.ptr(d2), N.ptr(qs), float(cond))
    if use_noalloc:
        st = lib.mg_grad_sweep_noalloc(*args, _stream())
    else:
        wsb = lib.mg_grad_sweep_workspace_bytes(nq)
        ws = torch.empty(wsb, dtype=torch.uint8, device=M.device)
        st = lib.mg_grad_sweep(*args, N.ptr(ws), wsb, _stream())
    N.check(st, "gradient sweep")
    torch.cuda.synchronize()
    return d1.double().cpu().numpy(), (d2.double().cpu().numpy() if d2 is not None else None)


@pytest.mark.parametrize("order", [1, 2])
def test_noalloc_matches_workspace_sweep_twice(order):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meshoid_gb300 import Meshoid
    from meshoid_gb300 import _native as N
    from meshoid_gb300 import synthetic as S
    lib = N.load()
    pos = S.plummer(1 << 15, seed=77)
    M = Meshoid(pos, des_ngb=32)
    fields = [S.fourier_fields(pos, 3, seed=5, kmax=3), np.c_[np.log(M.density.cpu().numpy()), pos[:, 0] * pos[:, 1]]]
    for f in fields:  # two calls in a row, different inputs
        hi, lo, nf, _ = M._fields(f)
        ref1, ref2 = _sweep(lib, N, M, hi, lo, nf, order, use_noalloc=False, cond=3.0)
        got1, got2 = _sweep(lib, N, M, hi, lo, nf, order, use_noalloc=True, cond=3.0)
        assert np.isfinite(got1).all()
        assert row_rel_err(got1, ref1).max() <= D1_TOL
        if order == 2:
            assert row_rel_err(got2, ref2).max() <= D1_TOL


def test_noalloc_rejects_oversized_requests():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meshoid_gb300 import _native as N
    lib = N.load()
    c = N.MgCells()
    st = lib.mg_grad_sweep_noalloc(ctypes.byref(c), None, N.MG_NOALLOC_MAX_QUERIES + 1, None, 32, None, None, 1, 1,
                                   None,
                                   None, 1, None, None, None, None, 0.0, None)
    assert st == N.MG_ERR_NOALLOC_LIMIT
    assert b"fixed scratch" in lib.mg_status_string(st)


def test_noalloc_calls_take_no_device_memory():
    """After a first call (which loads the library's module, with its fixed
    array, on the device), further calls leave the device's free memory
    unchanged: the entry point allocates nothing."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meshoid_gb300 import Meshoid
    from meshoid_gb300 import _native as N
    from meshoid_gb300 import synthetic as S
    lib = N.load()
    pos = S.plummer(1 << 14, seed=78)
    M = Meshoid(pos, des_ngb=32)
    hi, lo, nf, _ = M._fields(S.fourier_fields(pos, 2, seed=6, kmax=3))
    nq = M.Nmask
    d1 = torch.empty((nq, nf, 3), dtype=torch.float32, device=M.device)
    d2 = torch.empty((nq, nf, 6), dtype=torch.float32, device=M.device)
    qs = torch.zeros(nq, dtype=torch.int32, device=M.device)

    def call():
        N.check(lib.mg_grad_sweep_noalloc(M._cells, N.ptr(M._queries), nq, N.ptr(M._ngb_slots), M.des_ngb,
                                          N.ptr(M._hsml_q), N.ptr(M._hsml_lo_q), 2, 1, N.ptr(hi), N.ptr(lo), nf,
                                          N.ptr(M._out_rows),
                                          N.ptr(d1), N.ptr(d2), N.ptr(qs), 3.0, _stream()), "noalloc sweep")

    call()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(4):
        call()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 >= free0, f"free device memory dropped by {free0 - free1} bytes"
