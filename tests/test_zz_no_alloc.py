"""The allocation-free two-site H_eff entry point against the regular one.

tn_heff2_apply_noalloc serves callers that cannot allocate device memory
(they hand over buffers from their own arena): every argument is a device
pointer and its intermediates live in the library's static 64 MiB device
array.  Two calls in a row, on different inputs and shapes, must match
tn_heff2_apply (which allocates) to the FP64 unit tolerance of the parity
tests, 1e-12 relative.  Kept in a file of its own, collected last."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _crand(rng, *shape):
    return np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def test_noalloc_heff2_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    import tngpu

    ctx = tngpu.context()
    rng = np.random.default_rng(2024)
    d = 2
    for (cl, cr, wl, wm, wr) in [(96, 80, 5, 5, 5), (130, 64, 3, 4, 5)]:
        L, W1, W2 = _crand(rng, cl, wl, cl), _crand(rng, wl, d, d, wm), _crand(rng, wm, d, d, wr)
        R, th = _crand(rng, cr, wr, cr), _crand(rng, cl, d, d, cr)
        ref = np.zeros((cl, d, d, cr), dtype=np.complex128, order="F")
        ctx.check(ctx.lib.tn_heff2_apply(ctx.h, cl, cr, d, wl, wm, wr, _dp(L), _dp(W1), _dp(W2),
                                         _dp(R), _dp(th), _dp(ref), 0))

        def dev(a):  # column-major complex data as a flat device buffer
            return torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).to("cuda")

        dL, dW1, dW2, dR, dth = dev(L), dev(W1), dev(W2), dev(R), dev(th)
        dout = torch.zeros(cl * d * d * cr, dtype=torch.complex128, device="cuda")
        torch.cuda.synchronize()
        ctx.check(ctx.lib.tn_heff2_apply_noalloc(
            ctx.h, cl, cr, d, wl, wm, wr, dL.data_ptr(), dW1.data_ptr(), dW2.data_ptr(),
            dR.data_ptr(), dth.data_ptr(), dout.data_ptr()))
        got = dout.cpu().numpy().reshape((cl, d, d, cr), order="F")
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-12


def test_noalloc_rejects_oversized_problem():
    torch = pytest.importorskip("torch")
    import tngpu

    ctx = tngpu.context()
    cl = cr = 1024  # T1 + T2 need 640 MiB at w = 5, beyond the 64 MiB array
    buf = torch.zeros(8, dtype=torch.complex128, device="cuda")
    p = buf.data_ptr()
    rc = ctx.lib.tn_heff2_apply_noalloc(ctx.h, cl, cr, 2, 5, 5, 5, p, p, p, p, p, p)
    assert rc == -1
    assert "64 MiB" in ctx.lib.tn_last_error(ctx.h).decode()
