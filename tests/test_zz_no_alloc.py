"""The allocation-free two-site H_eff entry point against the regular one.

tn_heff2_apply_noalloc is for callers that cannot allocate device memory: a
host that owns the GPU memory through its own arena and budget hands the
library buffers from it, and a long run must not stop halfway on an
out-of-memory error.  Every argument is a device pointer and the
intermediates live in the library's static 64 MiB device array.

The tests check that
  * two calls in a row, on different inputs and shapes (one at the 4096-entry
    limit of the merged two-site operator), match tn_heff2_apply (which
    allocates) to the FP64 unit tolerance of the parity tests, 1e-12 relative;
  * a call allocates nothing: the high-water mark of the device's default
    memory pool (the one the library's contexts draw from) does not rise
    during the call, and the device's free memory does not change;
  * oversized problems and host pointers are rejected before anything runs.

Kept in a file of its own, collected last."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# CUmemPool_attribute values (cuda.h)
_USED_MEM_CURRENT, _USED_MEM_HIGH = 7, 8


def _crand(rng, *shape):
    return np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class _Pool:
    """The device's default memory pool, read through the driver API."""

    def __init__(self, device):
        self.cu = C.CDLL("libcuda.so.1")
        dev, self.pool = C.c_int(), C.c_void_p()
        assert self.cu.cuDeviceGet(C.byref(dev), device) == 0
        assert self.cu.cuDeviceGetDefaultMemPool(C.byref(self.pool), dev) == 0

    def get(self, attr):
        v = C.c_uint64()
        assert self.cu.cuMemPoolGetAttribute(self.pool, attr, C.byref(v)) == 0
        return v.value

    def reset_high(self):  # setting the high-water mark to 0 resets it to the current use
        z = C.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, _USED_MEM_HIGH, C.byref(z)) == 0


def _problem(rng, cl, cr, d, wl, wm, wr):
    return dict(L=_crand(rng, cl, wl, cl), W1=_crand(rng, wl, d, d, wm), W2=_crand(rng, wm, d, d, wr),
                R=_crand(rng, cr, wr, cr), th=_crand(rng, cl, d, d, cr))


def test_noalloc_heff2_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    import tngpu

    ctx = tngpu.context()
    pool = _Pool(ctx.device)
    rng = np.random.default_rng(2024)
    d = 2
    # the second shape sits at the operator limit: (wl d^2)(d^2 wr) = 64 x 64 = 4096
    for call, (cl, cr, wl, wm, wr) in enumerate([(96, 80, 5, 5, 5), (40, 24, 16, 3, 16)]):
        p = _problem(rng, cl, cr, d, wl, wm, wr)
        ref = np.zeros((cl, d, d, cr), dtype=np.complex128, order="F")
        ctx.check(ctx.lib.tn_heff2_apply(ctx.h, cl, cr, d, wl, wm, wr, _dp(p["L"]), _dp(p["W1"]),
                                         _dp(p["W2"]), _dp(p["R"]), _dp(p["th"]), _dp(ref), 0))

        def dev(a):  # column-major complex data as a flat device buffer
            return torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).to("cuda")

        dL, dW1, dW2, dR, dth = dev(p["L"]), dev(p["W1"]), dev(p["W2"]), dev(p["R"]), dev(p["th"])
        dout = torch.zeros(cl * d * d * cr, dtype=torch.complex128, device="cuda")
        torch.cuda.synchronize()

        def run():
            ctx.check(ctx.lib.tn_heff2_apply_noalloc(
                ctx.h, cl, cr, d, wl, wm, wr, dL.data_ptr(), dW1.data_ptr(), dW2.data_ptr(),
                dR.data_ptr(), dth.data_ptr(), dout.data_ptr()))

        if call == 0:
            run()  # the first call may load the module that holds the static array
        used0 = pool.get(_USED_MEM_CURRENT)
        pool.reset_high()
        free0 = torch.cuda.mem_get_info()[0]
        run()
        free1 = torch.cuda.mem_get_info()[0]
        assert pool.get(_USED_MEM_HIGH) <= used0, "the call drew memory from the pool"
        assert free1 == free0, "the device's free memory changed during the call"
        got = dout.cpu().numpy().reshape((cl, d, d, cr), order="F")
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-12


def test_noalloc_rejects_oversized_and_host_arguments():
    torch = pytest.importorskip("torch")
    import tngpu

    ctx = tngpu.context()
    buf = torch.zeros(8, dtype=torch.complex128, device="cuda")
    p = buf.data_ptr()
    cl = cr = 1024  # T1 + T2 need 640 MiB at w = 5, beyond the 64 MiB array
    assert ctx.lib.tn_heff2_apply_noalloc(ctx.h, cl, cr, 2, 5, 5, 5, p, p, p, p, p, p) == -1
    assert "64 MiB" in ctx.lib.tn_last_error(ctx.h).decode()
    # merged operator (17 * 4) x (4 * 17) = 4624 entries, above the 4096 limit
    assert ctx.lib.tn_heff2_apply_noalloc(ctx.h, 8, 8, 2, 17, 2, 17, p, p, p, p, p, p) == -1
    assert "4096" in ctx.lib.tn_last_error(ctx.h).decode()
    host = np.zeros(2 * 4 * 4 * 4 * 4, dtype=np.float64)
    hp = host.ctypes.data
    assert ctx.lib.tn_heff2_apply_noalloc(ctx.h, 4, 4, 2, 1, 1, 1, hp, p, p, p, p, p) == -1
    assert "device pointer" in ctx.lib.tn_last_error(ctx.h).decode()
