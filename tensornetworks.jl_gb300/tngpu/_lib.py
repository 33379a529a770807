"""ctypes binding of libtngpu.so (declared in include/tngpu.h).

The library must be built (``python tensornetworks.jl_gb300/build.py`` or
``__graft_entry__.build()``).  There is no CPU fallback: loading fails with an
error when the shared library or a CUDA device is missing.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libtngpu.so")

TN_OK = 0
TN_ERR = {-1: "invalid argument", -2: "CUDA error", -3: "out of device memory",
          -4: "device wait timed out", -5: "numerical failure"}
PREC = {"fp64": 0, "mixed": 1, "mixed-env64": 2}

i32, i64, f64 = C.c_int32, C.c_int64, C.c_double
P = C.c_void_p
dp = C.POINTER(C.c_double)
i32p, i64p = C.POINTER(C.c_int32), C.POINTER(C.c_int64)
dpp = C.POINTER(dp)


class TruncOpts(C.Structure):
    _fields_ = [("cutoff", f64), ("maxdim", i64), ("mindim", i64)]


class DmrgOpts(C.Structure):
    _fields_ = [("nsites", i32), ("krylovdim", i32), ("kryloviter", i32), ("minsweeps", i32),
                ("maxsweeps", i32), ("tol", f64), ("tolgrad", f64), ("numconverges", f64),
                ("cutoff", f64), ("maxdim", i64), ("mindim", i64), ("precision", i32),
                ("verbose", i32), ("max_bond_updates", i32), ("profile_from_sweep", i32),
                ("refine", i32)]


class VmpsOpts(C.Structure):
    _fields_ = [("nsites", i32), ("minsweeps", i32), ("maxsweeps", i32), ("tol", f64),
                ("numconverges", f64), ("cutoff", f64), ("maxdim", i64), ("mindim", i64),
                ("verbose", i32)]


class DmrgStats(C.Structure):
    _fields_ = [("sweeps", i32), ("maxbonddim", i32), ("matvecs", i64), ("seconds", f64),
                ("energy_fp64", f64), ("last_discarded", f64), ("sweep_cap", i32),
                ("sweep_seconds", dp), ("sweep_energies", dp), ("sweep_maxdim", i32p),
                ("bond_updates", i32), ("bond_cap", i32), ("bond_seconds", dp), ("bond_chi", i32p),
                ("bond_resid_in", dp), ("bond_resid_out", dp)]


_SIGS = {
    "tn_ctx_create": (i32, [i32, C.POINTER(P)]),
    "tn_ctx_destroy": (i32, [P]),
    "tn_last_error": (C.c_char_p, [P]),
    "tn_version": (i32, []),
    "tn_kernel_launches": (i64, [P]),
    "tn_mps_upload": (i32, [P, i32, i32, i64p, dpp, i32, C.POINTER(P)]),
    "tn_mps_download": (i32, [P, P, dpp]),
    "tn_mps_bonddims": (i32, [P, P, i64p, i32p]),
    "tn_mps_copy": (i32, [P, P, C.POINTER(P)]),
    "tn_mps_destroy": (i32, [P]),
    "tn_vmps": (i32, [P, i32, C.POINTER(P), dp, C.POINTER(VmpsOpts), C.POINTER(P), dp,
                      C.POINTER(i32)]),
    "tn_mpo_apply": (i32, [P, P, P, C.POINTER(TruncOpts), C.POINTER(P)]),
    "tn_mpo_mpo_apply": (i32, [P, P, P, i32, C.POINTER(TruncOpts), C.POINTER(P)]),
    "tn_mps_scale": (i32, [P, P, dp]),
    "tn_mps_overlap": (i32, [P, P, P, dp]),
    "tn_mpo_upload": (i32, [P, i32, i32, i64p, dpp, C.POINTER(P)]),
    "tn_mpo_destroy": (i32, [P]),
    "tn_mps_movecenter": (i32, [P, P, i32, C.POINTER(TruncOpts)]),
    "tn_mps_norm": (i32, [P, P, dp]),
    "tn_mps_normalize": (i32, [P, P]),
    "tn_mps_entropy": (i32, [P, P, i32, dp]),
    "tn_mps_singular_values": (i32, [P, P, i32, dp, i64p]),
    "tn_mps_applyop": (i32, [P, P, i32, dp]),
    "tn_inner_terms": (i32, [P, P, P, i32, i32p, i32p, dp, dp, dp]),
    "tn_dmrg": (i32, [P, P, P, C.POINTER(DmrgOpts), dp, C.POINTER(DmrgStats)]),
    "tn_dmrg_sum": (i32, [P, P, i32, C.POINTER(P), dp, i32, C.POINTER(P), dp,
                          C.POINTER(DmrgOpts), dp, C.POINTER(DmrgStats)]),
    "tn_gates_upload": (i32, [P, i32, i32, i32, i32p, i32p, i32p, dpp, C.POINTER(P)]),
    "tn_gates_destroy": (i32, [P]),
    "tn_applygates": (i32, [P, P, P, C.POINTER(TruncOpts)]),
    "tn_tebd_steps": (i32, [P, P, P, i32, C.POINTER(TruncOpts), dp]),
    "tn_tebd_steps_prec": (i32, [P, P, P, i32, C.POINTER(TruncOpts), i32, dp]),
    "tn_tebd_grad": (i32, [P, P, i32, C.POINTER(P), i32, i32p, C.POINTER(TruncOpts), i32, i32, dp,
                           C.c_double, dp, dp]),
    "tn_qjmc_rates": (i32, [P, P, i32, i32p, dp, dp, dp]),
    "tn_qjmc_run": (i32, [P, P, P, i32, i32p, dp, dp, i32, f64, dp, i64, C.POINTER(TruncOpts),
                          i32, i32, i32p, dp, dp, i32p, dp, i32p, i64p, i32]),
    "tn_qjmc_batch": (i32, [P, P, P, i32, i32p, dp, dp, i32, f64, i32, dp, i64, C.c_uint64,
                            C.POINTER(TruncOpts), i32, i32, i32p, dp, dp, i32p, i32]),
    "tn_qjmc_ensemble": (i32, [P, P, P, i32, i32p, dp, dp, i32, f64, i32, dp, i64, C.c_uint64,
                               C.c_uint32, C.POINTER(TruncOpts), i32, i32, i32p, dp, dp, i32p,
                               i32, i32p, dp, i32, dp, i32]),
    "tn_philox_uniforms": (i32, [C.c_uint64, C.c_uint32, i64, dp]),
    "tn_heff2_apply": (i32, [P, i64, i64, i32, i64, i64, i64, dp, dp, dp, dp, dp, dp, i32]),
    "tn_heff2_apply_noalloc": (i32, [P, i64, i64, i32, i64, i64, i64, P, P, P, P, P, P]),
    "tn_env_left": (i32, [P, i64, i64, i32, i64, i64, dp, dp, dp, dp, i32]),
    "tn_env_right": (i32, [P, i64, i64, i32, i64, i64, dp, dp, dp, dp, i32]),
    "tn_gate2_apply": (i32, [P, i64, i64, i64, i32, dp, dp, dp, dp]),
    "tn_truncate": (i32, [P, i64, i64, dp, C.POINTER(TruncOpts), i32, dp, dp, dp, i64p]),
    "tn_gemm": (i32, [P, i64, i64, i64, dp, i32, dp, dp, i32]),
    "tn_eigh_top": (i32, [P, i64, dp, i64, dp, dp]),
    "tn_profile_enable": (i32, [P, i32]),
    "tn_profile_reset": (i32, [P]),
    "tn_profile_read": (i32, [P, i64p, dp, dp, dp]),
    "tn_profile_phases": (i32, [P, dp]),
}

PROF_CLASSES = ("tc_cgemm_kernel (tcgen05 3xTF32)", "zgemm_kernel (FP64)", "eigensolver (own FP64: tridiagonal, bisection, inverse iteration, QR, back-transform)",
                "small_apply_kernel (FP64 legs)", "heff_mid_kernel (FP32 leg)",
                "operand conversion / partial reduction", "Lanczos vector ops",
                "all launches (count only)")

EXPORTED = tuple(_SIGS)

_lib = None


def load(path=None):
    """Load libtngpu.so and declare every prototype; raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIBPATH
    if not os.path.exists(p):
        raise RuntimeError(f"libtngpu.so not built ({p}); run __graft_entry__.build()")
    lib = C.CDLL(p)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class TNError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{msg} ({TN_ERR.get(code, code)})")
        self.code = code


class Context:
    """A CUDA device context of libtngpu (one stream, one memory pool)."""

    def __init__(self, device=0):
        self.lib = load()
        h = P()
        rc = self.lib.tn_ctx_create(device, C.byref(h))
        if rc != TN_OK:
            raise TNError(rc, self.lib.tn_last_error(None).decode())
        self.h = h
        self.device = device

    def check(self, rc):
        if rc != TN_OK:
            raise TNError(rc, self.lib.tn_last_error(self.h).decode())

    def launches(self):
        return int(self.lib.tn_kernel_launches(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.tn_ctx_destroy(self.h)
            self.h = None


_default = None


def context():
    """The process-wide default context on device 0."""
    global _default
    if _default is None:
        _default = Context(0)
    return _default


def as_dp(a):
    return a.ctypes.data_as(dp)


def ptr_array(arrays):
    arr = (dp * len(arrays))(*[as_dp(a) for a in arrays])
    return arr


def cplx_f(a):
    """complex128 Fortran-ordered copy (interleaved re/im, column-major)."""
    return np.asfortranarray(np.asarray(a, dtype=np.complex128))


def trunc(cutoff=0.0, maxdim=0, mindim=1):
    return TruncOpts(float(cutoff), int(maxdim), int(mindim))
