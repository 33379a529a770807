"""CPU checks: the C-ABI library loads and exports every declared symbol, and
the host-side model builders (MPO assembly, Trotter gates) agree with the
oracle.  No compute call reaches the GPU here."""

import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import oracle as O
from oracle import exact as X

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tngpu.h")
LIB = os.path.join(ROOT, "tensornetworks.jl_gb300", "tngpu", "libtngpu.so")


def header_functions():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int32_t|int64_t|const char\*)\s+(tn_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def built():
    if not os.path.exists(LIB):
        import importlib.util
        spec = importlib.util.spec_from_file_location("graft_entry", os.path.join(ROOT, "__graft_entry__.py"))
        m = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(m)
        m.build()
    return LIB


def test_library_exports_every_header_symbol(built):
    lib = ctypes.CDLL(built)
    names = header_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", built], capture_output=True, text=True).stdout
    for n in names:
        assert re.search(rf"\bT {n}\b", out), f"{n} not exported as a text symbol"


def test_python_binding_covers_header(built):
    from tngpu import _lib
    assert sorted(_lib.EXPORTED) == header_functions()
    lib = _lib.load()
    assert lib.tn_version() >= 100


def test_build_targets_sm103a_only():
    import importlib.util
    spec = importlib.util.spec_from_file_location("tnbuild", os.path.join(ROOT, "tensornetworks.jl_gb300", "build.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    assert m.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def xxz(N, delta=1.0, field=None, mod=None):
    H = mod.OpList(N)
    for i in range(1, N):
        H.add(["x", "x"], [i, i + 1], 1.0)
        H.add(["y", "y"], [i, i + 1], 1.0)
        H.add(["z", "z"], [i, i + 1], delta)
    if field:
        for i in range(1, N + 1):
            H.add("z", i, field(i))
    return H


def test_host_mpo_builder_matches_oracle_operator():
    import tngpu.models as M
    N = 7
    for field in (None, lambda i: 0.2 * (-1) ** i):
        Hp = xxz(N, 0.5, field, M)
        Ho = xxz(N, 0.5, field, O)
        W = M.mpo_tensors(M.spinhalf(), Hp)
        Wo = O.mpo_from_oplist(O.spinhalf(), Ho)
        g = O.GMPS(2, 2, W)
        assert np.allclose(X.mpo_to_dense(g), X.mpo_to_dense(Wo), atol=1e-12)
        assert [t.shape[3] for t in W] == [t.shape[3] for t in Wo.tensors]


def test_host_mpo_long_range_terms():
    import tngpu.models as M
    N = 6
    Hp, Ho = M.OpList(N), O.OpList(N)
    for H in (Hp, Ho):
        H.add(["z", "x", "z"], [1, 3, 4], 0.7)
        H.add(["y", "y"], [2, 5], -0.3)
        H.add("x", 6, 1.1)
    W = M.mpo_tensors(M.spinhalf(), Hp)
    dense = X.oplist_to_dense(O.spinhalf(), Ho)
    assert np.allclose(X.mpo_to_dense(O.GMPS(2, 2, W)), dense, atol=1e-12)


def test_host_trotter_rows_match_oracle():
    import tngpu.models as M
    N = 9
    Hp = xxz(N, 0.5, lambda i: 0.2 * (-1) ** i, M)
    Ho = xxz(N, 0.5, lambda i: 0.2 * (-1) ** i, O)
    rp = M.trotter_rows(M.spinhalf(), Hp, 0.05, 2, "real")
    ro = O.trotterize(O.spinhalf(), Ho, 0.05, 2, "real")
    assert len(rp) == len(ro) == 3
    for (sp, gp), (so, go) in zip(rp, ro):
        assert sp == so
        for a, b in zip(gp, go):
            assert a.shape == b.shape and np.allclose(a, b, atol=1e-14)


def test_host_opprod_and_qjmc_heff():
    import tngpu.models as M
    import tngpu.algorithms as A
    st = M.spinhalf()
    assert st.opprod(["s+", "s-"]) == "pu"
    assert st.opprod(["x", "z"]).startswith("temp")
    N = 4
    H = M.OpList(N)
    for i in range(1, N):
        H.add(["z", "z"], [i, i + 1])
    Lj = M.OpList(N)
    for i in range(1, N + 1):
        Lj.add("s-", i, np.sqrt(0.1))
    heff, rows = A.qjmc_gates(st, H, Lj, 0.01)
    Ho, Lo = O.OpList(N), O.OpList(N)
    for i in range(1, N):
        Ho.add(["z", "z"], [i, i + 1])
    for i in range(1, N + 1):
        Lo.add("s-", i, np.sqrt(0.1))
    _, ro = O.qjmc_gates(O.spinhalf(), Ho, Lo, 0.01)
    for (sp, gp), (so, go) in zip(rows, ro):
        assert sp == so
        for a, b in zip(gp, go):
            assert np.allclose(a, b, atol=1e-14)


def test_product_path_does_not_import_oracle():
    pkg = os.path.join(ROOT, "tensornetworks.jl_gb300", "tngpu")
    for f in os.listdir(pkg):
        if f.endswith(".py"):
            assert "oracle" not in open(os.path.join(pkg, f)).read(), f


def test_mps_checkpoint_record_round_trip(tmp_path):
    """The checkpoint layout (gmps.jl:359-383 field names) survives an .npz
    round trip, and a group of another type is rejected with the reference's
    message."""
    import tngpu.mps as M
    rng = np.random.default_rng(3)
    ts = [rng.standard_normal((1, 2, 3)) + 1j * rng.standard_normal((1, 2, 3)),
          rng.standard_normal((3, 2, 1)) + 0j]
    rec = M.mps_record(ts, 2, name="state")
    path = tmp_path / "ck.npz"
    np.savez(path, **rec)
    with np.load(path, allow_pickle=False) as z:
        back, center = M.mps_from_record({k: z[k] for k in z.files}, name="state")
    assert center == 2 and len(back) == 2
    assert all(np.array_equal(a, b) for a, b in zip(ts, back))
    bad = dict(rec)
    bad["state/type"] = np.array("MPO")
    with pytest.raises(ValueError, match="does not contain MPS data"):
        M.mps_from_record(bad, name="state")


def test_philox_stream_matches_oracle():
    """tn_philox_uniforms (the seeded QJMC streams) against the oracle's
    restatement of Philox4x32-10, across seeds, trajectories and lengths."""
    from oracle.philox import trajectory_uniforms
    import tngpu as tn
    for seed in (0, 4, 2 ** 40 + 17):
        for traj in (0, 1, 1023):
            for n in (1, 7, 64):
                a = tn.philox_uniforms(seed, traj, n)
                b = trajectory_uniforms(seed, traj, n)
                assert np.array_equal(a, b)
                assert np.all((a >= 0.0) & (a < 1.0))


def test_output_index_gate_lift():
    """A gate lifted to fused MPO sites (index o + d*i) acts as the gate on
    each site's output index and as the identity on the input index
    (gatelist.jl:146-154 with rank 2), for one- and two-site gates."""
    from tngpu.algorithms import lift_to_output_index
    rng = np.random.default_rng(8)
    d = 2
    g1 = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    g2 = rng.standard_normal((d,) * 4) + 1j * rng.standard_normal((d,) * 4)
    A = rng.standard_normal((3, d, d, 4)) + 1j * rng.standard_normal((3, d, d, 4))
    # one site: [a, o, i, b] -> sum_o' g[o, o'] A[a, o', i, b]
    ref = np.einsum("po,aoib->apib", g1, A)
    L1 = lift_to_output_index(g1, d)
    Af = np.reshape(A, (3, d * d, 4), order="F")
    got = np.einsum("PQ,aQb->aPb", L1, Af)
    assert np.allclose(np.reshape(got, (3, d, d, 4), order="F"), ref)
    # two sites: theta [a, o1, i1, o2, i2, b]
    th = rng.standard_normal((3, d, d, d, d, 4)) + 1j * rng.standard_normal((3, d, d, d, d, 4))
    ref2 = np.einsum("pkql,akilmb->apiqmb", g2, th)
    L2 = lift_to_output_index(g2, d)
    thf = np.reshape(th, (3, d * d, d * d, 4), order="F")
    got2 = np.einsum("PKQL,aKLb->aPQb", L2, thf)
    assert np.allclose(np.reshape(got2, (3, d, d, d, d, 4), order="F"), ref2)


# C struct -> (ctypes mirror, Julia shim struct)
_STRUCTS = {"tn_trunc_opts": ("TruncOpts", "TruncOpts"), "tn_dmrg_opts": ("DmrgOpts", "DmrgOpts"),
            "tn_dmrg_stats": ("DmrgStats", "DmrgStats"), "tn_vmps_opts": ("VmpsOpts", "VmpsOpts")}
_JL_SIZES = {"Int32": 4, "Int64": 8, "Float64": 8}


def _header_struct_fields(name):
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), open(HEADER).read(), re.S)
    body = re.sub(r"/\*.*?\*/", "", body.group(1), flags=re.S)
    return re.findall(r"^\s*[\w\s\*]+?[\s\*](\w+)\s*;", body, re.M)


def _julia_struct_fields(name):
    src = open(os.path.join(ROOT, "tensornetworks.jl_gb300", "julia", "TensorNetworksGB300.jl")).read()
    body = re.search(r"^(?:mutable )?struct %s\n(.*?)^end" % name, src, re.S | re.M).group(1)
    return re.findall(r"^\s*(\w+)::(\w+(?:\{\w+\})?)", body, re.M)


def test_struct_layouts_match_header(tmp_path):
    """Every option/stats struct of the header: gcc's sizeof and offsetof
    equal the ctypes mirror's, and the Julia shim declares the same fields in
    the same order with types of the same sizes (C layout rules then give
    the same offsets)."""
    from tngpu import _lib as L
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "tngpu.h"', "int main(void) {"]
    fields = {s: _header_struct_fields(s) for s in _STRUCTS}
    for s, fs in fields.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (s, s))
        for f in fs:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (s, f, s, f))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)],
                   check=True)
    got = {}
    for ln in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n"):
        if ln:
            s, f, v = ln.split()
            got[(s, f)] = int(v)
    for s, (py, jl) in _STRUCTS.items():
        cls = getattr(L, py)
        assert [f for f, _ in cls._fields_] == fields[s], s
        assert ctypes.sizeof(cls) == got[(s, "size")], s
        for f in fields[s]:
            assert getattr(cls, f).offset == got[(s, f)], (s, f)
        jf = _julia_struct_fields(jl)
        assert [f for f, _ in jf] == fields[s], (jl, jf)
        for (f, t), (_, ct) in zip(jf, cls._fields_):
            size = 8 if t.startswith("Ptr") else _JL_SIZES[t]
            assert size == ctypes.sizeof(ct), (jl, f, t)


def _split_top(s):
    """Split s at commas outside (), {} and []."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def _balanced(s, i):
    """The text inside the parenthesis opening at s[i]."""
    depth = 0
    for j in range(i, len(s)):
        depth += s[j] == "("
        depth -= s[j] == ")"
        if depth == 0:
            return s[i + 1:j]
    raise ValueError("unbalanced")


def _c_kind(param):
    param = re.sub(r"/\*.*?\*/", "", param).strip()
    if "*" in param:
        return "ptr"
    for t, k in (("uint64_t", "u64"), ("int64_t", "i64"), ("uint32_t", "u32"), ("int32_t", "i32"),
                 ("double", "f64")):
        if param.startswith(t) or param.startswith("const " + t):
            return k
    raise ValueError(param)


def _jl_kind(t):
    t = t.strip()
    if t.startswith(("Ptr", "Ref", "Cstring")):
        return "ptr"
    return {"Int32": "i32", "Cint": "i32", "Int64": "i64", "UInt64": "u64", "UInt32": "u32",
            "Float64": "f64"}[t]


def _header_decls():
    hdr = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    decl = {}
    for m in re.finditer(r"^\s*(?:int32_t|int64_t|const char\*)\s+(tn_\w+)\s*\(", hdr, re.M):
        params = _balanced(hdr, m.end() - 1)
        ps = [] if params.strip() in ("", "void") else _split_top(params)
        decl[m.group(1)] = [_c_kind(p) for p in ps]
    return decl


def test_python_signatures_match_header():
    """Every ctypes signature of the Python binding has the header's
    argument count and kinds."""
    from tngpu import _lib
    kinds = {ctypes.c_int32: "i32", ctypes.c_int64: "i64", ctypes.c_uint64: "u64",
             ctypes.c_uint32: "u32", ctypes.c_double: "f64"}
    decl = _header_decls()
    for name, (_, args) in _lib._SIGS.items():
        got = []
        for a in args:
            if a in kinds:
                got.append(kinds[a])
            else:
                assert a in (ctypes.c_void_p, ctypes.c_char_p) or issubclass(a, ctypes._Pointer), \
                    (name, a)
                got.append("ptr")
        assert got == decl[name], (name, got, decl[name])


def test_julia_shim_ccalls_match_header():
    """Every ccall of the Julia shim names a header entry point and passes
    the header's number of arguments, each of the same kind (pointer, int32,
    int64, uint64, double) -- the static half of a binding check, since no
    Julia runs here."""
    decl = _header_decls()
    src = open(os.path.join(ROOT, "tensornetworks.jl_gb300", "julia", "TensorNetworksGB300.jl")).read()
    calls = list(re.finditer(r"ccall\(\(:(tn_\w+), libtngpu\),\s*[\w{}]+,\s*\(", src))
    assert len(calls) >= 25
    for m in calls:
        name = m.group(1)
        assert name in decl, name
        kinds = [_jl_kind(t) for t in _split_top(_balanced(src, m.end() - 1))]
        assert kinds == decl[name], (name, kinds, decl[name])


def test_reference_free_functions():
    """The free-function forms of the reference's accessors and OpList /
    Sitetypes functions dispatch to the objects' methods with the
    reference's 1-based indices and errors (abstractmps.jl:64-81,
    gmps.jl:121-127, oplist.jl:102-183)."""
    import tngpu as tn
    from tngpu import models as Mo

    class State:
        rank, dim = 1, 2

        def __init__(self, center):
            self.center, self.calls = center, []

        def __len__(self):
            return 4

        def bonddims(self):
            return [1, 2, 4, 2, 1]

        def maxbonddim(self):
            return 4

        def tensors(self):
            return ["t"]

        def norm(self):
            return 1.5

        def movecenter(self, idx, **kw):
            self.calls.append((idx, kw))
            self.center = idx

    s = State(1)
    assert (tn.dim(s), tn.rank(s), tn.center(s), tn.tensors(s), tn.norm(s)) == (2, 1, 1, ["t"], 1.5)
    assert [tn.bonddim(s, i) for i in (0, 1, 2, 3, 5)] == [None, 2, 4, 2, None]
    with pytest.raises(IndexError):
        tn.bonddim(s, 4)
    assert tn.maxbonddim(s) == 4 and tn.ismps(s) and not tn.ismpo(s)
    tn.truncate(s, maxdim=3)
    assert s.calls == [(4, {"maxdim": 3})]
    tn.truncate(s)
    assert s.calls[-1] == (1, {})
    s.center = 2
    with pytest.raises(ValueError, match="out of range"):
        tn.truncate(s)
    st = tn.spinhalf()
    H = tn.OpList(5)
    H.add(["z", "z"], [2, 3], 0.5)
    H.add("x", 2, 2.0)
    H.add(["x", "z"], [1, 3], 1.0)
    assert tn.siterange(H) == 3 and tn.siteindexs(H, 2) == [1, 2] and tn.siteindexs(H, 5) == []
    assert np.array_equal(tn.totensor(H, st, 2), Mo.term_tensor(st, H, 1))
    assert np.array_equal(tn.sitetensor(H, st, 2), Mo.site_tensor(st, H, 2))
    assert tn.sitetensor(H, st, 4) is None
    assert np.array_equal(tn.op(st, "s+"), st.op("s+")) and tn.dag(st, "s+") == st.dag("s+")
    assert np.array_equal(tn.state(st, "up"), st.state("up"))
    assert tn.gatesize(np.zeros((2, 2, 2, 2))) == 2 and tn.gatesize(np.zeros((2, 2))) == 1
    with pytest.raises(ValueError, match="even number of dimensions"):
        tn.gatesize(np.zeros((2, 2, 2)))


def test_product_path_fails_loudly_without_a_gpu(built):
    """No CPU fallback: where no GPU can be used, creating a context returns
    TN_ERR_CUDA with the CUDA runtime's message, and every entry into the
    product path (state upload, MPO upload, the algorithms) raises it."""
    import tngpu as tn
    from tngpu import _lib as L
    TN_ERR_CUDA = -2  # include/tngpu.h
    assert L.TN_ERR[TN_ERR_CUDA] == "CUDA error"
    lib = L.load()
    h = ctypes.c_void_p()
    rc = lib.tn_ctx_create(0, ctypes.byref(h))
    if rc == L.TN_OK:
        lib.tn_ctx_destroy(h)
        pytest.skip("a GPU is present")
    assert rc == TN_ERR_CUDA and lib.tn_last_error(None).decode()
    st = tn.spinhalf()
    H = tn.OpList(4)
    H.add(["z", "z"], [1, 2], 1.0)
    for call in (lambda: tn.productMPS(st, ["up"] * 4),
                 lambda: tn.MPO(st, H),
                 lambda: tn.randomMPS(2, 4, 2, rng=np.random.default_rng(0)),
                 lambda: tn.trotterize(st, H, 0.1)):
        with pytest.raises(tn.TNError) as e:
            call()
        assert e.value.code == TN_ERR_CUDA
