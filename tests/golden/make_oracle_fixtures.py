"""Writes oracle_outputs.json: the oracle's outputs on the explicit seeded
inputs of the parity cases, with the inputs stored beside them.

Each case carries what a run of the reference needs to reproduce it:
- the model and keywords;
- the initial site tensors (column-major, flattened, with their shapes);
- the uniform-draw stream of a QJMC trajectory.

It also carries the oracle's results:
- energies, bond dimensions and singular values for DMRG;
- <Z_i>(t), log-norms and the entropy for TEBD;
- jump channels, jump times and <Z_i> for QJMC.

The file serves two purposes.  A CPU test checks that the oracle still
reproduces it.  And a host with Julia can run the reference on the same
inputs (gmps.jl:276-291 is replaced by the stored tensors, and Random by
the stored draws) and compare with a fixed file.

Run from the repository root:  python tests/golden/make_oracle_fixtures.py
"""

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle as O  # noqa: E402


def tfim(N, J=1.0, h=0.5):
    H = O.OpList(N)
    for i in range(1, N):
        H.add(["z", "z"], [i, i + 1], -J)
    for i in range(1, N + 1):
        H.add("x", i, -h)
    return H


def xxz(N, J=1.0, delta=1.0, field=None):
    H = O.OpList(N)
    for i in range(1, N):
        H.add(["x", "x"], [i, i + 1], J)
        H.add(["y", "y"], [i, i + 1], J)
        H.add(["z", "z"], [i, i + 1], J * delta)
    if field is not None:
        for i in range(1, N + 1):
            H.add("z", i, field(i))
    return H


def zlist(N):
    Z = O.OpList(N)
    for i in range(1, N + 1):
        Z.add("z", i)
    return Z


def seeded_draws(N, D, seed):
    """randomGMPS's draws from numpy PCG64(seed), column-major fill: N real
    site tensors [Dl, 2, Dr] and the replacement first site [1, 2, min(2, D)]."""
    rng = np.random.default_rng(seed)
    shapes = [((1 if i == 0 else D), 2, (1 if i == N - 1 else D)) for i in range(N)]
    out = [O.fr(rng.standard_normal(int(np.prod(s))), s) for s in shapes]
    out.append(O.fr(rng.standard_normal(2 * min(2, D)), (1, 2, min(2, D))))
    return out


def enc(a):
    a = np.asarray(a)
    return {"shape": list(a.shape), "data": O.fr(a, (-1,)).tolist()}


def dec(e):
    return O.fr(np.asarray(e["data"], dtype=np.float64), tuple(e["shape"]))


def dmrg_case(model, N, D, seed, kw, bond):
    draws = seeded_draws(N, D, seed)
    H = tfim(N) if model == "tfim" else xxz(N)
    psi = O.random_mps(2, N, D, draws)
    _, E = O.dmrg(psi, O.mpo_from_oplist(O.spinhalf(), H), **kw)
    z = np.real(O.inner(O.spinhalf(), psi, zlist(N), psi))
    return {"model": model, "N": N, "randomMPS_bonddim": D, "keywords": kw,
            "randomMPS_draws": [enc(t) for t in draws],
            "energy_last_lanczos": float(np.real(E)), "bonddims": psi.bonddims(),
            "singular_values_bond": bond,
            "singular_values": np.sort(psi.singular_values(bond))[::-1].tolist(),
            "entropy_bond": float(psi.entropy(bond)), "z": z.tolist()}


def run_dmrg_case(c):
    H = tfim(c["N"]) if c["model"] == "tfim" else xxz(c["N"])
    psi = O.random_mps(2, c["N"], c["randomMPS_bonddim"], [dec(t) for t in c["randomMPS_draws"]])
    kw = dict(c["keywords"])
    kw["numconverges"] = float(kw["numconverges"])
    _, E = O.dmrg(psi, O.mpo_from_oplist(O.spinhalf(), H), **kw)
    z = np.real(O.inner(O.spinhalf(), psi, zlist(c["N"]), psi))
    return float(np.real(E)), psi.bonddims(), \
        np.sort(psi.singular_values(c["singular_values_bond"]))[::-1], \
        float(psi.entropy(c["singular_values_bond"])), z


def tebd_case():
    N, steps, dt = 16, 12, 0.05
    rec = run_tebd_case({"N": N, "steps": steps, "dt": dt})
    return {"model": "xxz J=1 delta=0.5, field 0.2 (-1)^i", "N": N, "steps": steps, "dt": dt,
            "start": "Neel (up on odd sites)", "keywords": {"cutoff": 1e-10, "maxdim": 12,
                                                            "evol": "real"},
            "z_per_step": rec[0], "lognorm": rec[1], "bonddims": rec[2], "entropy_mid": rec[3]}


def run_tebd_case(c):
    N, steps, dt = c["N"], c["steps"], c["dt"]
    names = ["up" if i % 2 else "dn" for i in range(1, N + 1)]
    psi = O.product_mps(O.spinhalf(), names)
    rec = {}
    O.tebd(O.spinhalf(), psi, xxz(N, 1.0, 0.5, lambda i: 0.2 * (-1) ** i), dt, steps * dt, dt,
           [zlist(N)], cutoff=1e-10, maxdim=12, evol="real", record=rec)
    z = [np.real(r[0]).tolist() for r in rec["ops"]]
    return z, [float(x) for x in rec["lognorm"]], psi.bonddims(), float(psi.entropy(N // 2))


def qjmc_case(classical):
    N, dt, steps = 8, 0.05, 40
    draws = np.random.default_rng(5).random(3 * steps + 3)
    j, t, z = run_qjmc_case({"N": N, "dt": dt, "steps": steps, "draws": draws.tolist(),
                             "classical": classical})
    return {"model": "Ising H = sum ZZ + 0.8 sum X, L_i = sqrt(0.1) s-_i", "N": N, "dt": dt,
            "steps": steps, "start": "all up", "classical": classical,
            "keywords": {"cutoff": 1e-10, "maxdim": 16}, "draws": draws.tolist(),
            "jumps": j, "jump_times": t, "z_per_step": z}


def run_qjmc_case(c):
    N, dt, steps = c["N"], c["dt"], c["steps"]
    H, L = O.OpList(N), O.OpList(N)
    for i in range(1, N):
        H.add(["z", "z"], [i, i + 1], 1.0)
    for i in range(1, N + 1):
        H.add("x", i, 0.8)
        L.add("s-", i, np.sqrt(0.1))
    psi = O.product_mps(O.spinhalf(), ["up"] * N)
    rec = {}
    j, t = O.qjmc_simulation(O.spinhalf(), psi, H, L, steps * dt, dt,
                             O.algorithms.UniformStream(np.asarray(c["draws"])), [zlist(N)],
                             cutoff=1e-10, maxdim=16, record=rec, classical=c["classical"])
    return [int(x) for x in j], [float(x) for x in t], [np.real(r[0]).tolist() for r in rec["ops"]]


def fixtures():
    cfg1 = dict(maxdim=64, cutoff=1e-10, minsweeps=5, maxsweeps=5, numconverges="Inf",
                krylovdim=8, kryloviter=2)
    xxz_kw = dict(maxdim=32, cutoff=1e-12, minsweeps=4, maxsweeps=4, numconverges="Inf",
                  krylovdim=3, kryloviter=2)
    out = {}
    for name, args in (("dmrg_tfim_N20_config1", ("tfim", 20, 4, 1, cfg1, 10)),
                       ("dmrg_xxz_N16", ("xxz", 16, 8, 2, xxz_kw, 8))):
        model, N, D, seed, kw, bond = args
        kwf = dict(kw)
        kwf["numconverges"] = float(kwf["numconverges"])
        c = dmrg_case(model, N, D, seed, kwf, bond)
        c["keywords"] = kw
        out[name] = c
    out["tebd_xxz_N16_quench"] = tebd_case()
    out["qjmc_ising_N8_classical"] = qjmc_case(True)
    out["qjmc_ising_N8_norm_based"] = qjmc_case(False)
    return out


if __name__ == "__main__":
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_outputs.json")
    with open(path, "w") as f:
        json.dump(fixtures(), f, indent=1)
    print("wrote", path)
