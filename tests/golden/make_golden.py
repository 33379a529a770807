"""Writes known_answers.json: exact answers, independent of the reference and
of both implementations, that pin the oracle and the GPU path.

The reference ships no golden vectors (test/runtests.jl:1-6 is an empty
testset), and Julia is not installed to run it.  These values come from
closed forms for free-fermion chains instead:

* the open transverse-field Ising chain ground energy (Jordan-Wigner
  quadratic form: Lieb, Schultz & Mattis 1961; Pfeuty 1970);
* the open XX chain, H = sum (X X + Y Y): free fermions with hopping 2.  It
  gives the ground energy (sum of the negative single-particle energies
  4 cos(k pi / (N + 1))) and the Neel-quench magnetisation
  <Z_i>(t) = 2 [U diag(n0) U^H]_ii - 1, with U = exp(-i h t).

Run from the repository root:  python tests/golden/make_golden.py
"""

import json
import os

import numpy as np
import scipy.linalg as sla


def tfim_energy(N, J, h):
    A = np.zeros((N, N))
    B = np.zeros((N, N))
    for i in range(N):
        A[i, i] = 2 * h
    for i in range(N - 1):
        A[i, i + 1] = A[i + 1, i] = -J
        B[i, i + 1] = -J
        B[i + 1, i] = J
    lam = np.linalg.svd(A - B, compute_uv=False)
    return float(-h * N + 0.5 * np.trace(A) - 0.5 * np.sum(lam))


def xx_energy(N):
    eps = 4.0 * np.cos(np.arange(1, N + 1) * np.pi / (N + 1))
    return float(np.sum(eps[eps < 0]))


def xx_neel_quench_z(N, t):
    h = 2.0 * (np.eye(N, k=1) + np.eye(N, k=-1))
    U = sla.expm(-1j * h * t)
    n0 = np.array([1.0 if i % 2 else 0.0 for i in range(1, N + 1)])
    return (2.0 * np.real(np.diag(U @ np.diag(n0) @ U.conj().T)) - 1.0).tolist()


def answers():
    return {
        "tfim_open_N20_J1_h0.5_energy": tfim_energy(20, 1.0, 0.5),
        "xx_open_N32_energy": xx_energy(32),
        "xx_open_N24_neel_t0.5_z": xx_neel_quench_z(24, 0.5),
        "xx_open_N64_neel_t0.5_z": xx_neel_quench_z(64, 0.5),
    }


if __name__ == "__main__":
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "known_answers.json")
    with open(path, "w") as f:
        json.dump(answers(), f, indent=1)
    print("wrote", path)
