"""tngpu: the finite-MPS hot path of TensorNetworks.jl on GB300.

The names mirror the reference's exports (src/exports.jl): ``spinhalf``,
``OpList``, ``MPO``, ``randomMPS``, ``productMPS``, ``dmrg``,
``trotterize``, ``applygates``, ``tebd``, ``qjmc_simulation``, ``inner``,
observers, the MPO algebra (``productMPO``, ``applyMPO``, ``adjoint``,
``trace``), and free-function forms of the accessors and OpList/Sitetypes
functions (``center``, ``bonddim``, ``movecenter``, ``truncate``,
``applyop``, ``sitetensor``, ``op`` ...).  Every contraction, truncation and eigensolve runs in
``libtngpu.so`` on the GPU; nothing here computes on the CPU beyond building
model inputs (operator tables, MPO tensors, 4x4 gate exponentials and their
output-index lifts) and re-laying out MPO sites for ``adjoint``.
``tngpu.autotune`` holds the trajectory engine's launch-width autotuner.
"""

from . import autotune  # noqa: F401
from ._lib import Context, TNError, context, load  # noqa: F401
from .algorithms import (GateList, QJMCActivity, QJMCEntropy, QJMCOperators, TEBDEnergy,  # noqa: F401
                         TEBDGradProblem, TEBDNorm, TEBDOperators, applygates, dmrg, qjmc_gates,
                         philox_uniforms, qjmc_ensemble, qjmc_ensemble_sharded, qjmc_simulation,
                         shard_range, tebd, tune_qjmc_width,
                         tebd_grad, trotterize, vmps)
from .models import (OpList, Sitetypes, dag, gate_exp, gatesize, mpo_tensors, op, siteindexs,  # noqa: F401
                     siterange, sitetensor, spinhalf, state, totensor, trotter_rows)
from .mps import (GMPO, GMPS, MPO, MPOHandle, MPSProjector, adjoint, applyMPO, applyop,  # noqa: F401
                  as_gmpo, bonddim, center, dim, entropy, inner, ismpo, ismps, maxbonddim,
                  movecenter, mpo_product, norm, normalize, productMPO, rank, tensors, trace,
                  truncate, mps_from_record, mps_record, overlap, productMPS, randomMPS,
                  read_mps, write_mps)
