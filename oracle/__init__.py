"""CPU FP64 oracle for the finite-MPS hot path of TensorNetworks.jl.

TEST INFRASTRUCTURE ONLY.  This package is the checker: a plain numpy/scipy
restatement of the reference's algorithms (dmrg, tebd gate application, qjmc,
environment blocks, the truncated SVD rule, the MPO builder).  Only the test
suite, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may
import it.  The product (``libtngpu.so`` and the ``tngpu`` host package) never
imports or calls anything in here.

Parity status: the reference ships no golden vectors and no tests
(test/runtests.jl:1-6 is an empty testset) and Julia is not installed, so the
reference itself cannot be run to produce fixtures.  Parity with the reference
is therefore UNPINNED by reference outputs.  The oracle is instead pinned by
known-answer physics that does not depend on either code:

* transverse-field Ising open chain ground energy from the free-fermion
  (Lieb-Schultz-Mattis / Pfeuty) 2N x 2N diagonalisation,
* exact diagonalisation of small chains built term by term the way
  ``QO(st, H)`` builds the dense operator (structures/qs/qo.jl:224-242),
* untruncated TEBD against dense application of the same gates
  (structures/mps/gatelist.jl:230-255),
* QJMC trajectory averages against the Lindblad master equation.

Conventions (all column-major, complex128):
  MPS site  A[Dl, s, Dr]          (structures/mps/gmps.jl:8-13)
  MPO site  W[wl, s_out, s_in, wr] (structures/mps/mpo.jl:6-12)
  env block L[a_bra, w, b_ket]     (structures/mps/projmps.jl:50-95)
  gate      G[o1, i1, o2, i2]      (structures/mps/oplist.jl:134-156)
"""

from .core import *  # noqa: F401,F403
from .algorithms import *  # noqa: F401,F403
