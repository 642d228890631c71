"""CPU FP64 oracle for the PECS drift-diffusion--Poisson time step.

TEST INFRASTRUCTURE ONLY.  This package is a plain numpy/scipy restatement of
the reference's numerics (LDG carrier systems, mixed RT x DGQ Poisson system,
IMEX time loop).  It exists to check the GPU library: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
it, and never as the thing that is measured or shipped.

Parity status: the reference (deal.II 8.4 + UMFPACK + TBB) cannot be built in
this environment and ships no golden vectors, so the oracle is pinned against
the reference's own known-answer tests instead -- the manufactured-solution
problems of ``tests/Poisson_test.cpp`` and ``tests/IMEX_LDG_test.cpp``, whose
convergence rates ``oracle.manufactured`` reproduces -- plus structural
invariants.  Against deal.II itself the parity is unpinned.
"""
from .pecs_oracle import *  # noqa: F401,F403
