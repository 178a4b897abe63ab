"""CPU oracle for the Bernstein DG hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline and
reference-arm legs use this package, and only as the checker or the timed CPU baseline.
The product (the CUDA library and its host package) never imports it.

Contents
  cpu.py       ctypes wrapper of bbdg_oracle.cpp: the reference's fast operators and example
               right-hand sides restated loop for loop, plus LSRK45 time stepping.
  dense.py     dense definitions the reference's own tests compare against
               (getindex of the derivative matrices, ElevationMatrix, L0 = (N+1)^2/2 E'E,
               the explicit lift chain, and M^{-1} M^f from closed-form Bernstein mass
               matrices in place of StartUpDG's quadrature-based get_bernstein_lift).
  meshdata.py  StartUpDG-style MeshData for the oracle: Fmask, coordinate-matched mapP,
               geometric factors and scaled normals, computed independently of the
               product's compact connectivity.

Pinning: the reference is Julia and neither Julia nor StartUpDG/OrdinaryDiffEq exist on
these machines, so no reference outputs can be produced. The oracle is pinned against the
reference's own known-answer tests (test/runtests.jl:7-106, restated in dense.py and in
tests/test_oracle.py), against exact rational golden vectors in tests/golden/ computed from
the reference's dense definitions, and against the mass-matrix form of the lift. Mesh,
connectivity and time integrator are parity-unpinned at the StartUpDG / OrdinaryDiffEq
boundary.
"""
