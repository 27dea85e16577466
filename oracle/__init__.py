"""CPU oracle for the vivsim IB-LBM hot path — TEST INFRASTRUCTURE ONLY.

A NumPy restatement of the reference library (haimingz/vivsim) for the functions on
the IB-LBM time step: D2Q9/D3Q19 moments, equilibria, BGK/KBC/MRT/regularised
collisions, Guo/EDM forcing, periodic streaming, the face boundary conditions, the
immersed-boundary stencils/interpolation/spreading/multi-direct forcing and the
Newmark rigid-body update.  Every function cites the reference file:line it follows.

Precision semantics follow JAX:

* float32 inputs behave like JAX with ``jax_enable_x64`` off: every constant table is
  cast to float32 before it meets the data, Python scalars stay weakly typed;
* float64 inputs behave like JAX with ``jax_enable_x64`` on: the lattice tables that
  the reference declares as float32 (D2Q9/D3Q19 weights, the D3Q19 second-order
  projection and MRT basis) keep their float32-rounded values inside float64 math.

Pinned against golden vectors produced by running the reference's own source (see
``tests/golden/make_golden.py``); checked by ``tests/test_oracle_golden.py``.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
may import this package, and only as the checker / timed CPU baseline.  The product
path (``vivsim_gb300``) never calls it.
"""
