"""CPU oracle for the SlabLU factor-and-solve path -- TEST INFRASTRUCTURE ONLY.

This package is a NumPy/SciPy restatement of the reference algorithm
(annayesy/slabLU, pure Python).  It exists to check the GPU product and to time
the CPU baseline.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs
of ``bench.py`` may import it.  The product package ``slablu_gb300`` never
imports it and never falls back to it.

Parity pinning: the restatement is checked against golden vectors produced by
running the reference itself (``tests/golden/make_golden.py``) -- leaf
discretisation operators, leaf DtN maps, the assembled sparse operator, the slab
partition, batched block-tridiagonal factors and end-to-end solutions.

Modules
  leaf           -- Chebyshev leaf discretisation, Aloc, DtN build/solve
                    (src_disc/hps_subdomain_disc.py, src_disc/hps_parallel_leaf_ops.py)
  domain         -- multidomain grid, face numbering, sparse assembly, slab
                    partition, black-box and two-level slab solves
                    (src_disc/hps_multidomain_disc.py, src_solver/slablu_solver.py)
  block_tridiag  -- batched block-tridiagonal LU sweeps and the interface
                    block LU (src_solver/block_tridiag_solver_dense.py,
                    src_solver/block_tridiag_solver_structured.py)
"""
