"""Oracle: CPU restatement of TensorMol's BP+EE energy-and-force path.

TEST INFRASTRUCTURE ONLY. Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import anything from this package, and only
as the checker or the timed CPU baseline. The product (``tensormol_gb300``)
never imports it and has no CPU fallback.

Contents
--------
``nlist.c``       plain-C restatement of ``MolEmb.Make_NListNaive``
                  (C_API/MolEmb.cpp:1180-1251) and of the periodic image
                  construction of ``Lattice.TessLattice`` (Periodic.py:131-181).
``reference.py``  neighbour post-processing of ``ForceModifiers/Neighbors.py``,
                  the FP64 restatement of the TensorFlow graph
                  (``TFDescriptors/RawSymFunc.py`` + ``TFNetworks/
                  TFBehlerParinelloSymEE.py``) with autograd forces, central
                  finite differences, and the integrators of
                  ``Simulations/SimpleMD.py``.
``build_ref.sh``  builds the reference's own ``C_API/MolEmb.cpp`` from its
                  source tree into ``oracle/_ref/`` (only where the reference
                  tree is present) so the restatement can be pinned to it.

Pinning: the restatement is checked against golden vectors produced by the
reference's own code (MolEmb built from source, ``Neighbors.py`` imported
unchanged) and stored in ``tests/golden/``. The TensorFlow graph itself cannot
run (no TensorFlow), so the MLP/Coulomb/vdW part is pinned through the
descriptor and Jacobian cross-checks against MolEmb plus finite differences.
"""
