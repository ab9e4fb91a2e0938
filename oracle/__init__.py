"""Oracle for the GCG eigensolver hot path - TEST INFRASTRUCTURE ONLY.

This package restates, on the CPU and in numpy/scipy, the reference GCGE
algorithm (GCG outer loop, BlockPCG, modified Gram-Schmidt B-orthogonalisation,
the OPS default multivector operations and the app_ccs/app_lapack backends;
the block AMG V-cycle in ``amg_oracle.py``), citing the reference file:line
each function follows.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
and reference legs may import it, and only as the checker or as the timed CPU
baseline.  The GPU library (``gcge_gb300``) never imports, links or calls
anything here.

Pinning: ``tests/golden/`` holds eigenvalues, iteration counts and
eigenvectors produced by the reference's own C sources compiled in this
repository (``oracle/ref/Makefile`` -> ``oracle/_ref/libgcge_ref.so``, built
only where the reference tree is present).  ``tests/test_oracle_cpu.py``
checks this restatement against those fixtures.
"""
