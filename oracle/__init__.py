"""CPU FP64 restatement of the ADSCF SCF inner loop -- TEST INFRASTRUCTURE ONLY.

This package is the oracle the CUDA library is checked against.  It restates,
routine by routine, the Fortran 90 reference (leqiao/ADSCF); every function
cites the reference file:line it follows.  Array layout is C order
``[species][z][y][x]`` which is the same linear order as the reference's
Fortran ``(x, y, z, species)``.

Parity status: the reference ships no tests, fixtures or golden vectors and
cannot be built here (no Fortran compiler, no FFTW).  The oracle is therefore
pinned by analytic known answers (constant fields, single Fourier modes,
Crank-Nicolson eigenmode decay, dense-LU cross checks) and by its own
committed fixtures; see ``tests/test_oracle_*.py``.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package.  The product path (``adscf_gb300``) never does.
"""
