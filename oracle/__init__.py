"""CPU oracle for the GB300 NUFFT library -- test infrastructure only.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this package, and only as the checker.  The product path
(``jax-finufft_gb300``) never imports it and has no CPU fallback.

Contents:
  * ``direct``     -- FP64 direct NUDFT sums (types 1, 2, 3), the known-answer
                      oracle the reference's own tests use
                      (tests/ops_test.py:25-125, 494-567).
  * ``cpu_nufft``  -- CPU restatement of the fast algorithm (fold, bin, ES
                      kernel, spread/interp, FFT, deconvolve, type-3 phasing)
                      over the C code in ``nufft_oracle.c``.
  * ``build``      -- compiles ``nufft_oracle.c`` into ``oracle/_build``.

Parity status: the reference vendors FINUFFT as an empty submodule, so the
restatement is pinned against the direct-sum known answers of the reference's
tests (committed as fixtures under ``tests/golden``), not against FINUFFT's
own outputs.
"""
