"""CPU oracle for the MatMRI reconstruction hot path (TEST INFRASTRUCTURE ONLY).

This package restates, in FP64 numpy/scipy, the algorithms of the MatMRI
reference (fledo-dev/UWOBrainHack2026-MATMRI, pure MATLAB) for the operators
on the reconstruction hot path.  Every function cites the reference
``file:line`` it follows.

It is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it.  The product path
(``matmri_gb300``) never calls into this package and fails loudly when its
CUDA library is missing.

Parity pinning: the reference is MATLAB and cannot be executed here, and it
stores no golden vectors.  The oracle is pinned against the reference's own
known-answer tests (``@nufftOp/tests.m``, ``@sampHighOrder/tests.m``,
``@rcvrOp/tests.m``, ``mrSampFunc.m`` tests, ``powermethod.m`` unit test,
``@dwtND/tests.m``), which assert mathematical identities (adjointness,
equality with the centered FFT on Cartesian trajectories, PSF flatness,
circular-shift invariance, segmented == direct) at the reference's own
thresholds, plus an independent direct FP64 NUDFT.  ``tests/test_oracle_*``
runs those pins.
"""
