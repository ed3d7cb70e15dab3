"""CPU oracle for the reconstruction hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, on the CPU, what ParticleHolography.jl computes on its
reconstruction hot path (``src/holofunc.jl`` and ``src/ccl.jl``).  It exists so
that the CUDA implementation can be checked against it:

* ``ref_semantics`` -- the reference's own arithmetic, step by step, in
  complex64 (Float32 square-root term, Float64 ``exp`` rounded to ComplexF32,
  cumulative transfer products, clamp / N0f8 rounding, strict ``<`` projection).
* ``fp64``          -- the exact angular-spectrum physics in complex128 and the
  seeded synthetic-hologram generator used for small parity cases.
* ``ccl``           -- the Playne-Hawick label-equivalence CCL of ``ccl.jl``
  restated in plain C (``ccl_ref.c``), compiled with gcc and loaded by ctypes.
* ``detect_ref``    -- the reference's 3-D detection bookkeeping (per-slice
  rectangles, particle neighbourhoods, Tamura depth and centre of mass), the
  checker of the end-to-end detection case below.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import this package, and only as
the checker or the timed CPU baseline.  The product path never calls it.

Parity status: pinned to the reference's own output.  The reference's
end-to-end detection test (``test/runtests.jl:153-193``) wrote
``test/data/particles.json`` (22 particles) from its cuFFT path; this oracle
run on the same inputs reproduces all 22 (same slice, x and y to one Float32
ulp), which pins its transfer functions, Gerchberg-Saxton, reconstruction and
N0f8 rounding.  The CCL row is also pinned by the reference's known answer (84
components on ``test/data/binaryparticles.png``).
"""
