"""CPU oracle for the ray-integration path of jdhare/turbulence_tracing.

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``, by ``__graft_entry__.smoke``
and by the CPU-baseline / reference legs of ``bench.py`` -- always as the
checker or the timed CPU reference, never by the product package.

Contents
  tto        -- ctypes front end of the C restatement (tt_oracle.c): calc_dndr,
                trilinear interpolation, per-ray RK45 (scipy controller
                semantics), histogram2d.
  restated   -- numpy restatements: ray_at_exit, init_beam, ray transfer
                matrices and filters, Rays.histogram, gaussian3D_FFT, the
                band-limited unit-variance field used by the benchmark
                workloads, Philox4x32-10 + Box-Muller.
  ref_path   -- the reference's own CPU path (scipy solve_ivp over all rays
                with one global step, RegularGridInterpolator lookups) restated
                with the current API and run across host cores the way
                example_multiprocess.py does; timed as the CPU baseline.

Parity pinning: tests/golden holds fixtures produced by importing the
reference itself (tests/golden/make_golden.py); tests/test_oracle_golden.py
checks every function above against them.
"""
