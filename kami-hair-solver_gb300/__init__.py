"""GB300-native kami-hair-solver: the per-substep incremental-potential solve.

The product is the shared library ``libkami_hair_solver.so`` built from
``csrc/`` (C ABI declared in ``include/kami_hair_solver.h``).  The Python
modules here are host-side helpers:

* ``khs_native``  -- ctypes binding mirroring the reference's ``HairSolver``
                     (blender_extension/kami_hair_solver/native.py:180-413);
* ``khs_build``   -- nvcc build of the library for sm_103a;
* ``scenes``      -- seeded synthetic scene generators for the benchmark
                     workloads;
* ``serving``     -- continuous-batching request loop over several solvers.

The directory name contains hyphens, so import these modules by putting this
directory on ``sys.path`` (``import khs_native``).
"""
