"""CPU oracle for the StarPolymersMD MD/MPC step -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this package, and only as the checker / baseline, never as the
product path.

Two implementations live here:

* ``smpc_oracle.c`` -- a plain-C, FP64 restatement of the reference algorithm
  (star-polymers/lib/Hydrodynamics/MPC.cpp, star-polymers/lib/Box.cpp,
  star-polymers/lib/Thermostats/Thermostat_None.cpp,
  star-polymers/lib/Molecules/Potentials.h) in the reference's arithmetic
  order, built with ``-ffp-contract=off``; it travels to the GPU machine and is
  built there.
* ``refbuild/`` -- a recipe that compiles the reference's OWN sources
  (unmodified) against a project-written Eigen subset and a recording
  ``Rand.cpp`` into ``_ref/libsmpc_ref.so``. It needs the reference checkout,
  so it exists only where the reference does; it pins the restatement and
  generates the fixtures under ``tests/golden``.
"""
