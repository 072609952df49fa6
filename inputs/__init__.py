"""inputs - seeded synthetic workloads for the tests, the benchmark and the
profiler targets. Not part of the drop-in library (grasp_gb300): in GRASP
these inputs come from rwfnestimate (screened hydrogenic orbitals),
rcsfgenerate (CSF lists) and rangular (T/V lists).

Layout:
  csrc/synth.cpp     libgraspsynth.so: Dirac hydrogenic spinors, screening,
                     synthetic CI blocks and large synthetic Hamiltonians
  grasp_synth.h      its C interface
  synth.py           Python bindings
  workloads.py       the named workloads (ne7, fe15, rk40, large, batch)
  profile_targets.py fixed command lines for the ncu captures in profiles/
"""
