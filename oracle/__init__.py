"""Test infrastructure: CPU oracles for the path-tracing hot path.

Only tests/, __graft_entry__.smoke() and bench.py (its CPU-baseline leg and
reference arm) may use this package.  It holds
  * oracle.cpp      — the project's CPU restatement of the reference algorithm
                      (with node-visit counters, HIP/WGSL semantics, libm or
                      portable transcendentals, FP64 accumulation);
  * ref_driver.cpp  — a driver that compiles the reference's own HIP kernel
                      source unmodified for the host through oracle/shim;
  * build_oracle.py — the build recipe for both;
  * oracle_lib.py   — ctypes wrappers.
"""
