"""GB300-native flow right-hand side of PFFRGSolver.jl.

Host-side modules mirror the reference's layers on the path:
``lattice`` (src/Lattice), ``frequency`` (src/Frequency), ``action``
(src/Action), ``flow`` (src/Flow, on the GPU through libpffrg_gpu.so),
``launcher`` (src/Launcher: launch!, the Bogacki-Shampine loop and the
parquet iteration).  ``workloads`` builds the seeded synthetic states the
benchmarks and parity tests use.
"""
from . import action, frequency, lattice  # noqa: F401

__all__ = ["action", "frequency", "lattice", "flow", "launcher", "workloads", "build"]
