"""CPU oracle for the HiQ SimulatorMPI state-vector path.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference arm of bench.py, never by the product package.

- ``sv_oracle.c`` / ``sched_oracle.c``: plain C (+OpenMP) restatements of the
  reference kernels, reductions, measurement and greedy clustering.
- ``engine.py``: a Python restatement of the reference engine's host logic
  (qubit map, gate fusion, run/measure/collapse/deallocate) over those kernels.
- ``build_ref.sh``: builds the unmodified reference modules from their sources
  into ``oracle/_ref`` where the sources are present; they pin the oracle.
"""
from .lib import load_oracle_lib, build_oracle_lib  # noqa: F401
