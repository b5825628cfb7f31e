"""GB300-native state-vector engine with the interface of HiQ's SimulatorMPI
C++ engine (the ``_cppsim_mpi`` module behind
``hiq.projectq.backends.SimulatorMPI``).

    from hiqsimulator_gb300 import SimulatorMPI
    sim = SimulatorMPI(seed, max_local, max_cluster_size)   # same as _cppsim_mpi

The compute path is the CUDA library ``libhqs.so`` (sm_103a) built in place by
``hiqsimulator_gb300.build()``; there is no CPU fallback: importing the module
without the built extension raises ImportError.
"""
import os

from ._build import build  # noqa: F401

_PKG = os.path.dirname(os.path.abspath(__file__))

try:
    from ._cppsim_mpi import SimulatorMPI  # noqa: F401
except ImportError as e:  # pragma: no cover - exercised only without a build
    raise ImportError(
        "hiqsimulator_gb300: the CUDA extension (libhqs.so / _cppsim_mpi) is not built or cannot be "
        "loaded; run `python -c 'import __graft_entry__ as g; g.build()'` first (%s)" % (e,)
    ) from e

from . import capi  # noqa: E402,F401
from .circuits import greedy_clusters  # noqa: E402,F401

__all__ = ["SimulatorMPI", "build", "capi", "greedy_clusters"]
