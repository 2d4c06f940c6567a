"""GB300-native (sm_103a, FP64) transient engine for CedarSim circuits.

The package is loaded under the module name ``cedarsim_gb300`` (its directory name
is not a Python identifier); see ``load()`` in the repository's ``__graft_entry__``.
"""
from .circuit import Circuit, Flat, Pulse, PWL, Sin  # noqa: F401
from .abi import load_library, make_opts, CedarError, STATUS_NAMES  # noqa: F401
from .api import System, Solution, Sweep, BatchResult, costs, dc, tran  # noqa: F401
from .api import ACSol, NoiseSol, ac, acdec, ac_drive, ac_last_stats, noise  # noqa: F401
from . import generators  # noqa: F401

__all__ = ["Circuit", "Flat", "Pulse", "PWL", "Sin", "System", "Solution", "Sweep", "BatchResult", "dc", "tran",
           "load_library", "make_opts", "generators", "CedarError", "STATUS_NAMES",
           "ACSol", "NoiseSol", "ac", "acdec", "ac_drive", "ac_last_stats", "noise"]
