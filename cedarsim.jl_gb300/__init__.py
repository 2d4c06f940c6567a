"""GB300-native (sm_103a, FP64) transient engine for CedarSim circuits.

The package is loaded under the module name ``cedarsim_gb300`` (its directory name
is not a Python identifier); see ``load()`` in the repository's ``__graft_entry__``.
"""
from .circuit import Circuit, Flat, Pulse, PWL, Sin  # noqa: F401
from .abi import load_library, make_opts, CedarError, STATUS_NAMES  # noqa: F401
from .api import System, Solution, Batch, BatchResult, costs, dc, tran  # noqa: F401
from .sweeps import (Sweep, ProductSweep, TandemSweep, SerialSweep, CircuitSweep, ParamSim, alter,  # noqa: F401
                     sweepvars, split_axes, sweepify, find_param_ranges, nest_param_list, flatten_param_list,
                     write_csv)
from .api import ACSol, NoiseSol, ac, acdec, ac_drive, ac_last_stats, noise  # noqa: F401
from . import generators  # noqa: F401
from . import va  # noqa: F401

__all__ = ["Circuit", "Flat", "Pulse", "PWL", "Sin", "System", "Solution", "Batch", "BatchResult", "Sweep", "ProductSweep",
           "TandemSweep", "SerialSweep", "CircuitSweep", "ParamSim", "alter", "sweepvars", "split_axes", "sweepify",
           "find_param_ranges", "nest_param_list", "flatten_param_list", "write_csv", "dc", "tran",
           "load_library", "make_opts", "generators", "CedarError", "STATUS_NAMES",
           "ACSol", "NoiseSol", "ac", "acdec", "ac_drive", "ac_last_stats", "noise", "va"]
