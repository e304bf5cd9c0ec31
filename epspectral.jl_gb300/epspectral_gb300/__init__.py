"""Host side of the GB300 scGD0 / ladder library: the ABI mirror, grids, synthetic inputs and the
Python mirror of the reference's loop interface (`api`)."""
from .grids import ArgumentError, FrequencyGrid, graded_frequency_grid  # noqa: F401
from . import abi, synthetic  # noqa: F401
