"""GB300-native two-layer finite-volume time step (LandSlide-HySEA scheme)."""
from ._abi import VARS, LshParams, default_params  # noqa: F401
