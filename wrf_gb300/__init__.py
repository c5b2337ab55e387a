"""GB300-native WRF-ARW dynamical-core large step (solve_em RK3 + acoustic
sub-steps, physics off) behind the reference's model-layer interfaces."""
from . import abi, cases  # noqa: F401
