"""GB300-native Ant Colony Optimization engine for the symmetric Euclidean
TSP: the reference's Colony / AntSystem / RankBasedAntSystem hot path as
sm_103a CUDA kernels behind the C ABI of include/acogpu.h."""
from ._abi import AcoParams, default_params  # noqa: F401
from .colony import AcoError, AntSystem, Batch, Colony, RankBasedAntSystem, lib  # noqa: F401
