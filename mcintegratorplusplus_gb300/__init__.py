"""GB300-native Monte Carlo integrator: the hot path of MCIntegrator++'s
MCI::integrate (Metropolis sampling, accumulators, estimators) as sm_103a CUDA
kernels behind the C ABI of include/mcig.h (libmcigpu.so)."""
from .mci import *  # noqa: F401,F403
from .mci import MCI, Flow, Batch, Plugin, integrate_flow, estimate, accumulate_walk, philox_block  # noqa: F401
