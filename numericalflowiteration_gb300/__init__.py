"""GB300-native (sm_103a) NuFI hot path: backward characteristic trace,
f0 at the foot, v-reduction into rho, and the periodic Poisson + spline
interpolation solve, behind the C ABI in include/nufi_gb300.h."""
from .config import (Config, NufiConfigC, landau_1d, two_stream_1d, bump_on_tail_1d, landau_2d,
                     landau_3d, WORKLOADS, PREC_FP64, PREC_FP32_SPLIT)
from ._lib import Batch, Simulation, NufiError, load, plan, solve_kernels
