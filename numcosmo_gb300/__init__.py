"""numcosmo_gb300: GB300 (sm_103a) KDE/VKDE proposal engine for NumCosmo's APES sampler.

The product is the native library lib/libncg.so (C host layer + hand-written
CUDA kernels, C-ABI in include/ncg.h); this package is its Python binding and
its build recipe.
"""
from .stats_dist import (  # noqa: F401
    NcgError,
    Precision,
    RNG,
    StatsDistCV,
    StatsDistKDE,
    StatsDistKDECovType,
    StatsDistKernelGauss,
    StatsDistKernelST,
    StatsDistVKDE,
    measure_fp64_peak,
)
from .batch import Batch  # noqa: F401
from .serve import Server, poisson_arrivals, run_schedule  # noqa: F401
from . import workloads  # noqa: F401

__version__ = "0.1.0"
