"""gpjax_gb300: GPJax's exact- and sparse-GP hot path on GB300 (sm_103a).

Module names follow the reference package (gpjax/__init__.py): kernels,
objectives, gps, likelihoods, mean_functions, linalg, distributions,
variational_families, Dataset.  All arithmetic runs in libgpk.so (CUDA,
sm_103a) through its C ABI (include/gpk.h).
"""
from . import (computations, config, distributions, fit, gps, kernels, likelihoods, linalg,
               mean_functions, objectives, parameters, variational_families)
from ._lib import GPKError
from .dataset import Dataset

__version__ = "0.1.0"

__all__ = ["Dataset", "GPKError", "computations", "config", "distributions", "fit", "gps",
           "kernels",
           "likelihoods", "linalg", "mean_functions", "objectives", "parameters",
           "variational_families"]
