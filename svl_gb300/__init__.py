"""svl_gb300: GB300-native (sm_103a) time-stepping hot path of SeismoVLAB.

The product is the C-ABI library svl_gb300/lib/libsvl_gb300.so (CUDA kernels
and C++ host code, declared in include/svl_gb300.h).  This package is its
Python binding: model/load containers, the structured-grid generator, and a
mirror of the reference's Integrator interface.
"""
from ._capi import SvlError, lib, pinned_empty  # noqa: F401
from .integrators import (CentralDifference, CentralDifferenceSolve, ExtendedNewmarkBeta, NewmarkBeta,  # noqa: F401
                          StructuredCentralDifference, StructuredEnsemble)
from .model import Loads, Model, elastic_params, j2_params, ricker  # noqa: F401

__all__ = ["CentralDifference", "CentralDifferenceSolve", "ExtendedNewmarkBeta", "NewmarkBeta", "StructuredCentralDifference", "StructuredEnsemble", "Loads", "Model", "SvlError", "lib", "pinned_empty", "ricker", "elastic_params", "j2_params"]
