"""GB300-native Schmidt-form (Gamma-Lambda) MPS trajectory engine.

A drop-in for the ``MPS<Q, C64>`` trajectory path of whooie/tensor-net: the
state lives in HBM, every bond operation (theta contraction, Jacobi SVD,
truncation, Lambda renormalisation), measurement and entropy read runs in
hand-written sm_103a kernels behind the C ABI of ``include/tn_mps.h``.
This package is the host-side mirror of the reference API over that ABI.
"""
from . import build
from ._lib import STATUS, TN_CANCELLED as STATUS_CANCELLED, TnError, lib, library_path
from . import circuits, gates, layers
from .batch import Batch
from .coev import REFERENCE_BONDS, run_coevolution, run_coevolution_files, run_coevolution_layers
from .gates import Gate, Meas, Uni
from .inputs import gen_layer, gen_trajectory, ginibre, haar_u4
from .mps import MPS, Trunc
from .serve import Server, poisson_requests, run_poisson

__all__ = ["MPS", "Trunc", "Batch", "run_coevolution", "run_coevolution_files", "run_coevolution_layers",
           "REFERENCE_BONDS", "TnError", "STATUS", "STATUS_CANCELLED", "lib", "library_path", "build", "circuits", "gates", "layers", "Gate", "Uni",
           "Meas", "gen_layer", "gen_trajectory", "ginibre", "haar_u4", "Server", "poisson_requests", "run_poisson"]
