"""pbf_cuda_gb300 — GB300-native Position Based Fluids step.

A headless drop-in for the per-frame simulation path of naeioi/PBF-CUDA's
``Simulator`` (fluids/Simulator.h:7-61): hand-written sm_103a CUDA kernels in
libpbf.so behind the C ABI of include/pbf.h, and this host-side mirror of the
reference's interface.  The directory name has a hyphen, so load it with
``importlib`` under the module name ``pbf_cuda_gb300`` (see ``load()`` in
__graft_entry__.py).
"""
from ._abi import (PBF_ERR_CAPACITY, PBF_ERR_CUDA, PBF_ERR_INVALID_ARG, PBF_ERR_NOT_READY, PBF_ERR_TIMEOUT,
                   PBF_MAX_PARTICLES, PBF_OK, EXPORTED, EXPORTED_SSF, PbfError, PbfParams, PbfSsfParams,
                   PbfSsfProfile, PbfStepProfile, PbfTuning, check, default_params, lib, lib_path)
from .simulator import Ensemble, ParticleState, Simulator
from .ssf import SSFRenderer, ssf_default_params
from . import adjoint, driver, inverse, scenes, ssf

__all__ = [
    "PBF_OK", "PBF_ERR_INVALID_ARG", "PBF_ERR_CAPACITY", "PBF_ERR_CUDA", "PBF_ERR_TIMEOUT",
    "PBF_ERR_NOT_READY", "PBF_MAX_PARTICLES", "EXPORTED", "EXPORTED_SSF", "PbfError", "PbfParams",
    "PbfSsfParams", "PbfSsfProfile", "PbfStepProfile", "PbfTuning", "check", "default_params", "lib", "lib_path",
    "Simulator", "ParticleState", "Ensemble", "SSFRenderer", "ssf_default_params", "adjoint", "driver", "inverse",
    "scenes", "ssf",
]
