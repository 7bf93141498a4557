"""GB300-native shallow-water hot path of omega_playground.

Hand-written sm_103a CUDA kernels (FP64) for the TRiSK tendencies, tracer
transport / diffusion / hyperdiffusion and the RK4 / low-storage RK stage
updates on the doubly periodic planar hexagonal MPAS mesh, behind the C ABI
in include/swgpu.h.  This package is the Python mirror of the reference's
C++ classes (see shallow_water.py); the C++ mirror is cxx/omega_gpu.hpp.
"""
from .shallow_water import (AddMode, Adjoint, AdjointEnsemble, Batch, LSRKStepper,  # noqa: F401
                            HostStepper, pinned_empty,
                            MPASMesh, adjoint_batch_backward,
                            adjoint_batch_forward, adjoint_plan,
                            checkpoint_cost,
                            PlanarHexagonalMesh, RK4Stepper,
                            ShallowWaterModel, ShallowWaterParams,
                            ShallowWaterState, TimeStepper,
                            circulation_integral, energy_integral,
                            fp64_issue_rate,
                            kernel_launches, mass_integral,
                            LinearShallowWaterModel, LinearShallowWaterParams,
                            profile_enable, profile_read, sync)
from ._capi import SwgError, exported_symbols  # noqa: F401
from . import workloads  # noqa: F401

__all__ = ["AddMode", "Adjoint", "AdjointEnsemble", "Batch", "adjoint_plan", "checkpoint_cost", "HostStepper",
           "pinned_empty",
           "LinearShallowWaterModel", "LinearShallowWaterParams",
           "adjoint_batch_forward", "adjoint_batch_backward", "LSRKStepper", "MPASMesh", "PlanarHexagonalMesh",
           "RK4Stepper", "ShallowWaterModel", "ShallowWaterParams",
           "ShallowWaterState", "TimeStepper", "circulation_integral",
           "energy_integral", "fp64_issue_rate", "mass_integral", "sync", "kernel_launches",
           "profile_enable", "profile_read",
           "SwgError", "exported_symbols", "workloads"]
