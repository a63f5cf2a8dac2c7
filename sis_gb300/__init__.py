"""sis_gb300: GB300 (sm_103a) engine for the force and integration hot path of
the SIS coarse-grained RNA model (Hori-Lab/SIS).

The compute path is libsisgpu.so (CUDA kernels + C ABI, include/sis_gpu.h);
this package holds its Python binding, the input readers and the synthetic
workload builders.
"""
from .model import (BD_EM, FP64, GJF2GJ, MIXED, MOLT_CIRC, MOLT_LINEAR, SEQT, Chain, ForceField, Instance, Options,
                    System)

__all__ = ["BD_EM", "FP64", "GJF2GJ", "MIXED", "MOLT_CIRC", "MOLT_LINEAR", "SEQT", "Chain", "ForceField", "Instance",
           "Options", "System", "Engine", "build"]


def __getattr__(name):
    if name == "Engine":
        from .engine import Engine

        return Engine
    raise AttributeError(name)
