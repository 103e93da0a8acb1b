"""nbody_gb300: the FMM gravity step of duanebyer/nbody, rebuilt for one GB300.

The compute path is libnbody_gb300.so (hand-written sm_103a CUDA behind a C
ABI, include/nbody_gb300.h); this package is its Python host binding.
"""
from .simulation import (INTEG_EULER, INTEG_LEAPFROG, PREC_FP32, PREC_FP64, PREC_MIXED, CudaSimulation, NbodyError,
                         Particle, params)

__all__ = ["CudaSimulation", "Particle", "params", "NbodyError", "PREC_FP32", "PREC_MIXED", "PREC_FP64",
           "INTEG_LEAPFROG", "INTEG_EULER"]
