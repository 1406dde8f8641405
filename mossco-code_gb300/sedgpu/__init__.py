"""GB300 sediment-column solver: MOSSCO's fabm_sediment right-hand side
integrated by the solver_library stepper, as sm_103a CUDA kernels behind a C
ABI (include/mossco_sed.h).

Modules: ``model`` (tracers, parameters, ColumnSet), ``synth`` (seeded
workloads), ``capi`` (ctypes binding of the C ABI), ``driver`` (host mirror
of the reference's driver and ode_solver interface), ``build`` (nvcc
recipe).
"""
from .model import (ADAPTIVE_EULER, EULER, NTR, RUNGE_KUTTA_4,  # noqa: F401
                    RUNGE_KUTTA_4_38, TRACERS, ColumnSet, DriverParams)
