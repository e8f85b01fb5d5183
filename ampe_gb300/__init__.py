"""GB300-native implementation of AMPE's per-level implicit step (phi + c).

Public surface:
  ampe_gb300.abi        ctypes mirror of include/ampe_gb300.h structs
  ampe_gb300.configs    model / integrator parameter sets
  ampe_gb300.initial    seeded synthetic initial conditions
  ampe_gb300.stepper    ImplicitStepper (loads libampe_gb300.so on import)
  ampe_gb300.build      nvcc build of the library for sm_103a
"""
__all__ = ["abi", "configs", "initial", "calphad_db"]
