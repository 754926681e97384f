"""GB300-native SALSA microphysics step (drop-in for UCLALES-SALSA run_SALSA).

Modules:
  capi    -- ctypes mirror of include/salsa_gb300.h
  config  -- the &salsa configuration (reference defaults, measured workloads)
  layout  -- bin layout (host restatement of mo_salsa_init)
  inputs  -- seeded synthetic fields in the run_SALSA layout
  api     -- SalsaStep: the Python binding of the C-ABI
  build   -- builds csrc/ into _build/libsalsa_gb300.so for sm_103a
"""
from .config import reference_defaults, workload_config  # noqa: F401
