"""GB300 (sm_103a) implementation of Parmec's explicit DEM time step.

`parmec_gb300.parmec` holds the input commands (MATERIAL, SPHERE, ..., DEM);
`parmec_gb300.model.Model` is the scene they build; the compute runs in
libparmec_gb300.so through the C ABI declared in include/parmec_gb300.h.
"""
__version__ = "0.1.0"
