"""GB300-native (sm_103a) NeRF hot path of jaxngp: hash-grid encoder, occupancy-grid ray marcher,
volume integrator and fused field MLP, behind volrendjax's operator API.

Submodules:
    volrendjax  drop-in ops (march_rays, integrate_rays, packbits, morton3d, ...)
    encoders    HashGridEncoder
    field       the NGP NeRF field (encoder + fused MLP)
    build       compiles libngp_gb300.so
"""
__version__ = "0.1.0"
