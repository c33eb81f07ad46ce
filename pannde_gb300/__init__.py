"""GB300-native (sm_103a) rotated-staggered-grid elastodynamic leapfrog on hex
meshes, behind PanNDE's Model API.

The compute path is the CUDA library ``_build/libpannde_gb300.so`` reached
through the C ABI of ``include/pannde_gb300.h``; this package is its host-side
mirror (ctypes bindings, the reference-style model classes, case generators).
"""
__version__ = "0.1.0"
