"""GB300-native implicit MPM snow substep (Stomakhin-style plasticity, matrix-free implicit
CG) behind a C ABI (include/mpm_gb300.h). The compute path is hand-written sm_103a CUDA in
csrc/; host/ holds the C++ driver surface (MPM_Driver / MPM_Example / Standard_Tests) and
the scene presets; capi.py is the ctypes binding used by the tests and the bench."""
from .capi import Context, MPMError, preset, default_scene, lib, LIB_PATH  # noqa: F401
