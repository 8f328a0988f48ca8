"""GB300-native particle-in-cell hot path of the Entity code.

The compute path is libentity_pic.so (C ABI in include/entity_pic.h, CUDA
kernels for sm_103a); `abi` binds it with ctypes, `sim` mirrors the reference's
SR phase functions on top, `inputs` makes seeded synthetic plasmas.
"""
from . import abi  # noqa: F401
