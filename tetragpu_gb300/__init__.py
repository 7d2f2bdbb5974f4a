"""GB300-native (sm_103a) simplex-relation extraction and critical-point
classification for tetrahedral meshes.

The compute path is libtetragpu.so (CUDA C++ behind the C ABI in
include/tetragpu.h); this package holds its sources (csrc/), the in-tree
build, a ctypes binding and the seeded synthetic mesh generator.
"""
from ._lib import (ALL_RELATIONS, FIELD_F32, FIELD_F64, OPT_LINK_ADJACENCY, OPT_TT_VERTEX_SHARING,
                   REL, RELATIONS, Batch, Mesh, Server, TetraGPUError, export_classes,
                   batch_tuning, kernel_launch_count, load, mask_of, profile_kernel, profile_read,
                   tuning_info, version)

__all__ = ["ALL_RELATIONS", "FIELD_F32", "FIELD_F64", "OPT_LINK_ADJACENCY", "OPT_TT_VERTEX_SHARING",
           "REL", "RELATIONS", "Batch", "Mesh", "Server", "TetraGPUError", "export_classes",
           "batch_tuning", "kernel_launch_count", "load", "mask_of", "profile_kernel",
           "profile_read", "tuning_info", "version"]
