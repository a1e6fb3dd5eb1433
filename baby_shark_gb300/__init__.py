"""baby_shark_gb300 — GB300 (sm_103a) implementation of baby_shark's
implicit-modelling path: mesh -> narrow-band SDF with fast-winding-number
signs, SDF booleans and offset, dual-contouring extraction.

The compute lives in libbs_gb300.so (csrc/, C ABI in include/baby_shark_gb300.h);
this package is the host-side mirror of the reference's builder API.
"""
from .api import (Context, CornerTable, DualContouringMesher, LearnedFarField, MarchingCubesMesher,  # noqa: F401
                  MeshToVolume, Volume, VolumeBuilder, VoxelRemesher, WindingNumbers, convert_batch,
                  default_context, winding_numbers_exact)
from ._native import BsError  # noqa: F401
