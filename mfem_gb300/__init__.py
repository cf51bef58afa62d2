"""GB300-native mixed-FEM Newton timestep (tytrusty/mfem's mixed-stretch path).

The compute path is libmfem_gb300.so (hand-written sm_103a CUDA behind a C
ABI, include/mfem_gb300.h).  This package holds the host-side mirror of the
reference's interfaces: scene specs (desc), the scene-JSON schema with the
reference's factory names (scene_json), scenes and batches on the GPU (gpu)
and the serving loop (server).
"""
from . import abi  # noqa: F401

__all__ = ["abi", "gpu", "configs", "meshgen", "desc", "scene_json", "server"]
