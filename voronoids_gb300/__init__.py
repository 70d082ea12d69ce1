"""GB300-native parallel Delaunay construction (2D/3D) with the DelaunayTree
interface of kazewong/Voronoids.  The compute path is the CUDA library
``libvoronoids_gpu.so`` (sm_103a); see include/voronoids_gpu.h."""
from .tree import DelaunayTree, Server, VDError, check_triangulation, delaunay, delaunay_batch  # noqa: F401

__all__ = ["DelaunayTree", "Server", "VDError", "check_triangulation", "delaunay", "delaunay_batch"]
