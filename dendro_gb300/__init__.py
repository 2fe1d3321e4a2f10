"""dendro_gb300: GB300-native (sm_103a) octree hot path of Dendro4.

Morton sort -> ot::points2Octree -> ot::balanceOctree(incCorner) -> ot::DA
-> Laplacian + mass element matVec, as hand-written CUDA kernels behind the
C ABI of include/dendro_gb300.h.
"""
from .api import (DA, Context, Csr, DendroError, MultiGrid, Octree, balanceOctree, coarsenOctree, completeOctree,
                  default_context, points2Octree, points2OctreeBatch, readNodesFromFile, readNodesFromFile_binary,
                  readPtsFromFile, sortOctants, sortUniquePoints, treeSort, writeNodesToFile, writeNodesToFile_binary, writePtsToFile)

__all__ = [
    "DA", "Context", "Csr", "DendroError", "MultiGrid", "Octree", "balanceOctree", "coarsenOctree", "completeOctree",
    "default_context", "points2Octree", "points2OctreeBatch",
    "sortUniquePoints", "sortOctants", "treeSort", "readPtsFromFile", "writePtsToFile", "readNodesFromFile", "writeNodesToFile",
    "readNodesFromFile_binary", "writeNodesToFile_binary",
]
