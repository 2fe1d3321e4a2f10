// Point and octree files in the reference's formats (src/octFunctions.cpp):
//   .pts   readPtsFromFile / writePtsToFile (:319, :380): uint32 count, then
//          x y z per point in FP64;
//   text   readNodesFromFile / writeNodesToFile (:452, :496): "dim maxDepth",
//          the count, then "x y z level" per octant, one per line;
//   binary readNodesFromFile_binary / writeNodesToFile_binary (:435, :482):
//          28-byte records x y z level weight dim maxDepth (uint32 each).
// Files move through pinned staging buffers straight to or from device
// memory; octree text is formatted and parsed on the GPU.
#pragma once

#include <string>

#include "dg_octree.cuh"

namespace dg {

size_t pts_file_count(const char *path);
// reads the file's points into xyz (capacity points); returns the count
size_t pts_file_read(Context &ctx, const char *path, double *xyz, size_t capacity, bool dst_on_device);
void pts_file_write(Context &ctx, const char *path, const double *xyz, size_t n, bool src_on_device);

void octree_write_text(Context &ctx, const Octree &o, const char *path);
void octree_read_text(Context &ctx, const char *path, Octree &out);
void octree_write_binary(Context &ctx, const Octree &o, const char *path);
void octree_read_binary(Context &ctx, const char *path, Octree &out);

}  // namespace dg
