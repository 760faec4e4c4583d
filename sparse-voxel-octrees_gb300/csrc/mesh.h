// mesh.h — host-side triangle mesh as PlyLoader reads it, shared by the PLY
// reader (ply_reader.cpp) and the GPU voxelizer (voxelize.cu).
#pragma once

#include <cstdint>
#include <vector>

#include "svo_internal.h"

namespace svo {

// Vertices and fan triangles before PlyLoader::rescaleVertices: raw FP32
// positions, the file's normals when it has all of nx, ny, nz, colours with
// 255 for a missing channel (PlyLoader.cpp:128-158), and per-axis bounds
// taken with std::min / std::max from 1e30 / -1e30 (PlyLoader.cpp:160-163).
struct MeshHost {
    std::vector<float> pos;     // 3 per vertex
    std::vector<float> nrm;     // 3 per vertex, or empty
    std::vector<float> col;     // 3 per vertex
    std::vector<int32_t> tris;  // 3 vertex indices per triangle (v0, v1, v2)
    float lower[3] = {1e30f, 1e30f, 1e30f};
    float upper[3] = {-1e30f, -1e30f, -1e30f};
};

// Parses a PLY file (ascii, binary_little_endian or binary_big_endian).
int ply_read(const char *path, MeshHost &out);

// Adds one vertex (updating the bounds) / one polygon (fan-triangulated as
// PlyLoader::readTriangles does; fewer than 3 indices give no triangle).
void mesh_add_vertex(MeshHost &m, const float p[3], const float *n, const float c[3]);
int mesh_add_face(MeshHost &m, const int32_t *idx, int count, uint64_t n_vertices);

}  // namespace svo
