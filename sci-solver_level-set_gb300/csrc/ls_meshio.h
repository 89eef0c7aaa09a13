// ls_meshio.h -- mesh readers and the VTK writer (host).
#pragma once
#include <string>
#include <vector>

namespace lsgb {
// tetgen basename (or .node / .ele path): 0-based tets (4 per element)
std::string read_tetgen(const std::string& path, std::vector<float>& xyz, std::vector<int>& tets);
// ASCII PLY: triangles (3 per element, polygons fanned)
std::string read_ply(const std::string& path, std::vector<float>& xyz, std::vector<int>& tris);
// Positive orientation for every tet (TetMesh::reorient, called by
// LevelSet::initializeMesh, src/LevelSet.cu:139): a tet whose signed volume
// (b-a).((c-a)x(d-a)) is negative gets its last two vertices swapped.
// Returns the number of flipped tets.
int reorient_tets(const std::vector<float>& xyz, std::vector<int>& tets);
// read_ply for triangle handles, read_tetgen + reorient_tets for tet handles
std::string read_mesh(const std::string& path, bool is_tri, std::vector<float>& xyz, std::vector<int>& elems);
// legacy VTK unstructured grid with point scalars "traveltime"
std::string write_vtk(const std::string& path, const std::vector<float>& xyz, const std::vector<int>& elems,
                      int verts_per_elem, const float* phi);
}  // namespace lsgb
