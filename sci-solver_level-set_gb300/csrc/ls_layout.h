// ls_layout.h -- patch layout of a partitioned triangle / tetrahedral mesh.
//
// The layout orders vertices and element copies exactly as GPUTUM Level-Set
// does (src/core3d/cuda/meshFIM3d.cu:423-570), so that the reference's
// layout arrays can be reproduced bit for bit, and adds the GB300 slab view:
// per patch, owned vertices [vs, ve) followed by a sorted ghost list, with
// each element copy's vertices given as 16-bit slab-local indices.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace lsgb {

// Per-vertex slots the reference's patch kernels keep (3D 32, 2D 16).
inline int ref_slot_cap(int dim) { return dim == 3 ? 32 : 16; }

struct Layout {
  int dim = 3;          // 2 = triangles, 3 = tetrahedra
  int nv = 0, ne = 0;   // vertices, elements
  int nparts = 0;
  long long full = 0;   // element copies (sum over patches)
  int lep = 0;          // largest number of element copies in a patch
  int lvp = 0;          // largest number of owned vertices in a patch
  int lgp = 0;          // largest number of ghost vertices in a patch
  int lim = 0;          // largest number of elements at one vertex
  double mean_edge = 0; // mean element edge length

  // vertex order: new id -> old id and inverse; patch ranges of new ids
  std::vector<int> vert_permute, vert_ipermute, vert_offsets;
  // copies: original element of each copy; patch ranges of copies
  std::vector<int> ele_permute, ele_offsets;
  // ghost vertices of each patch (new ids, ascending)
  std::vector<int> ghost_offsets, ghost_ids;
  // per copy: slab-local vertex indices (owned i -> i, ghost j -> nvp + j),
  // four entries per copy (the fourth is 0xffff for triangles)
  std::vector<uint16_t> conn_local;
  // per copy: global new vertex ids, (d+1) per copy
  std::vector<int> conn;
  // owned-vertex slot lists in the reference reduction order: for vertex v,
  // slots (c - es)*4 + k of copies c of its own patch, ordered by k then c
  std::vector<int> vslot_off;
  std::vector<uint16_t> vslot;
  // per copy: bit k set when corner k's slot comes after the first
  // ref_slot_cap(dim) slots of its vertex.  The reference's patch kernels
  // keep only that many slots per vertex (the fixed l_mem array of
  // redistance_kernels3d.h:303-338 and meshFIM_kernels.h:71-105; 16 in 2D):
  // a capped corner neither enters its vertex's minimum or sums nor receives
  // the vertex value.  any_capped: some corner is capped.
  std::vector<uint8_t> slot_capped;
  bool any_capped = false;
  // patch adjacency (proper CSR, sorted neighbour lists)
  std::vector<int> padj_off, padj;
  bool has_internal_edge = false;
  // permuted coordinates, SoA [3][nv]
  std::vector<float> xyz_p;
  // batches of independent meshes (merge_layouts): mesh of each patch and
  // the mean edge length of each mesh; empty for a single mesh
  std::vector<int> patch_mesh;
  std::vector<double> mesh_edge;
};

// Build the layout.  Returns an empty string on success, else the reason.
std::string build_layout(int dim, int nv, const float* xyz, int ne, const int* elems,
                         const int* npart, int nparts, Layout& L);

// Layout of the disjoint union of independently laid-out meshes: mesh k's
// vertices, elements, patches and copies follow those of meshes 0..k-1, so
// the result equals build_layout() on the union mesh with mesh k's patch
// labels offset by the patch count of the meshes before it.
std::string merge_layouts(const std::vector<const Layout*>& parts, Layout& out);

// Reference-format arrays (meshFIM3d member arrays) for bit-exact checks.
enum RefArray {
  REF_ELE_PERMUTE = 0,
  REF_ELE_OFFSETS = 1,
  REF_VERT_PERMUTE = 2,
  REF_VERT_OFFSETS = 3,
  REF_ELE_AFTER_PERMUTE = 4,
  REF_MEM_LOCATIONS = 5,
  REF_MEM_LOCATION_OFFSETS = 6,
  REF_BLOCK_XADJ = 7,
  REF_BLOCK_ADJNCY = 8,
  REF_LOCAL_COORDS = 9,
  REF_VERT_IPERMUTE = 10
};
long long ref_array_size(const Layout& L, int which);
bool ref_array_copy(const Layout& L, int which, void* dst);

// FP32 local coordinates of one tetrahedron (A,B,C,D): |AB|, AC.X, AC.Y,
// AD.X, AD.Y, AD.Z in the frame X = AB/|AB|, Z = (AB x AC)/|AB x AC|,
// Y = Z x X (src/core3d/include/meshFIM_kernels.h:448-500).
void tet_local_coords(const float P[4][3], float Lc[6]);
// Local coordinates of one triangle and its velocity projected into the
// triangle frame (src/core2d/include/meshFIM2d_kernels.h:477-520), double.
void tri_local_coords(const double P[3][3], const double vel[3], double Lc[3], double sig[2]);

}  // namespace lsgb
