/*
 * Runs the reference's own 3D patch-layout code -- meshFIM3d::InitPatches,
 * InitPatches2 and GenerateBlockNeighbors (src/core3d/cuda/meshFIM3d.cu:
 * 423-570) and, for structured inputs, GraphPartition_Square (:269-352) --
 * compiled from the reference source file, with its layout kernels executed
 * on the CPU (oracle/ref_host_launch.cpp).  Test infrastructure only: it
 * pins the product's layout arrays to the reference's.
 *
 * Inputs: the mesh, the vertex 1-ring as CSR (the TetMesh neighbour lists
 * the partition functions turn into m_xadj_d / m_adjncy_d), and either a
 * vertex partition (npart, nparts) or, with npart == NULL, the lattice side
 * and block side of GraphPartition_Square.
 */
#include <meshFIM3d.h>

#include <cstring>
#include <vector>

// METIS stand-in for Partition_METIS: the labels lsref_metis_labels set
// (nothing otherwise; the layout entry point sets the partition members)
namespace {
std::vector<int>& metis_labels() {
  static std::vector<int> v;
  return v;
}
}  // namespace
extern "C" void METIS_PartGraphKway(int* nn, int*, int*, int*, int*, int*, int*, int*, int*, int*, int* part) {
  const std::vector<int>& l = metis_labels();
  if ((int)l.size() == *nn) std::memcpy(part, l.data(), sizeof(int) * l.size());
}
extern "C" int lsref_host_launches(int* unknown);
extern "C" int lsref_host_ipermute(int* out, int n);

namespace {
struct Result {
  int nv = 0, ne = 0, nparts = 0, full = 0, largest_ele_part = 0, launches = 0;
  std::vector<int> npart, ele_permute, ele_offsets, vert_permute, vert_offsets, ele_after_permute;
  std::vector<int> mem_locations, mem_location_offsets, block_xadj, block_adjncy, vert_ipermute;
  std::vector<float> local_coords;
};
Result g_res;

template <class V>
std::vector<int> ints(const V& v) {
  return std::vector<int>(v.begin(), v.end());
}
}  // namespace

extern "C" int lsref_layout3d(int nv, const float* xyz, int ne, const int* tets, const int* ring_off,
                              const int* ring, const int* npart, int nparts, int side, int block) {
  TetMesh mesh;
  mesh.vertices.resize(nv);
  for (int v = 0; v < nv; ++v) mesh.vertices[v] = point(xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]);
  mesh.tets.resize(ne);
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < 4; ++k) mesh.tets[e][k] = tets[4 * e + k];
  mesh.neighbors.resize(nv);
  mesh.adjacenttets.resize(nv);
  for (int v = 0; v < nv; ++v) mesh.neighbors[v].assign(ring + ring_off[v], ring + ring_off[v + 1]);
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < 4; ++k) mesh.adjacenttets[tets[4 * e + k]].push_back(e);
  mesh.vertT.assign(nv, 0.f);
  meshFIM3d fim(&mesh);
  lsref_host_launches(nullptr);
  if (npart) {
    // a given partition: the members Partition_METIS fills
    fim.nparts = nparts;
    fim.npart_h = IdxVector_h(npart, npart + nv);
    std::vector<int> xadj(ring_off, ring_off + nv + 1);
    fim.m_xadj_d = IdxVector_d(xadj.begin(), xadj.end());
    fim.m_adjncy_d = IdxVector_d(ring, ring + ring_off[nv]);
  } else {
    fim.GraphPartition_Square(side, side, side, block, block, block, false);
  }
  fim.m_vertT_d = Vector_d(mesh.vertT.begin(), mesh.vertT.end());
  fim.InitPatches(false);
  // the per-copy velocity K6 copies (its values do not enter the layout)
  fim.m_cadv_global_d = Vector_d(3 * (size_t)fim.full_num_ele, 0.f);
  fim.InitPatches2();
  fim.GenerateBlockNeighbors();
  int unknown = 0;
  g_res = Result();
  g_res.launches = lsref_host_launches(&unknown);
  if (unknown) return -1;
  g_res.nv = nv;
  g_res.ne = ne;
  g_res.nparts = fim.nparts;
  g_res.full = fim.full_num_ele;
  g_res.largest_ele_part = fim.largest_ele_part;
  g_res.npart = ints(fim.npart_h);
  g_res.ele_permute = ints(fim.ele_permute);
  g_res.ele_offsets = ints(fim.m_ele_offsets_d);
  g_res.vert_permute = ints(fim.m_vert_permute_d);
  g_res.vert_offsets = ints(fim.m_vert_offsets_d);
  g_res.ele_after_permute = ints(fim.m_ele_after_permute_d);
  g_res.mem_locations = ints(fim.m_mem_locations);
  g_res.mem_location_offsets = ints(fim.m_mem_location_offsets);
  g_res.block_xadj = ints(fim.m_block_xadj_d);
  g_res.block_adjncy = ints(fim.m_block_adjncy_d);
  g_res.local_coords.assign(fim.m_ele_local_coords_d.begin(), fim.m_ele_local_coords_d.end());
  g_res.vert_ipermute.resize(nv);
  if (lsref_host_ipermute(g_res.vert_ipermute.data(), nv) != 0) return -2;
  return 0;
}

/* info: nv, ne, nparts, full, largest_ele_part, kernel launches, nadj */
extern "C" void lsref_layout3d_info(long long* info) {
  info[0] = g_res.nv;
  info[1] = g_res.ne;
  info[2] = g_res.nparts;
  info[3] = g_res.full;
  info[4] = g_res.largest_ele_part;
  info[5] = g_res.launches;
  info[6] = (long long)g_res.block_adjncy.size();
}

/* which: the product's layout selectors (0 ele_permute ... 10 vert_ipermute),
 * 11 npart; returns the element count copied, -1 for an unknown selector. */
extern "C" long long lsref_layout3d_array(int which, void* dst) {
  const std::vector<int>* v = nullptr;
  switch (which) {
    case 0: v = &g_res.ele_permute; break;
    case 1: v = &g_res.ele_offsets; break;
    case 2: v = &g_res.vert_permute; break;
    case 3: v = &g_res.vert_offsets; break;
    case 4: v = &g_res.ele_after_permute; break;
    case 5: v = &g_res.mem_locations; break;
    case 6: v = &g_res.mem_location_offsets; break;
    case 7: v = &g_res.block_xadj; break;
    case 8: v = &g_res.block_adjncy; break;
    case 9:
      if (dst) std::memcpy(dst, g_res.local_coords.data(), sizeof(float) * g_res.local_coords.size());
      return (long long)g_res.local_coords.size();
    case 10: v = &g_res.vert_ipermute; break;
    case 11: v = &g_res.npart; break;
    default: return -1;
  }
  if (dst) std::memcpy(dst, v->data(), sizeof(int) * v->size());
  return (long long)v->size();
}

/*
 * The reference's whole time-step loop, meshFIM3d::GenerateData
 * (meshFIM3d.cu:572-690): partition (GraphPartition_Square for side > 0, else
 * Partition_METIS with the given labels standing in for METIS' result),
 * layout, then per step seed search, sign capture, FIM redistance
 * (redistance3d.cu:67-274), narrowband and `inside_niter` advection updates
 * (meshFIM3d.cu:83-99).  phi0: nv floats; vel: 3 floats per element (the
 * TetMesh normals GenerateData reads as the element velocity).  history:
 * (nsteps + 1) x nv floats, row 0 = phi0 (the rows GenerateData returns).
 * Returns the number of steps run (GenerateData stops early on an empty
 * narrowband), or a negative code.
 */
extern "C" void lsref_metis_labels(const int* npart, int nv) { metis_labels().assign(npart, npart + nv); }

extern "C" int lsref_solve3d(int nv, const float* xyz, int ne, const int* tets, const int* ring_off, const int* ring,
                             const int* npart, int nparts, int side, int block, const float* phi0, const float* vel,
                             int nsteps, float dt, float bandwidth, int inside_niter, float* history) {
  TetMesh mesh;
  mesh.vertices.resize(nv);
  for (int v = 0; v < nv; ++v) mesh.vertices[v] = point(xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]);
  mesh.tets.resize(ne);
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < 4; ++k) mesh.tets[e][k] = tets[4 * e + k];
  mesh.neighbors.resize(nv);
  mesh.adjacenttets.resize(nv);
  for (int v = 0; v < nv; ++v) mesh.neighbors[v].assign(ring + ring_off[v], ring + ring_off[v + 1]);
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < 4; ++k) mesh.adjacenttets[tets[4 * e + k]].push_back(e);
  mesh.vertT.assign(phi0, phi0 + nv);
  mesh.normals.resize(ne);
  for (int e = 0; e < ne; ++e) mesh.normals[e] = point(vel[3 * e], vel[3 * e + 1], vel[3 * e + 2]);
  int part_type = 1, metis_size = 0;
  if (side <= 0) {
    // Partition_METIS makes ceil(nv / metis_size) parts: pick a size that
    // gives the caller's part count
    part_type = 0;
    metis_size = (nv + nparts - 1) / nparts;
    if ((nv + metis_size - 1) / metis_size != nparts) return -3;
    lsref_metis_labels(npart, nv);
  }
  meshFIM3d fim(&mesh);
  lsref_host_launches(nullptr);
  std::vector<std::vector<float>> ans =
      fim.GenerateData((char*)"", nsteps, dt, inside_niter, side, block, bandwidth, part_type, metis_size, false);
  int failed = 0;
  g_res.launches = lsref_host_launches(&failed);
  if (failed) return -1;
  for (size_t s = 0; s < ans.size(); ++s)
    std::memcpy(history + s * (size_t)nv, ans[s].data(), sizeof(float) * nv);
  return (int)ans.size() - 1;
}
