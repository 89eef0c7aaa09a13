/*
 * Runs the reference's host mean-curvature update
 * meshFIM3d::updateT_single_stage (src/core3d/cuda/meshFIM3d.cu:103-267),
 * compiled from the reference source file, on a caller-supplied tet mesh.
 * Built with LSREF_HOST_ONLY so that the meshFIM3d object holds host arrays
 * and needs no GPU.  Used only to pin the oracle's curvature update.
 */
#include <meshFIM3d.h>
#include <cstring>

extern "C" void METIS_PartGraphKway(int*, int*, int*, int*, int*, int*, int*, int*, int*,
                                    int*, int*) {}

/* phi is updated in place; tets lists the narrowband elements. */
extern "C" int lsref_curvature_step(int nv, const float* xyz, int ne, const int* tets,
                                    const int* nb_tets, int nnb, float dt, float* phi) {
  TetMesh mesh;
  mesh.vertices.resize(nv);
  for (int v = 0; v < nv; ++v) mesh.vertices[v] = point(xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]);
  mesh.tets.resize(ne);
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < 4; ++k) mesh.tets[e][k] = tets[4 * e + k];
  mesh.vertT.assign(phi, phi + nv);
  meshFIM3d fim(&mesh);
  std::vector<int> nb(nb_tets, nb_tets + nnb);
  fim.updateT_single_stage(dt, 0, 1, nb);
  std::memcpy(phi, mesh.vertT.data(), sizeof(float) * nv);
  return 0;
}
