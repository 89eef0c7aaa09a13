// Drop-in check: the reference's example program pattern (src/examples/
// example1.cu "center" case) written against include/LevelSet.h.
//   levelset_example <mesh> <is_tri 0|1> <nsteps> <dt> <bandwidth> <block> <out.bin>
// Writes numIterations(), nv, every stored iteration (float32), ne and the
// per-element velocity to out.bin,
// and result<j>.vtk / result.fld into the working directory.
#include <LevelSet.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <iostream>

int main(int argc, char* argv[]) {
  if (argc < 8) {
    std::fprintf(stderr, "usage: %s mesh is_tri nsteps dt bandwidth block out.bin\n", argv[0]);
    return 2;
  }
  const bool tri = std::atoi(argv[2]) != 0;
  LevelSet data(tri, argv[1], false);
  data.numSteps_ = std::atoi(argv[3]);
  data.timeStep_ = std::atof(argv[4]);
  data.bandwidth_ = std::atof(argv[5]);
  data.blockSize_ = std::atoi(argv[6]);
  data.partitionType_ = 0;
  data.exitOnError_ = false;
  data.initializeMesh();
  const std::vector<point>& V = tri ? data.triMesh_->vertices : data.tetMesh_->vertices;
  point center(0, 0, 0);
  for (size_t i = 0; i < V.size(); i++) center = center + V[i];
  center = center / static_cast<float>(V.size());
  float max = 0.;
  for (size_t i = 0; i < V.size(); i++) max = std::max(max, len(V[i] - center));
  std::vector<float> vals;
  for (size_t i = 0; i < V.size(); i++) vals.push_back(len(V[i] - center) - max / 2.f);
  std::vector<point> adv;
  const size_t ne = tri ? data.triMesh_->faces.size() : data.tetMesh_->tets.size();
  for (size_t e = 0; e < ne; e++) {
    point c(0, 0, 0);
    const int d1 = tri ? 3 : 4;
    for (int k = 0; k < d1; ++k) c = c + V[tri ? data.triMesh_->faces[e][k] : data.tetMesh_->tets[e][k]];
    point p = c / static_cast<float>(d1) - center;
    float mag = len(p) / (max / 20.f);
    adv.push_back(mag > 0 ? p / mag / mag : point(0, 0, 0));
  }
  data.initializeVertices(vals);
  data.initializeAdvection(adv);
  try {
    data.solveLevelSet();
  } catch (const std::exception& e) {
    std::fprintf(stderr, "solve failed: %s\n", e.what());
    return 1;
  }
  data.writeVTK();
  data.writeFLD();
  FILE* f = std::fopen(argv[7], "wb");
  if (!f) return 1;
  const int n = (int)data.numIterations(), nv = (int)V.size();
  std::fwrite(&n, sizeof(int), 1, f);
  std::fwrite(&nv, sizeof(int), 1, f);
  for (int i = 0; i < n; ++i) std::fwrite(data.getResultAtIteration(i).data(), sizeof(float), nv, f);
  const int nel = (int)ne;
  std::fwrite(&nel, sizeof(int), 1, f);
  for (size_t e = 0; e < ne; ++e) std::fwrite(adv[e].v, sizeof(float), 3, f);
  std::fclose(f);
  std::printf("iterations %d vertices %d visits %lld\n", n, nv, data.stats_.patch_visits);
  return 0;
}
