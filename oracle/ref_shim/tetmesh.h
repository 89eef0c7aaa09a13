/* Stand-in for the dependency's TetMesh: plain vectors only. */
#pragma once
#include <array>
#include <vector>
#include <Vec.h>
struct TetMesh {
  std::vector<point> vertices;
  std::vector<std::array<int, 4>> tets;
  std::vector<std::vector<int>> neighbors, adjacenttets;
  std::vector<float> vertT;
  std::vector<point> normals;
  void init(double*, int, int*, int, int*, int, double*, std::vector<float>, bool) {}
  void reorient() {}
  void need_neighbors(bool = false) {}
  void need_adjacenttets(bool = false) {}
};
