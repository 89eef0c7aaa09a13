/* Stand-in for the dependency's TriMesh: plain vectors only. */
#pragma once
#include <array>
#include <vector>
#include <Vec.h>
struct TriMesh {
  std::vector<point> vertices;
  std::vector<std::array<int, 3>> faces;
  std::vector<std::vector<int>> neighbors, adjacentfaces;
  std::vector<float> vertT;
  std::vector<point> normals;
  std::vector<double> radiusInscribe;
  static TriMesh* read(const char*, bool) { return 0; }
  void need_neighbors(bool = false) {}
  void need_adjacentfaces(bool = false) {}
  void need_Rinscribe() {}
};
