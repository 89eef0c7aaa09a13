/* LevelSet.h -- C++ drop-in for the reference's `class LevelSet`
 * (src/LevelSet.h:19-67): same constructor, public fields, defaults and
 * methods, implemented over the C ABI of lsgb300.h (sources in
 * sci-solver_level-set_gb300/csrc/LevelSet.cpp, built into liblsgb300.so).
 *
 * Differences a caller sees:
 *   - triMesh_ / tetMesh_ are small structs holding what callers of the
 *     reference read from trimesh2 / TetMesh (vertices, faces or tets,
 *     vertT, normals), not the third-party mesh classes;
 *   - FIMPtr2d_ / FIMPtr3d_ are replaced by handle_ (the C ABI handle);
 *   - solveLevelSet() never calls cudaDeviceReset();
 *   - errors print the reference's message and exit(0) as the reference
 *     does, unless exitOnError_ is false, in which case std::runtime_error
 *     is thrown instead;
 *   - flags_ selects LS_REF_COMPAT / LS_FP64_FLAGGED / LS_BITEXACT, and
 *     updateKind_ LS_UPDATE_ADVECT (the reference's update) or
 *     LS_UPDATE_CURVATURE.
 */
#ifndef LSGB300_LEVELSET_H
#define LSGB300_LEVELSET_H

#include <cmath>
#include <string>
#include <vector>

#include "lsgb300.h"

/* 3-vector with the arithmetic the reference's examples use on trimesh2's
 * `point` (Vec<3,float>). */
struct point {
  float v[3];
  point() : v{0.f, 0.f, 0.f} {}
  point(float x, float y, float z) : v{x, y, z} {}
  float& operator[](int i) { return v[i]; }
  const float& operator[](int i) const { return v[i]; }
  point operator+(const point& o) const { return point(v[0] + o.v[0], v[1] + o.v[1], v[2] + o.v[2]); }
  point operator-(const point& o) const { return point(v[0] - o.v[0], v[1] - o.v[1], v[2] - o.v[2]); }
  point operator*(float s) const { return point(v[0] * s, v[1] * s, v[2] * s); }
  point operator/(float s) const { return point(v[0] / s, v[1] / s, v[2] / s); }
  /* dot product (trimesh2 spells it with the DOT macro = ^) */
  float operator^(const point& o) const { return v[0] * o.v[0] + v[1] * o.v[1] + v[2] * o.v[2]; }
  /* cross product (trimesh2 spells it with the CROSS macro = %) */
  point operator%(const point& o) const {
    return point(v[1] * o.v[2] - v[2] * o.v[1], v[2] * o.v[0] - v[0] * o.v[2], v[0] * o.v[1] - v[1] * o.v[0]);
  }
};
inline point operator*(float s, const point& p) { return p * s; }
inline float len(const point& p) { return std::sqrt(p ^ p); }
#ifndef DOT
#define DOT ^
#endif
#ifndef CROSS
#define CROSS %
#endif

struct lsgb_face {
  int v[3];
  int& operator[](int i) { return v[i]; }
  const int& operator[](int i) const { return v[i]; }
};
struct lsgb_tet {
  int v[4];
  int& operator[](int i) { return v[i]; }
  const int& operator[](int i) const { return v[i]; }
};

/* what LevelSet callers read from trimesh2's TriMesh */
struct TriMesh {
  std::vector<point> vertices;
  std::vector<lsgb_face> faces;
  std::vector<float> vertT;    /* initial values (initializeVertices) */
  std::vector<point> normals;  /* per-face velocity (initializeAdvection) */
};
/* what LevelSet callers read from TetMesh */
struct TetMesh {
  std::vector<point> vertices;
  std::vector<lsgb_tet> tets;
  std::vector<float> vertT;
  std::vector<point> normals;  /* per-tet velocity */
};

class LevelSet {
 public:
  LevelSet(bool isTriMesh, std::string fname = "../src/test/test_data/sphere_266verts.ply", bool verbose = false);
  virtual ~LevelSet();

  /* helper functions */
  std::vector<float>& getResultAtIteration(size_t i);
  size_t numIterations();
  /* result<j>.vtk for every stored iteration (meshFIM3d.cu:48-81) */
  void writeVTK();
  /* result.fld: the mesh in SCIRun's ASCII field format (meshFIM3d.cu:20-46) */
  void writeFLD();
  /* main functions */
  void initializeVertices(std::vector<float> values);
  void initializeAdvection(std::vector<point> values);
  void initializeMesh();
  void solveLevelSet();
  void printErrorGraph(std::vector<float> solution);

  /* data (src/LevelSet.h:49-66; defaults src/LevelSet.cu:4-21) */
  bool verbose_;
  std::string filename_;
  int partitionType_;
  int numSteps_;
  double timeStep_;
  int insideIterations_;
  int blockSize_;
  int sideLengths_;
  double bandwidth_;
  int metisSize_;
  bool userSetInitial_;
  bool userSetAdvection_;
  TriMesh* triMesh_;
  TetMesh* tetMesh_;
  std::vector<std::vector<float> > time_values_;
  bool isTriMesh_;

  /* additions (no counterpart in the reference) */
  ls_handle* handle_;   /* valid after solveLevelSet() */
  unsigned flags_;      /* LS_REF_COMPAT, LS_FP64_FLAGGED, LS_BITEXACT, ... */
  int updateKind_;      /* LS_UPDATE_ADVECT (default), LS_UPDATE_CURVATURE, LS_UPDATE_NONE */
  double curvCoeff_;    /* curvature coefficient */
  bool exitOnError_;    /* true: print and exit(0) like the reference; false: throw */
  ls_stats stats_;      /* work counters and timings of the last solve */

 private:
  void fail(const std::string& msg);
};

#endif
