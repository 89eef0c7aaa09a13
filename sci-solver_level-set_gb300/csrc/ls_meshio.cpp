// ls_meshio.cpp -- mesh readers and the VTK writer used by the LevelSet
// drop-in.  Host code, not on the time-step path.
//
//   tetgen .node/.ele   (what LevelSet::initializeMesh loads for tet meshes,
//                        src/LevelSet.cu:125-141)
//   ASCII PLY           (what it loads for triangle meshes, src/LevelSet.cu:112-123);
//                        polygons with more than three vertices are split into
//                        a triangle fan
//   legacy VTK          (the unstructured-grid file of meshFIM3d::writeVTK,
//                        src/core3d/cuda/meshFIM3d.cu:48-81; cell type 10 for
//                        tetrahedra, 5 for triangles)
#include "ls_meshio.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <fstream>
#include <utility>
#include <sstream>

namespace lsgb {

namespace {
bool ends_with(const std::string& s, const std::string& t) {
  return s.size() >= t.size() && s.compare(s.size() - t.size(), t.size(), t) == 0;
}

// next non-empty, non-comment line
bool next_line(std::istream& in, std::string& line) {
  while (std::getline(in, line)) {
    size_t h = line.find('#');
    if (h != std::string::npos) line = line.substr(0, h);
    if (line.find_first_not_of(" \t\r\n") != std::string::npos) return true;
  }
  return false;
}
}  // namespace

std::string read_tetgen(const std::string& path, std::vector<float>& xyz, std::vector<int>& tets) {
  std::string base = path;
  if (ends_with(base, ".node") || ends_with(base, ".ele")) base = base.substr(0, base.rfind('.'));
  std::ifstream fn(base + ".node"), fe(base + ".ele");
  if (!fn || !fe) return "File open failed!! (" + base + ".node/.ele)";
  std::string line;
  if (!next_line(fn, line)) return "empty .node file";
  long long np = 0;
  int dim = 0, nattr = 0, nmark = 0;
  {
    std::istringstream ss(line);
    ss >> np >> dim >> nattr >> nmark;
    if (np <= 0 || dim != 3) return "bad .node header";
  }
  xyz.assign((size_t)np * 3, 0.f);
  int first = -1;
  for (long long i = 0; i < np; ++i) {
    if (!next_line(fn, line)) return "truncated .node file";
    std::istringstream ss(line);
    long long id;
    double x, y, z;
    if (!(ss >> id >> x >> y >> z)) return "bad .node line";
    if (i == 0) first = (int)id;
    long long k = id - first;
    if (k < 0 || k >= np) return ".node index out of range";
    xyz[k * 3] = (float)x;
    xyz[k * 3 + 1] = (float)y;
    xyz[k * 3 + 2] = (float)z;
  }
  if (!next_line(fe, line)) return "empty .ele file";
  long long ne = 0;
  int npe = 0;
  {
    std::istringstream ss(line);
    ss >> ne >> npe;
    if (ne <= 0 || npe < 4) return "bad .ele header";
  }
  tets.assign((size_t)ne * 4, 0);
  for (long long e = 0; e < ne; ++e) {
    if (!next_line(fe, line)) return "truncated .ele file";
    std::istringstream ss(line);
    long long id, a[4];
    if (!(ss >> id >> a[0] >> a[1] >> a[2] >> a[3])) return "bad .ele line";
    for (int k = 0; k < 4; ++k) {
      long long v = a[k] - first;
      if (v < 0 || v >= np) return ".ele vertex index out of range";
      tets[e * 4 + k] = (int)v;
    }
  }
  return "";
}

std::string read_ply(const std::string& path, std::vector<float>& xyz, std::vector<int>& tris) {
  std::ifstream f(path);
  if (!f) return "File open failed!! (" + path + ")";
  std::string line;
  if (!std::getline(f, line) || line.compare(0, 3, "ply") != 0) return "not a PLY file";
  long long nv = -1, nf = -1;
  int nvprop = 0;
  bool in_vertex = false, ascii = false;
  while (std::getline(f, line)) {
    std::istringstream ss(line);
    std::string w;
    ss >> w;
    if (w == "format") {
      std::string fmt;
      ss >> fmt;
      ascii = (fmt == "ascii");
    } else if (w == "element") {
      std::string what;
      long long n;
      ss >> what >> n;
      in_vertex = (what == "vertex");
      if (what == "vertex") nv = n;
      else if (what == "face") nf = n;
    } else if (w == "property") {
      if (in_vertex) nvprop++;
    } else if (w == "end_header") {
      break;
    }
  }
  if (!ascii) return "only ASCII PLY is supported";
  if (nv <= 0 || nf <= 0 || nvprop < 3) return "bad PLY header";
  xyz.assign((size_t)nv * 3, 0.f);
  for (long long i = 0; i < nv; ++i) {
    if (!std::getline(f, line)) return "truncated PLY vertices";
    std::istringstream ss(line);
    double x, y, z;
    if (!(ss >> x >> y >> z)) return "bad PLY vertex";
    xyz[i * 3] = (float)x;
    xyz[i * 3 + 1] = (float)y;
    xyz[i * 3 + 2] = (float)z;
  }
  tris.clear();
  long long lo = nv, hi = -1;
  for (long long i = 0; i < nf; ++i) {
    if (!std::getline(f, line)) return "truncated PLY faces";
    std::istringstream ss(line);
    int n;
    if (!(ss >> n) || n < 3) return "bad PLY face";
    std::vector<long long> v(n);
    for (int k = 0; k < n; ++k) {
      if (!(ss >> v[k])) return "bad PLY face";
      lo = std::min(lo, v[k]);
      hi = std::max(hi, v[k]);
    }
    for (int k = 1; k + 1 < n; ++k) {
      tris.push_back((int)v[0]);
      tris.push_back((int)v[k]);
      tris.push_back((int)v[k + 1]);
    }
  }
  // Files whose face indices run 1..nv instead of 0..nv-1 (the reference's
  // own SquareMesh_size16.ply is one) are shifted down by one, as the
  // trimesh2 reader behind TriMesh::read does; any other index outside
  // 0..nv-1 is an error.
  if (lo == 1 && hi == nv) {
    for (int& t : tris) t -= 1;
  } else if (lo < 0 || hi >= nv) {
    return "PLY face index out of range";
  }
  return "";
}

int reorient_tets(const std::vector<float>& xyz, std::vector<int>& tets) {
  int flipped = 0;
  for (size_t e = 0; e + 3 < tets.size(); e += 4) {
    const float* a = &xyz[3 * (size_t)tets[e]];
    const float* b = &xyz[3 * (size_t)tets[e + 1]];
    const float* c = &xyz[3 * (size_t)tets[e + 2]];
    const float* d = &xyz[3 * (size_t)tets[e + 3]];
    const double u[3] = {(double)b[0] - a[0], (double)b[1] - a[1], (double)b[2] - a[2]};
    const double v[3] = {(double)c[0] - a[0], (double)c[1] - a[1], (double)c[2] - a[2]};
    const double w[3] = {(double)d[0] - a[0], (double)d[1] - a[1], (double)d[2] - a[2]};
    const double vol = u[0] * (v[1] * w[2] - v[2] * w[1]) - u[1] * (v[0] * w[2] - v[2] * w[0]) +
                       u[2] * (v[0] * w[1] - v[1] * w[0]);
    if (vol < 0) {
      std::swap(tets[e + 2], tets[e + 3]);
      ++flipped;
    }
  }
  return flipped;
}

std::string read_mesh(const std::string& path, bool is_tri, std::vector<float>& xyz, std::vector<int>& elems) {
  if (is_tri) return read_ply(path, xyz, elems);
  std::string r = read_tetgen(path, xyz, elems);
  if (r.empty()) reorient_tets(xyz, elems);
  return r;
}

std::string write_vtk(const std::string& path, const std::vector<float>& xyz, const std::vector<int>& elems,
                      int verts_per_elem, const float* phi) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) return "cannot open " + path;
  const size_t nv = xyz.size() / 3, ne = elems.size() / verts_per_elem;
  std::fprintf(f, "# vtk DataFile Version 3.0\nvtk output\nASCII\nDATASET UNSTRUCTURED_GRID\n");
  std::fprintf(f, "POINTS %zu float\n", nv);
  for (size_t i = 0; i < nv; ++i) std::fprintf(f, "%.12f %.12f %.12f\n", xyz[i * 3], xyz[i * 3 + 1], xyz[i * 3 + 2]);
  std::fprintf(f, "CELLS %zu %zu\n", ne, ne * (verts_per_elem + 1));
  for (size_t e = 0; e < ne; ++e) {
    std::fprintf(f, "%d", verts_per_elem);
    for (int k = 0; k < verts_per_elem; ++k) std::fprintf(f, " %d", elems[e * verts_per_elem + k]);
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "CELL_TYPES %zu\n", ne);
  const int type = verts_per_elem == 4 ? 10 : 5;
  for (size_t e = 0; e < ne; ++e) std::fprintf(f, "%d\n", type);
  std::fprintf(f, "POINT_DATA %zu\nSCALARS traveltime float 1\nLOOKUP_TABLE default\n", nv);
  for (size_t i = 0; i < nv; ++i) std::fprintf(f, "%.12f\n", phi[i]);
  std::fclose(f);
  return "";
}

}  // namespace lsgb
