// LevelSet.cpp -- the reference's `class LevelSet` facade (src/LevelSet.cu)
// over the C ABI.  Every device step goes through ls_* calls; this file only
// keeps the reference's fields, defaults, file names and error messages.
#include "../../include/LevelSet.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <limits>
#include <sstream>
#include <stdexcept>

LevelSet::LevelSet(bool isTriMesh, std::string fname, bool verbose)
    : verbose_(verbose),
      filename_(fname),
      partitionType_(0),
      numSteps_(10),
      timeStep_(1.),
      insideIterations_(1),
      blockSize_(16),
      sideLengths_(1),
      bandwidth_(16.),
      metisSize_(16),
      userSetInitial_(false),
      userSetAdvection_(false),
      triMesh_(nullptr),
      tetMesh_(nullptr),
      isTriMesh_(isTriMesh),
      handle_(nullptr),
      flags_(0),
      updateKind_(LS_UPDATE_ADVECT),
      curvCoeff_(1.0),
      exitOnError_(true) {
  std::memset(&stats_, 0, sizeof(stats_));
}

LevelSet::~LevelSet() {
  if (handle_) ls_destroy(handle_);
  delete tetMesh_;
  delete triMesh_;
}

void LevelSet::fail(const std::string& msg) {
  std::cerr << msg << std::endl;
  if (exitOnError_) std::exit(0);
  throw std::runtime_error(msg);
}

std::vector<float>& LevelSet::getResultAtIteration(size_t i) { return time_values_.at(i); }

size_t LevelSet::numIterations() { return time_values_.size(); }

void LevelSet::initializeMesh() {
  if ((isTriMesh_ && triMesh_) || (!isTriMesh_ && tetMesh_)) return;
  ls_handle* h = nullptr;
  if (ls_create(&h, isTriMesh_ ? 1 : 0) != LS_OK) fail("File open failed!!");
  int nv = 0, ne = 0;
  if (ls_load_mesh(h, filename_.c_str()) != LS_OK) {
    std::string why = ls_last_error(h);
    ls_destroy(h);
    fail("File open failed!! (" + why + ")");
  }
  ls_get_mesh_info(h, &nv, &ne);
  const int d1 = isTriMesh_ ? 3 : 4;
  std::vector<float> xyz((size_t)nv * 3);
  std::vector<int> el((size_t)ne * d1);
  ls_get_mesh(h, xyz.data(), el.data());
  ls_destroy(h);
  std::vector<point> verts(nv);
  for (int i = 0; i < nv; ++i) verts[i] = point(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
  if (isTriMesh_) {
    triMesh_ = new TriMesh();
    triMesh_->vertices.swap(verts);
    triMesh_->faces.resize(ne);
    for (int e = 0; e < ne; ++e)
      for (int k = 0; k < 3; ++k) triMesh_->faces[e][k] = el[(size_t)e * 3 + k];
  } else {
    tetMesh_ = new TetMesh();
    tetMesh_->vertices.swap(verts);
    tetMesh_->tets.resize(ne);
    for (int e = 0; e < ne; ++e)
      for (int k = 0; k < 4; ++k) tetMesh_->tets[e][k] = el[(size_t)e * 4 + k];
  }
}

void LevelSet::initializeVertices(std::vector<float> values) {
  if (!triMesh_ && !tetMesh_) fail("You must initialize the mesh first!");
  const size_t nv = triMesh_ ? triMesh_->vertices.size() : tetMesh_->vertices.size();
  if (values.size() != nv) fail("Initialize values size does not match number of vertices!");
  if (triMesh_) triMesh_->vertT = values;
  else tetMesh_->vertT = values;
  userSetInitial_ = true;
}

void LevelSet::initializeAdvection(std::vector<point> values) {
  if (!triMesh_ && !tetMesh_) fail("You must initialize the mesh first!");
  const size_t ne = triMesh_ ? triMesh_->faces.size() : tetMesh_->tets.size();
  if (values.size() != ne) fail("Initialize advection size does not match number of elements!");
  if (triMesh_) triMesh_->normals = values;
  else tetMesh_->normals = values;
  userSetAdvection_ = true;
}

void LevelSet::solveLevelSet() {
  if ((isTriMesh_ && !triMesh_) || (!isTriMesh_ && !tetMesh_)) initializeMesh();
  if (verbose_) std::cout << "Narrowband width is " << bandwidth_ << std::endl;
  if (handle_) {
    ls_destroy(handle_);
    handle_ = nullptr;
  }
  if (ls_create(&handle_, isTriMesh_ ? 1 : 0) != LS_OK) fail("ls_create failed");
  ls_params p;
  ls_default_params(&p);
  p.num_steps = numSteps_;
  p.time_step = timeStep_;
  p.inside_iterations = insideIterations_;
  p.block_size = blockSize_;
  p.side_lengths = sideLengths_;
  p.bandwidth = bandwidth_;
  p.metis_size = metisSize_;
  p.partition_type = partitionType_;
  p.verbose = verbose_ ? 1 : 0;
  p.update_kind = updateKind_;
  p.curv_coeff = curvCoeff_;
  p.flags = flags_;
  if (ls_set_params(handle_, &p) != LS_OK) fail(std::string("bad parameters: ") + ls_last_error(handle_));

  const std::vector<point>& V = isTriMesh_ ? triMesh_->vertices : tetMesh_->vertices;
  const int d1 = isTriMesh_ ? 3 : 4;
  const int nv = (int)V.size();
  const int ne = isTriMesh_ ? (int)triMesh_->faces.size() : (int)tetMesh_->tets.size();
  std::vector<float> xyz((size_t)nv * 3);
  for (int i = 0; i < nv; ++i)
    for (int j = 0; j < 3; ++j) xyz[(size_t)i * 3 + j] = V[i][j];
  std::vector<int> el((size_t)ne * d1);
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < d1; ++k)
      el[(size_t)e * d1 + k] = isTriMesh_ ? triMesh_->faces[e][k] : tetMesh_->tets[e][k];
  if (ls_set_mesh(handle_, xyz.data(), nv, el.data(), ne) != LS_OK)
    fail(std::string("bad mesh: ") + ls_last_error(handle_));
  // initial values and velocity; when the caller set none, ls_prepare fills
  // the reference's defaults (phi0 = x - midX, velocity (rangeX/100, 0, 0) in
  // 3D and 0 in 2D, src/LevelSet.cu:178-233)
  if (userSetInitial_) {
    const std::vector<float>& T = isTriMesh_ ? triMesh_->vertT : tetMesh_->vertT;
    if (ls_set_phi(handle_, T.data()) != LS_OK) fail(ls_last_error(handle_));
  }
  if (userSetAdvection_) {
    const std::vector<point>& N = isTriMesh_ ? triMesh_->normals : tetMesh_->normals;
    std::vector<float> vel((size_t)ne * 3);
    for (int e = 0; e < ne; ++e)
      for (int j = 0; j < 3; ++j) vel[(size_t)e * 3 + j] = N[e][j];
    if (ls_set_velocity(handle_, vel.data()) != LS_OK) fail(ls_last_error(handle_));
  }
  if (ls_setup(handle_) != LS_OK) fail(std::string("setup failed: ") + ls_last_error(handle_));
  std::vector<float> hist((size_t)(numSteps_ + 1) * nv);
  int done = 0;
  const ls_status st = ls_solve(handle_, numSteps_, hist.data(), &done);
  if (st != LS_OK) fail(std::string("solve failed: ") + ls_last_error(handle_));
  time_values_.assign((size_t)done + 1, std::vector<float>(nv));
  for (int s = 0; s <= done; ++s)
    std::copy(hist.begin() + (size_t)s * nv, hist.begin() + (size_t)(s + 1) * nv, time_values_[s].begin());
  ls_get_stats(handle_, &stats_);
  if (verbose_) std::cout << "Computing time : " << stats_.ms_total << " ms" << std::endl;
}

void LevelSet::writeVTK() {
  if (!handle_) fail("call solveLevelSet first");
  for (size_t j = 0; j < time_values_.size(); ++j) {
    std::stringstream ss;
    ss << "result" << j << ".vtk";
    if (ls_write_vtk(handle_, ss.str().c_str(), time_values_[j].data()) != LS_OK) fail(ls_last_error(handle_));
  }
}

void LevelSet::writeFLD() {
  if (!triMesh_ && !tetMesh_) fail("You must initialize the mesh first!");
  FILE* f = std::fopen("result.fld", "w");
  if (!f) fail("cannot open result.fld");
  const bool tri = triMesh_ != nullptr;
  const std::vector<point>& V = tri ? triMesh_->vertices : tetMesh_->vertices;
  const size_t nv = V.size(), nt = tri ? triMesh_->faces.size() : tetMesh_->tets.size();
  const int d1 = tri ? 3 : 4;
  const char* mesh = tri ? "TriSurfMesh<TriLinearLgn<Point>>" : "TetVolMesh<TetLinearLgn<Point>>";
  const char* basis = tri ? "TriLinearLgn<Point>" : "TetLinearLgn<Point>";
  std::fprintf(f, "SCI\nASC\n2\n{@1 {GenericField<%s,ConstantBasis<float>,vector<float>> 3 {Field 3 "
                  "{PropertyManager 2 0 }\n}\n{@2 {%s 4 {Mesh 2 {PropertyManager 2 0 }\n}\n", mesh, mesh);
  std::fprintf(f, "{STLVector 2 %zu ", nv);
  for (size_t i = 0; i < nv; ++i) std::fprintf(f, "{%.12f %.12f %.12f}", V[i][0], V[i][1], V[i][2]);
  std::fprintf(f, "}\n{STLIndexVector 1 %zu 8 ", nt * d1);
  for (size_t e = 0; e < nt; ++e)
    for (int k = 0; k < d1; ++k) std::fprintf(f, "%d ", tri ? triMesh_->faces[e][k] : tetMesh_->tets[e][k]);
  std::fprintf(f, "}\n{%s  1 }\n}\n}{ConstantBasis<float>  1 }\n{STLVector 2 %zu ", basis, nt);
  for (size_t e = 0; e < nt; ++e) std::fprintf(f, " 0");
  std::fprintf(f, "}\n}\n}");
  std::fclose(f);
}

void LevelSet::printErrorGraph(std::vector<float> solution) {
  const size_t n = numIterations();
  if (n == 0 || solution.empty()) return;
  std::vector<float> rms(n);
  for (size_t i = 0; i < n; ++i) {
    const std::vector<float>& r = getResultAtIteration(i);
    double sum = 0;
    for (size_t j = 0; j < solution.size() && j < r.size(); ++j) {
      const double e = (double)solution[j] - r[j];
      sum += e * e;
    }
    rms[i] = (float)std::sqrt(sum / (double)solution.size());
  }
  int max_log = -10, min_log = 10;
  while (std::pow(10.f, (float)max_log) < rms[0]) max_log++;
  while (min_log > -30 && std::pow(10.f, (float)min_log) > rms[n - 1]) min_log--;
  std::printf("\n\nlog(Err)|\n");
  bool tick = true;
  for (int i = max_log; i >= min_log; --i) {
    if (tick) std::printf("   10^%2d|", i);
    else std::printf("        |");
    for (size_t j = 0; j < n; ++j)
      std::printf("%c", (rms[j] > std::pow(10.f, (float)i) && rms[j] < std::pow(10.f, (float)(i + 1))) ? '*' : ' ');
    std::printf("\n");
    tick = !tick;
  }
  std::printf("--------|------------------------------------------  Converged to: %.4f\n", rms[n - 1]);
  std::printf("        |1   5    10   15   20   25   30   35\n");
  std::printf("                   Iteration\n");
}
