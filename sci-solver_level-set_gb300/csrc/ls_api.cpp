// ls_api.cpp -- C ABI (include/lsgb300.h) over the layout builder and the
// device solver.  Mirrors the call sequence of LevelSet (src/LevelSet.cu):
// create -> mesh -> phi / velocity -> solve -> results, with status codes in
// place of the reference's exit(0) on bad input.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/lsgb300.h"
#include "ls_layout.h"
#include "ls_meshio.h"
#include "ls_mlp.h"
#include "ls_partition.h"
#include "ls_solver.h"

struct ls_handle {
  int is_tri = 0;
  ls_params prm;
  std::vector<float> xyz;
  std::vector<int> elems;
  int nv = 0, ne = 0;
  std::vector<int> npart;
  int nparts = 0;
  bool user_partition = false;  // npart came from ls_set_partition
  std::vector<float> phi;
  std::vector<float> vel;
  bool have_phi = false, have_vel = false;
  std::unique_ptr<lsgb::Layout> layout;
  std::unique_ptr<lsgb::Solver> solver;
  std::string err;
};

// A batch of independent meshes stepped together (no counterpart in the
// reference): the members' layouts are merged into one patch set, so every
// FIM iteration, narrowband and update pass covers all meshes at once.
struct ls_batch {
  struct Member {
    lsgb::Layout layout;
    std::vector<float> phi, vel;
    ls_params prm;
    int nv = 0, ne = 0;
    // the member's mesh and partition inputs, kept so that the batch
    // autotuner can lay the member out again with another patch size
    std::vector<float> xyz;
    std::vector<int> elems;
    std::vector<int> npart;  // the caller's partition (user_partition)
    int nparts = 0;
    bool user_partition = false;
  };
  std::vector<Member> members;
  int is_tri = -1;
  std::vector<int> vbase;  // first vertex of each member in the merged numbering
  std::unique_ptr<lsgb::Layout> layout;
  std::unique_ptr<lsgb::Solver> solver;
  std::vector<float> stage;
  std::string err;
};

namespace {
ls_status fail(ls_handle* h, ls_status s, const std::string& msg) {
  if (h) h->err = msg;
  return s;
}

ls_status solver_status(ls_handle* h, const std::string& msg) {
  if (msg.empty()) return LS_OK;
  h->err = msg;
  switch (h->solver ? h->solver->status_code() : 4) {
    case 2: return LS_PATCH_TOO_LARGE;
    case 3: return LS_DEVICE_TIMEOUT;
    default: return LS_CUDA_ERROR;
  }
}

// Recursive coordinate bisection: split the longest extent at the median
// until each part holds at most `target` vertices.
void rcb(const float* xyz, std::vector<int>& idx, int lo, int hi, int nparts, int first, int* npart) {
  if (nparts <= 1 || hi - lo <= 1) {
    for (int i = lo; i < hi; ++i) npart[idx[i]] = first;
    return;
  }
  float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int i = lo; i < hi; ++i)
    for (int j = 0; j < 3; ++j) {
      mn[j] = std::min(mn[j], xyz[(size_t)idx[i] * 3 + j]);
      mx[j] = std::max(mx[j], xyz[(size_t)idx[i] * 3 + j]);
    }
  int ax = 0;
  for (int j = 1; j < 3; ++j)
    if (mx[j] - mn[j] > mx[ax] - mn[ax]) ax = j;
  const int left = nparts / 2;
  const int mid = lo + (int)((long long)(hi - lo) * left / nparts);
  std::nth_element(idx.begin() + lo, idx.begin() + mid, idx.begin() + hi, [&](int a, int b) {
    float xa = xyz[(size_t)a * 3 + ax], xb = xyz[(size_t)b * 3 + ax];
    return xa < xb || (xa == xb && a < b);
  });
  rcb(xyz, idx, lo, mid, left, first, npart);
  rcb(xyz, idx, mid, hi, nparts - left, first + left, npart);
}

void fill_stats(const lsgb::SolverStats& t, ls_stats* s) {
  s->steps_run = (int)t.steps_run;
  s->fim_iters = t.fim_iters;
  s->patch_visits = t.patch_visits;
  s->check_visits = t.check_visits;
  s->nb_vertex_updates = t.nb_vertex_updates;
  s->nb_patch_vertices = t.nb_patch_vertices;
  s->nb_patches = t.nb_patches;
  s->flagged_copies = t.flagged_copies;
  s->ms_total = t.ms_total;
  s->ms_sweep = t.ms_sweep; s->ms_check = t.ms_check; s->ms_schedule = t.ms_schedule;
  s->ms_seed = t.ms_seed; s->ms_narrowband = t.ms_narrowband; s->ms_update = t.ms_update;
  s->n_sweep = t.n_sweep; s->n_check = t.n_check; s->n_schedule = t.n_schedule;
  s->n_seed = t.n_seed; s->n_narrowband = t.n_narrowband; s->n_update = t.n_update;
  s->sweep_slab_bytes = t.sweep_slab_bytes;
  s->kernel_launches = t.kernel_launches;
  s->warm_vertices = t.warm_vertices;
  s->unsupported_resets = t.unsupported_resets;
  s->support_rounds = t.support_rounds;
  s->moved_vertices = t.moved_vertices;
  s->learned_fallbacks = t.learned_fallbacks;
  s->pairs_collected = t.pairs_collected;
  s->early_visits = t.early_visits;
}

// Solver configuration from a handle's parameters.
lsgb::SolverConfig solver_config(const ls_params& p) {
  lsgb::SolverConfig cfg;
  cfg.update_kind = p.update_kind;
  cfg.ref_compat = (p.flags & LS_REF_COMPAT) ? 1 : 0;
  cfg.fp64_flagged = (p.flags & LS_FP64_FLAGGED) ? 1 : 0;
  cfg.profile = (p.flags & LS_PROFILE) ? 1 : 0;
  cfg.use_graph = (p.flags & LS_NO_GRAPH) ? 0 : 1;
  cfg.bit_exact = (p.flags & LS_BITEXACT) ? 1 : 0;
  cfg.host_staging = (p.flags & LS_HOST_STAGING) ? 1 : 0;
  cfg.persistent = (p.flags & LS_PERSISTENT) ? 1 : 0;
  cfg.spin_limit = p.barrier_wait_limit != 0 ? (p.barrier_wait_limit > 0 ? p.barrier_wait_limit : -1) : (1 << 22);
  cfg.niter = p.fim_sweeps;
  cfg.inside_niter = p.inside_iterations > 0 ? p.inside_iterations : 1;
  cfg.max_fim_iters = p.max_fim_iters > 0 ? p.max_fim_iters : 100000;
  cfg.graph_chunk = p.graph_chunk > 0 ? p.graph_chunk : 4;
  cfg.fim_ctas = p.fim_ctas_per_sm > 0 ? p.fim_ctas_per_sm : 5;
  cfg.dt = p.time_step;
  cfg.bandwidth = p.bandwidth;
  cfg.curv_coeff = p.curv_coeff;
  cfg.smallnum = p.smallnum > 0 ? p.smallnum : 1e-5;
  cfg.largenum = p.largenum > 0 ? p.largenum : 1e9;
  cfg.length_scale = p.length_scale;
  if (p.fp64_threshold > 0) cfg.fp64_tau = p.fp64_threshold;
  return cfg;
}
}  // namespace

extern "C" {

const char* ls_version(void) { return "lsgb300 1.0 (sm_103a)"; }

ls_status ls_default_params(ls_params* p) {
  if (!p) return LS_BAD_INPUT;
  std::memset(p, 0, sizeof(*p));
  p->num_steps = 10;
  p->time_step = 1.0;
  p->inside_iterations = 1;
  p->block_size = 16;
  p->side_lengths = 1;
  p->bandwidth = 16.0;
  p->metis_size = 16;
  p->partition_type = 0;
  p->verbose = 0;
  p->update_kind = LS_UPDATE_ADVECT;
  p->curv_coeff = 1.0;
  p->flags = 0;
  p->fim_sweeps = 0;
  p->max_fim_iters = 100000;
  p->smallnum = 1e-5;
  p->largenum = 1e9;
  p->length_scale = 0.0;
  p->fp64_threshold = 3.814697265625e-06;
  p->graph_chunk = 4;
  p->fim_ctas_per_sm = 5;
  p->barrier_wait_limit = 0;
  return LS_OK;
}

ls_status ls_create(ls_handle** h, int is_tri) {
  if (!h) return LS_BAD_INPUT;
  ls_handle* x = new (std::nothrow) ls_handle();
  if (!x) return LS_NO_MEMORY;
  x->is_tri = is_tri ? 1 : 0;
  ls_default_params(&x->prm);
  *h = x;
  return LS_OK;
}

ls_status ls_destroy(ls_handle* h) {
  delete h;
  return LS_OK;
}

const char* ls_last_error(ls_handle* h) { return h ? h->err.c_str() : "null handle"; }

ls_status ls_set_params(ls_handle* h, const ls_params* p) {
  if (!h || !p) return LS_BAD_INPUT;
  if (p->inside_iterations < 0 || p->bandwidth < 0 || p->update_kind < 0 || p->update_kind > 2)
    return fail(h, LS_BAD_INPUT, "invalid parameter");
  h->prm = *p;
  h->solver.reset();  // parameters are baked into the device setup
  return LS_OK;
}

ls_status ls_get_params(ls_handle* h, ls_params* p) {
  if (!h || !p) return LS_BAD_INPUT;
  *p = h->prm;
  return LS_OK;
}

ls_status ls_set_mesh(ls_handle* h, const float* xyz, int nv, const int* elems, int ne) {
  if (!h) return LS_BAD_INPUT;
  if (!xyz || !elems || nv <= 0 || ne <= 0) return fail(h, LS_BAD_INPUT, "empty mesh");
  const int d1 = h->is_tri ? 3 : 4;
  for (long long i = 0; i < (long long)ne * d1; ++i)
    if (elems[i] < 0 || elems[i] >= nv) return fail(h, LS_BAD_INPUT, "element vertex index out of range");
  h->xyz.assign(xyz, xyz + (size_t)nv * 3);
  h->elems.assign(elems, elems + (size_t)ne * d1);
  h->nv = nv;
  h->ne = ne;
  h->npart.clear();
  h->nparts = 0;
  h->user_partition = false;
  h->have_phi = h->have_vel = false;
  h->layout.reset();
  h->solver.reset();
  return LS_OK;
}

ls_status ls_load_mesh(ls_handle* h, const char* filename) {
  if (!h || !filename) return LS_BAD_INPUT;
  std::vector<float> xyz;
  std::vector<int> el;
  std::string r = lsgb::read_mesh(filename, h->is_tri != 0, xyz, el);
  if (!r.empty()) return fail(h, LS_BAD_INPUT, r);
  const int d1 = h->is_tri ? 3 : 4;
  return ls_set_mesh(h, xyz.data(), (int)(xyz.size() / 3), el.data(), (int)(el.size() / d1));
}

ls_status ls_get_mesh_info(ls_handle* h, int* nv, int* ne) {
  if (!h || !nv || !ne) return LS_BAD_INPUT;
  *nv = h->nv;
  *ne = h->ne;
  return LS_OK;
}

ls_status ls_get_mesh(ls_handle* h, float* xyz, int* elems) {
  if (!h) return LS_BAD_INPUT;
  if (xyz) std::memcpy(xyz, h->xyz.data(), sizeof(float) * h->xyz.size());
  if (elems) std::memcpy(elems, h->elems.data(), sizeof(int) * h->elems.size());
  return LS_OK;
}

ls_status ls_write_vtk(ls_handle* h, const char* path, const float* phi) {
  if (!h || !path || !phi) return LS_BAD_INPUT;
  if (h->nv == 0) return fail(h, LS_BAD_INPUT, "no mesh");
  std::string r = lsgb::write_vtk(path, h->xyz, h->elems, h->is_tri ? 3 : 4, phi);
  if (!r.empty()) return fail(h, LS_BAD_INPUT, r);
  return LS_OK;
}

ls_status ls_set_partition(ls_handle* h, const int* npart, int nparts) {
  if (!h) return LS_BAD_INPUT;
  if (h->nv == 0) return fail(h, LS_BAD_INPUT, "set the mesh first");
  if (!npart || nparts <= 0) return fail(h, LS_BAD_INPUT, "empty partition");
  for (int v = 0; v < h->nv; ++v)
    if (npart[v] < 0 || npart[v] >= nparts) return fail(h, LS_BAD_INPUT, "partition label out of range");
  h->npart.assign(npart, npart + h->nv);
  h->nparts = nparts;
  h->user_partition = true;
  h->layout.reset();
  h->solver.reset();
  return LS_OK;
}

ls_status ls_set_phi(ls_handle* h, const float* phi) {
  if (!h) return LS_BAD_INPUT;
  if (h->nv == 0) return fail(h, LS_BAD_INPUT, "You must initialize the mesh first!");
  if (!phi) return fail(h, LS_BAD_INPUT, "null phi");
  h->phi.assign(phi, phi + h->nv);
  h->have_phi = true;
  if (h->solver) return solver_status(h, h->solver->set_phi(phi));
  return LS_OK;
}

ls_status ls_set_velocity(ls_handle* h, const float* vel) {
  if (!h) return LS_BAD_INPUT;
  if (h->nv == 0) return fail(h, LS_BAD_INPUT, "You must initialize the mesh first!");
  if (!vel) return fail(h, LS_BAD_INPUT, "null velocity");
  h->vel.assign(vel, vel + (size_t)h->ne * 3);
  h->have_vel = true;
  h->solver.reset();
  return LS_OK;
}

ls_status ls_partition_structured(int dim, int nside, int block, int nv, int* npart, int* nparts) {
  if ((dim != 2 && dim != 3) || nside <= 0 || block <= 0 || !npart || !nparts) return LS_BAD_INPUT;
  const long long expect = dim == 3 ? (long long)nside * nside * nside : (long long)nside * nside;
  if (expect != nv) return LS_BAD_INPUT;
  const int nb = (nside + block - 1) / block;
  if (dim == 3) {
    for (int k = 0; k < nside; ++k)
      for (int i = 0; i < nside; ++i)
        for (int j = 0; j < nside; ++j)
          npart[(size_t)k * nside * nside + (size_t)i * nside + j] = (k / block) * nb * nb + (i / block) * nb + (j / block);
    *nparts = nb * nb * nb;
  } else {
    for (int i = 0; i < nside; ++i)
      for (int j = 0; j < nside; ++j) npart[(size_t)i * nside + j] = (i / block) * nb + (j / block);
    *nparts = nb * nb;
  }
  return LS_OK;
}

ls_status ls_partition_graph(int dim, const int* elems, int ne, int nv, int target, int* npart, int* nparts) {
  if ((dim != 2 && dim != 3) || !elems || ne <= 0 || nv <= 0 || target <= 0 || !npart || !nparts)
    return LS_BAD_INPUT;
  const int d1 = dim + 1;
  for (long long i = 0; i < (long long)ne * d1; ++i)
    if (elems[i] < 0 || elems[i] >= nv) return LS_BAD_INPUT;
  int np = dim == 3 ? (int)std::ceil((double)nv / target) : std::max(2, nv / target);
  np = std::max(1, std::min(np, nv));
  *nparts = lsgb::partition_graph(nv, elems, ne, d1, np, npart);
  return LS_OK;
}

ls_status ls_edge_cut(int dim, const int* elems, int ne, int nv, const int* npart, long long* cut) {
  if ((dim != 2 && dim != 3) || !elems || ne <= 0 || nv <= 0 || !npart || !cut) return LS_BAD_INPUT;
  *cut = lsgb::edge_cut(nv, elems, ne, dim + 1, npart);
  return LS_OK;
}

ls_status ls_partition_rcb(int dim, const float* xyz, int nv, int target, int* npart, int* nparts) {
  if ((dim != 2 && dim != 3) || !xyz || nv <= 0 || target <= 0 || !npart || !nparts) return LS_BAD_INPUT;
  int np = dim == 3 ? (int)std::ceil((double)nv / target) : std::max(2, nv / target);
  np = std::max(1, std::min(np, nv));
  std::vector<int> idx(nv);
  std::iota(idx.begin(), idx.end(), 0);
  rcb(xyz, idx, 0, nv, np, 0, npart);
  *nparts = np;
  return LS_OK;
}

ls_status ls_prepare(ls_handle* h) {
  if (!h) return LS_BAD_INPUT;
  if (h->nv == 0) return fail(h, LS_BAD_INPUT, "You must initialize the mesh first!");
  const int dim = h->is_tri ? 2 : 3;
  if (h->npart.empty()) {
    h->npart.resize(h->nv);
    ls_status s;
    if (h->prm.partition_type == 1)
      s = ls_partition_structured(dim, h->prm.side_lengths, h->prm.block_size, h->nv, h->npart.data(), &h->nparts);
    else if (h->prm.partition_type == 2)
      s = ls_partition_rcb(dim, h->xyz.data(), h->nv, h->prm.metis_size, h->npart.data(), &h->nparts);
    else  // the reference's METIS path: a graph partition of metis_size-vertex patches
      s = ls_partition_graph(dim, h->elems.data(), h->ne, h->nv, h->prm.metis_size, h->npart.data(), &h->nparts);
    if (s != LS_OK) {
      h->npart.clear();
      return fail(h, s, "partitioning failed (structured partition needs side_lengths^dim vertices)");
    }
  }
  if (!h->have_phi) {
    // LevelSet.cu:194-199 / 228-233: phi0 = x - midX
    float mn = INFINITY, mx = -INFINITY;
    for (int v = 0; v < h->nv; ++v) {
      mn = std::min(mn, h->xyz[(size_t)v * 3]);
      mx = std::max(mx, h->xyz[(size_t)v * 3]);
    }
    const double mid = ((double)mn + (double)mx) / 2.0;
    h->phi.resize(h->nv);
    for (int v = 0; v < h->nv; ++v) h->phi[v] = (float)(h->xyz[(size_t)v * 3] - mid);
    h->have_phi = true;
  }
  if (!h->have_vel) {
    // LevelSet.cu:187-192 / 221-226: 3D (rangeX/100, 0, 0), 2D zero
    float mn = INFINITY, mx = -INFINITY;
    for (int v = 0; v < h->nv; ++v) {
      mn = std::min(mn, h->xyz[(size_t)v * 3]);
      mx = std::max(mx, h->xyz[(size_t)v * 3]);
    }
    const float vx = h->is_tri ? 0.f : (float)(((double)mx - mn) / 100.0);
    h->vel.assign((size_t)h->ne * 3, 0.f);
    for (int e = 0; e < h->ne; ++e) h->vel[(size_t)e * 3] = vx;
    h->have_vel = true;
  }
  if (!h->layout) {
    auto L = std::make_unique<lsgb::Layout>();
    std::string r = lsgb::build_layout(dim, h->nv, h->xyz.data(), h->ne, h->elems.data(), h->npart.data(),
                                       h->nparts, *L);
    if (!r.empty()) return fail(h, LS_BAD_INPUT, r);
    if (L->lep > 1024) return fail(h, LS_PATCH_TOO_LARGE, "Error: largest_ele_part > 1024");
    h->layout = std::move(L);
  }
  return LS_OK;
}

ls_status ls_setup(ls_handle* h) {
  ls_status ps = ls_prepare(h);
  if (ps != LS_OK) return ps;
  lsgb::SolverConfig cfg = solver_config(h->prm);
  h->solver = std::make_unique<lsgb::Solver>();
  std::string r = h->solver->init(*h->layout, cfg, h->vel.data());
  if (!r.empty()) {
    ls_status s = solver_status(h, r);
    h->solver.reset();
    return s;
  }
  return solver_status(h, h->solver->set_phi(h->phi.data()));
}

ls_status ls_solve(ls_handle* h, int nsteps, float* history, int* steps_done) {
  if (!h) return LS_BAD_INPUT;
  if (!h->solver) return fail(h, LS_NOT_READY, "call ls_setup first");
  if (nsteps < 0) return fail(h, LS_BAD_INPUT, "negative step count");
  return solver_status(h, h->solver->run(nsteps, history, steps_done));
}

ls_status ls_step(ls_handle* h, int nsteps, int* steps_done) { return ls_solve(h, nsteps, nullptr, steps_done); }

ls_status ls_step_host(ls_handle* h, const float* phi_in, float* phi_out) {
  if (!h) return LS_BAD_INPUT;
  if (!h->solver) return fail(h, LS_NOT_READY, "call ls_setup first");
  if (!phi_in || !phi_out) return fail(h, LS_BAD_INPUT, "null buffer");
  return solver_status(h, h->solver->step_host(phi_in, phi_out));
}

ls_status ls_eikonal(ls_handle* h, const int* seeds, const float* values, int nseeds, float* dist) {
  if (!h || !dist || nseeds < 0 || (nseeds > 0 && (!seeds || !values))) return LS_BAD_INPUT;
  if (!h->solver) return fail(h, LS_NOT_READY, "call ls_setup first");
  for (int i = 0; i < nseeds; ++i)
    if (seeds[i] < 0 || seeds[i] >= h->nv || !(values[i] >= 0.f)) return fail(h, LS_BAD_INPUT, "bad seed");
  return solver_status(h, h->solver->eikonal(seeds, values, nseeds, dist));
}

ls_status ls_get_phi(ls_handle* h, float* phi) {
  if (!h || !phi) return LS_BAD_INPUT;
  if (!h->solver) return fail(h, LS_NOT_READY, "call ls_setup first");
  return solver_status(h, h->solver->get_phi(phi));
}

ls_status ls_get_stats(ls_handle* h, ls_stats* s) {
  if (!h || !s) return LS_BAD_INPUT;
  std::memset(s, 0, sizeof(*s));
  if (!h->solver) return LS_OK;
  lsgb::SolverStats t;
  h->solver->stats(t);
  fill_stats(t, s);
  return LS_OK;
}

ls_status ls_set_profile(ls_handle* h, int on) {
  if (!h) return LS_BAD_INPUT;
  if (!h->solver) return fail(h, LS_NOT_READY, "call ls_setup first");
  h->solver->set_profile(on != 0);
  return LS_OK;
}

ls_status ls_reset_stats(ls_handle* h) {
  if (!h) return LS_BAD_INPUT;
  if (h->solver) h->solver->reset_stats();
  return LS_OK;
}

ls_status ls_get_launch_log(ls_handle* h, int cap, int* kinds, double* ms, long long* bytes, int* n) {
  if (!h || !n || cap < 0) return LS_BAD_INPUT;
  *n = 0;
  if (!h->solver) return LS_OK;
  const std::vector<lsgb::LaunchRec>& log = h->solver->launch_log();
  *n = (int)log.size();
  const int k = std::min(cap, *n);
  for (int i = 0; i < k; ++i) {
    if (kinds) kinds[i] = log[i].kind;
    if (ms) ms[i] = log[i].ms;
    if (bytes) bytes[i] = log[i].bytes;
  }
  return LS_OK;
}

ls_status ls_get_narrowband(ls_handle* h, unsigned char* flags) {
  if (!h || !flags) return LS_BAD_INPUT;
  if (!h->solver) return fail(h, LS_NOT_READY, "call ls_setup first");
  return solver_status(h, h->solver->narrowband(flags));
}

ls_status ls_debug_active(ls_handle* h, int* list, int cap, int* count, float* dt) {
  if (!h || !count) return LS_BAD_INPUT;
  if (!h->solver) return fail(h, LS_NOT_READY, "call ls_setup first");
  std::vector<int> v;
  std::string r = h->solver->active_patches(v);
  if (!r.empty()) return solver_status(h, r);
  *count = (int)v.size();
  if (list)
    for (int i = 0; i < (int)v.size() && i < cap; ++i) list[i] = v[i];
  if (dt) return solver_status(h, h->solver->dt_values(dt));
  return LS_OK;
}

ls_status ls_autotune(ls_handle* h, int trial_steps, ls_tune_report* rep) {
  if (!h) return LS_BAD_INPUT;
  if (h->nv == 0) return fail(h, LS_BAD_INPUT, "You must initialize the mesh first!");
  if (trial_steps <= 0) trial_steps = 2;
  // patch-size candidates: structured block side, or RCB target size
  std::vector<int> sizes;
  const bool structured = h->prm.partition_type == 1;
  if (h->user_partition) sizes.push_back(0);
  else if (structured) sizes = (h->is_tri ? std::vector<int>{4, 5, 6, 8} : std::vector<int>{2, 3, 4});
  else sizes = (h->is_tri ? std::vector<int>{16, 25, 36, 64} : std::vector<int>{8, 16, 27, 32, 64});
  // 2-4: one element copy per thread; 5, 6: two per thread; 7: the
  // two-copies kernel with one copy per thread (tetrahedra only)
  const std::vector<int> ctas = h->is_tri ? std::vector<int>{2, 3, 4} : std::vector<int>{2, 3, 4, 5, 6, 7};
  const ls_params saved = h->prm;
  struct Trial { int size, ctas; double ms, rate; };
  std::vector<Trial> trials;
  const std::vector<float> phi0 = h->phi;
  const bool had_phi = h->have_phi;
  for (int sz : sizes) {
    if (sz > 0) {
      if (structured) h->prm.block_size = sz;
      else h->prm.metis_size = sz;
      h->npart.clear();
      h->layout.reset();
      h->solver.reset();
    }
    ls_status s = ls_prepare(h);
    if (s == LS_PATCH_TOO_LARGE) continue;
    if (s != LS_OK) { h->prm = saved; return s; }
    // CTAs per SM only matter for patches of up to 384 element copies
    const std::vector<int> cs = h->layout->lep <= 384 ? ctas : std::vector<int>{saved.fim_ctas_per_sm};
    for (int nc : cs) {
      h->prm.fim_ctas_per_sm = nc;
      h->prm.flags &= ~(unsigned)LS_PROFILE;
      s = ls_setup(h);
      if (s == LS_PATCH_TOO_LARGE) break;
      if (s != LS_OK) { h->prm = saved; return s; }
      int done = 0;
      std::string r = h->solver->run(1, nullptr, &done);  // warm-up (graph upload, caches)
      if (!r.empty()) { h->prm = saved; return solver_status(h, r); }
      h->solver->reset_stats();
      r = h->solver->run(trial_steps, nullptr, &done);
      if (!r.empty()) { h->prm = saved; return solver_status(h, r); }
      lsgb::SolverStats t;
      h->solver->stats(t);
      const double ms = done > 0 ? t.ms_total / done : 0.0;
      const double rate = t.ms_total > 0 ? (double)t.nb_vertex_updates / (t.ms_total / 1000.0) : 0.0;
      trials.push_back({sz, nc, ms, rate});
      h->phi = phi0;
      h->have_phi = had_phi;
    }
  }
  if (trials.empty()) { h->prm = saved; return fail(h, LS_PATCH_TOO_LARGE, "no candidate fits"); }
  int best = 0;
  for (int i = 1; i < (int)trials.size(); ++i)
    if (trials[i].rate > trials[best].rate) best = i;
  // leave the handle set up with the best candidate, phi back at phi0
  h->prm = saved;
  if (trials[best].size > 0) {
    if (structured) h->prm.block_size = trials[best].size;
    else h->prm.metis_size = trials[best].size;
    h->npart.clear();
    h->layout.reset();
  }
  h->prm.fim_ctas_per_sm = trials[best].ctas;
  h->solver.reset();
  ls_status s = ls_setup(h);
  if (rep) {
    std::memset(rep, 0, sizeof(*rep));
    rep->ntrials = std::min((int)trials.size(), LS_TUNE_MAX_TRIALS);
    for (int i = 0; i < rep->ntrials; ++i) {
      rep->trials[i].patch_size = trials[i].size;
      rep->trials[i].fim_ctas_per_sm = trials[i].ctas;
      rep->trials[i].ms_per_step = trials[i].ms;
      rep->trials[i].updates_per_s = trials[i].rate;
    }
    rep->best = best;
  }
  return s;
}

ls_status ls_get_layout_info(ls_handle* h, long long* info) {
  if (!h || !info) return LS_BAD_INPUT;
  if (!h->layout) return fail(h, LS_NOT_READY, "call ls_setup first");
  const lsgb::Layout& L = *h->layout;
  info[0] = L.nparts; info[1] = L.full; info[2] = L.lep; info[3] = L.lvp; info[4] = L.lgp;
  info[5] = L.lim; info[6] = lsgb::ref_array_size(L, lsgb::REF_BLOCK_ADJNCY); info[7] = L.nv;
  info[8] = L.ne; info[9] = L.dim;
  return LS_OK;
}

ls_status ls_get_layout(ls_handle* h, int which, void* dst) {
  if (!h || !dst) return LS_BAD_INPUT;
  if (!h->layout) return fail(h, LS_NOT_READY, "call ls_setup first");
  if (!lsgb::ref_array_copy(*h->layout, which, dst)) return fail(h, LS_BAD_INPUT, "unknown layout array");
  return LS_OK;
}

// ---------------------------------------------------------------------------
// Batches of independent meshes.

namespace {
ls_status bfail(ls_batch* b, ls_status s, const std::string& msg) {
  if (b) b->err = msg;
  return s;
}
ls_status bsolver_status(ls_batch* b, const std::string& msg) {
  if (msg.empty()) return LS_OK;
  b->err = msg;
  switch (b->solver ? b->solver->status_code() : 4) {
    case 1: return LS_BAD_INPUT;
    case 2: return LS_PATCH_TOO_LARGE;
    case 3: return LS_DEVICE_TIMEOUT;
    default: return LS_CUDA_ERROR;
  }
}
}  // namespace

ls_status ls_batch_create(ls_batch** b) {
  if (!b) return LS_BAD_INPUT;
  *b = new (std::nothrow) ls_batch();
  return *b ? LS_OK : LS_NO_MEMORY;
}

ls_status ls_batch_destroy(ls_batch* b) {
  delete b;
  return LS_OK;
}

const char* ls_batch_last_error(ls_batch* b) { return b ? b->err.c_str() : "null batch"; }

ls_status ls_batch_add(ls_batch* b, ls_handle* h, int* index) {
  if (!b || !h) return LS_BAD_INPUT;
  if (b->solver) return bfail(b, LS_BAD_INPUT, "batch already set up");
  ls_status s = ls_prepare(h);
  if (s != LS_OK) return bfail(b, s, std::string("member: ") + h->err);
  if (b->is_tri < 0) b->is_tri = h->is_tri;
  if (h->is_tri != b->is_tri) return bfail(b, LS_BAD_INPUT, "members of different dimension");
  if (!b->members.empty()) {
    const ls_params& a = b->members[0].prm;
    const ls_params& q = h->prm;
    const unsigned mask = ~(unsigned)LS_PROFILE;
    if (a.update_kind != q.update_kind || (a.flags & mask) != (q.flags & mask) || a.fim_sweeps != q.fim_sweeps ||
        a.inside_iterations != q.inside_iterations || a.smallnum != q.smallnum || a.largenum != q.largenum ||
        a.fp64_threshold != q.fp64_threshold)
      return bfail(b, LS_BAD_INPUT, "members must share the update kind, flags, sweeps and constants");
  }
  ls_batch::Member m;
  m.layout = *h->layout;
  m.phi = h->phi;
  m.vel = h->vel;
  m.prm = h->prm;
  m.nv = h->nv;
  m.ne = h->ne;
  m.xyz = h->xyz;
  m.elems = h->elems;
  m.user_partition = h->user_partition;
  if (h->user_partition) {
    m.npart = h->npart;
    m.nparts = h->nparts;
  }
  b->members.push_back(std::move(m));
  if (index) *index = (int)b->members.size() - 1;
  return LS_OK;
}

ls_status ls_batch_setup(ls_batch* b) {
  if (!b) return LS_BAD_INPUT;
  if (b->members.empty()) return bfail(b, LS_BAD_INPUT, "empty batch");
  std::vector<const lsgb::Layout*> parts;
  for (auto& m : b->members) parts.push_back(&m.layout);
  auto L = std::make_unique<lsgb::Layout>();
  std::string r = lsgb::merge_layouts(parts, *L);
  if (!r.empty()) return bfail(b, LS_BAD_INPUT, r);
  lsgb::SolverConfig cfg = solver_config(b->members[0].prm);
  std::vector<float> vel, phi;
  b->vbase.clear();
  int vb = 0;
  for (auto& m : b->members) {
    cfg.mesh_dt.push_back(m.prm.time_step);
    cfg.mesh_bandwidth.push_back(m.prm.bandwidth);
    cfg.mesh_curv.push_back(m.prm.curv_coeff);
    cfg.mesh_length_scale.push_back(m.prm.length_scale);
    vel.insert(vel.end(), m.vel.begin(), m.vel.end());
    phi.insert(phi.end(), m.phi.begin(), m.phi.end());
    b->vbase.push_back(vb);
    vb += m.nv;
  }
  b->vbase.push_back(vb);
  b->layout = std::move(L);
  b->solver = std::make_unique<lsgb::Solver>();
  r = b->solver->init(*b->layout, cfg, vel.data());
  if (!r.empty()) {
    ls_status s = bsolver_status(b, r);
    b->solver.reset();
    return s;
  }
  b->stage.assign(vb, 0.f);
  return bsolver_status(b, b->solver->set_phi(phi.data()));
}

namespace {
// Lays member m out again with patch size `size` (block side or partition
// target, by its partition type) through a temporary handle.
ls_status relayout_member(ls_batch* b, ls_batch::Member& m, int size) {
  ls_handle t;
  t.is_tri = b->is_tri;
  t.prm = m.prm;
  if (t.prm.partition_type == 1) t.prm.block_size = size;
  else t.prm.metis_size = size;
  t.xyz = m.xyz;
  t.elems = m.elems;
  t.nv = m.nv;
  t.ne = m.ne;
  t.phi = m.phi;
  t.vel = m.vel;
  t.have_phi = t.have_vel = true;
  ls_status s = ls_prepare(&t);
  if (s != LS_OK) return bfail(b, s, "member layout: " + t.err);
  m.layout = *t.layout;
  m.prm = t.prm;
  return LS_OK;
}
}  // namespace

ls_status ls_batch_autotune(ls_batch* b, int trial_steps, ls_tune_report* rep) {
  if (!b) return LS_BAD_INPUT;
  if (b->members.empty()) return bfail(b, LS_BAD_INPUT, "empty batch");
  if (trial_steps <= 0) trial_steps = 2;
  // patch sizes: only when every member is partitioned by the library with
  // the same partition type (a caller's partition is kept as it is)
  const int ptype = b->members[0].prm.partition_type;
  bool tunable = true;
  for (auto& m : b->members) tunable &= !m.user_partition && m.prm.partition_type == ptype;
  std::vector<int> sizes;
  if (!tunable) sizes.push_back(0);
  else if (ptype == 1) sizes = b->is_tri ? std::vector<int>{4, 5, 6, 8} : std::vector<int>{2, 3, 4};
  else sizes = b->is_tri ? std::vector<int>{16, 25, 36, 64} : std::vector<int>{8, 16, 27, 32, 64};
  const std::vector<int> ctas = b->is_tri ? std::vector<int>{2, 3, 4} : std::vector<int>{2, 3, 4, 5, 6, 7};
  std::vector<ls_params> saved;
  std::vector<lsgb::Layout> saved_layouts;
  for (auto& m : b->members) {
    saved.push_back(m.prm);
    saved_layouts.push_back(m.layout);
  }
  auto restore = [&] {
    for (size_t i = 0; i < b->members.size(); ++i) {
      b->members[i].prm = saved[i];
      b->members[i].layout = saved_layouts[i];
    }
  };
  struct Trial { int size, ctas; double ms, rate; };
  std::vector<Trial> trials;
  for (int sz : sizes) {
    b->solver.reset();
    bool fits = true;
    for (auto& m : b->members) {
      ls_status s = sz > 0 ? relayout_member(b, m, sz) : LS_OK;
      if (s == LS_PATCH_TOO_LARGE) { fits = false; break; }
      if (s != LS_OK) { restore(); return s; }
    }
    if (!fits) continue;
    int lep = 0;
    for (auto& m : b->members) lep = std::max(lep, m.layout.lep);
    // CTAs per SM only matter for patches of up to 384 element copies
    const std::vector<int> cs = lep <= 384 ? ctas : std::vector<int>{saved[0].fim_ctas_per_sm};
    for (int nc : cs) {
      for (auto& m : b->members) {
        m.prm.fim_ctas_per_sm = nc;
        m.prm.flags &= ~(unsigned)LS_PROFILE;
      }
      b->solver.reset();
      ls_status s = ls_batch_setup(b);
      if (s == LS_PATCH_TOO_LARGE) break;
      if (s != LS_OK) { restore(); return s; }
      int done = 0;
      std::string r = b->solver->run(1, nullptr, &done);  // warm-up (graph upload, caches)
      if (!r.empty()) { restore(); return bsolver_status(b, r); }
      b->solver->reset_stats();
      r = b->solver->run(trial_steps, nullptr, &done);
      if (!r.empty()) { restore(); return bsolver_status(b, r); }
      lsgb::SolverStats t;
      b->solver->stats(t);
      const double ms = done > 0 ? t.ms_total / done : 0.0;
      const double rate = t.ms_total > 0 ? (double)t.nb_vertex_updates / (t.ms_total / 1000.0) : 0.0;
      trials.push_back({sz, nc, ms, rate});
    }
  }
  b->solver.reset();
  if (trials.empty()) {
    restore();
    return bfail(b, LS_PATCH_TOO_LARGE, "no candidate fits");
  }
  int best = 0;
  for (int i = 1; i < (int)trials.size(); ++i)
    if (trials[i].rate > trials[best].rate) best = i;
  // leave the batch set up with the best candidate, every member at its phi0
  restore();
  if (trials[best].size > 0)
    for (auto& m : b->members) {
      ls_status s = relayout_member(b, m, trials[best].size);
      if (s != LS_OK) return s;
    }
  for (auto& m : b->members) m.prm.fim_ctas_per_sm = trials[best].ctas;
  ls_status s = ls_batch_setup(b);
  if (rep) {
    std::memset(rep, 0, sizeof(*rep));
    rep->ntrials = std::min((int)trials.size(), LS_TUNE_MAX_TRIALS);
    for (int i = 0; i < rep->ntrials; ++i) {
      rep->trials[i].patch_size = trials[i].size;
      rep->trials[i].fim_ctas_per_sm = trials[i].ctas;
      rep->trials[i].ms_per_step = trials[i].ms;
      rep->trials[i].updates_per_s = trials[i].rate;
    }
    rep->best = best;
  }
  return s;
}

ls_status ls_batch_solve(ls_batch* b, int nsteps, int* steps_done) {
  if (!b) return LS_BAD_INPUT;
  if (!b->solver) return bfail(b, LS_NOT_READY, "call ls_batch_setup first");
  if (nsteps < 0) return bfail(b, LS_BAD_INPUT, "negative step count");
  return bsolver_status(b, b->solver->run(nsteps, nullptr, steps_done));
}

ls_status ls_batch_get_phi(ls_batch* b, int index, float* phi) {
  if (!b || !phi) return LS_BAD_INPUT;
  if (!b->solver) return bfail(b, LS_NOT_READY, "call ls_batch_setup first");
  if (index < 0 || index >= (int)b->members.size()) return bfail(b, LS_BAD_INPUT, "bad member index");
  std::string r = b->solver->get_phi(b->stage.data());
  if (!r.empty()) return bsolver_status(b, r);
  std::memcpy(phi, b->stage.data() + b->vbase[index], sizeof(float) * (size_t)b->members[index].nv);
  return LS_OK;
}

ls_status ls_batch_get_stats(ls_batch* b, ls_stats* s) {
  if (!b || !s) return LS_BAD_INPUT;
  std::memset(s, 0, sizeof(*s));
  if (!b->solver) return LS_OK;
  lsgb::SolverStats t;
  b->solver->stats(t);
  fill_stats(t, s);
  return LS_OK;
}

ls_status ls_batch_reset_stats(ls_batch* b) {
  if (!b) return LS_BAD_INPUT;
  if (b->solver) b->solver->reset_stats();
  return LS_OK;
}

ls_status ls_batch_set_profile(ls_batch* b, int on) {
  if (!b) return LS_BAD_INPUT;
  if (!b->solver) return bfail(b, LS_NOT_READY, "call ls_batch_setup first");
  b->solver->set_profile(on != 0);
  return LS_OK;
}

ls_status ls_batch_get_layout_info(ls_batch* b, long long* info) {
  if (!b || !info) return LS_BAD_INPUT;
  if (!b->layout) {
    // merge on the host only (no device work), for layout checks
    std::vector<const lsgb::Layout*> parts;
    for (auto& m : b->members) parts.push_back(&m.layout);
    if (parts.empty()) return bfail(b, LS_BAD_INPUT, "empty batch");
    auto L = std::make_unique<lsgb::Layout>();
    std::string r = lsgb::merge_layouts(parts, *L);
    if (!r.empty()) return bfail(b, LS_BAD_INPUT, r);
    b->layout = std::move(L);
  }
  const lsgb::Layout& L = *b->layout;
  info[0] = L.nparts; info[1] = L.full; info[2] = L.lep; info[3] = L.lvp; info[4] = L.lgp;
  info[5] = L.lim; info[6] = lsgb::ref_array_size(L, lsgb::REF_BLOCK_ADJNCY); info[7] = L.nv;
  info[8] = L.ne; info[9] = L.dim;
  return LS_OK;
}

ls_status ls_batch_get_layout(ls_batch* b, int which, void* dst) {
  if (!b || !dst) return LS_BAD_INPUT;
  long long info[10];
  ls_status s = ls_batch_get_layout_info(b, info);
  if (s != LS_OK) return s;
  if (!lsgb::ref_array_copy(*b->layout, which, dst)) return bfail(b, LS_BAD_INPUT, "unknown layout array");
  return LS_OK;
}

// ---------------------------------------------------------------------------
// The learned warm start's network.

}  // extern "C"

struct ls_mlp {
  lsgb::mlp::Net net;
  std::string err;
};

namespace {
ls_status mfail(ls_mlp* m, const std::string& msg, ls_status s = LS_CUDA_ERROR) {
  if (msg.empty()) return LS_OK;
  if (m) m->err = msg;
  return s;
}
}  // namespace

extern "C" {

ls_status ls_mlp_create(ls_mlp** m, unsigned long long seed) {
  if (!m) return LS_BAD_INPUT;
  ls_mlp* x = new (std::nothrow) ls_mlp();
  if (!x) return LS_NO_MEMORY;
  std::string r = x->net.init(seed);
  if (!r.empty()) {
    delete x;
    *m = nullptr;
    return LS_CUDA_ERROR;
  }
  *m = x;
  return LS_OK;
}

ls_status ls_mlp_destroy(ls_mlp* m) {
  delete m;
  return LS_OK;
}

const char* ls_mlp_last_error(ls_mlp* m) { return m ? m->err.c_str() : "null network"; }

int ls_mlp_num_params(void) { return lsgb::mlp::Net::num_params(); }

ls_status ls_mlp_set_params(ls_mlp* m, const float* p) {
  if (!m || !p) return LS_BAD_INPUT;
  return mfail(m, m->net.set_params(p));
}

ls_status ls_mlp_get_params(ls_mlp* m, float* p) {
  if (!m || !p) return LS_BAD_INPUT;
  return mfail(m, m->net.get_params(p));
}

ls_status ls_mlp_predict(ls_mlp* m, const float* x, int n, float* y) {
  if (!m || n < 0 || (n > 0 && (!x || !y))) return LS_BAD_INPUT;
  return mfail(m, m->net.predict(x, n, y));
}

ls_status ls_mlp_gradients(ls_mlp* m, const float* x, const float* t, int n, float* g, float* loss) {
  if (!m || n <= 0 || !x || !t || !g) return LS_BAD_INPUT;
  return mfail(m, m->net.gradients(x, t, n, g, loss));
}

ls_status ls_mlp_train(ls_mlp* m, const float* x, const float* t, int n, int epochs, int batch, float lr,
                       float* loss) {
  if (!m || n <= 0 || !x || !t || epochs <= 0 || batch <= 0 || !(lr > 0.f)) return LS_BAD_INPUT;
  return mfail(m, m->net.train(x, t, n, epochs, batch, lr, loss));
}

ls_status ls_mlp_reserve_pairs(ls_mlp* m, long long capacity) {
  if (!m || capacity <= 0) return LS_BAD_INPUT;
  return mfail(m, m->net.reserve_pairs(capacity), LS_NO_MEMORY);
}

ls_status ls_mlp_clear_pairs(ls_mlp* m) {
  if (!m) return LS_BAD_INPUT;
  return mfail(m, m->net.clear_pairs());
}

ls_status ls_mlp_num_pairs(ls_mlp* m, long long* n) {
  if (!m || !n) return LS_BAD_INPUT;
  *n = m->net.num_pairs();
  return LS_OK;
}

ls_status ls_mlp_train_pairs(ls_mlp* m, int epochs, int batch, float lr, unsigned long long seed, float* loss) {
  if (!m || epochs <= 0 || batch <= 0 || !(lr > 0.f)) return LS_BAD_INPUT;
  return mfail(m, m->net.train_pairs(epochs, batch, lr, seed, loss));
}

ls_status ls_mlp_eval_pairs(ls_mlp* m, long long first, long long count, float* abs_err) {
  if (!m || first < 0 || count < 0 || (count > 0 && !abs_err)) return LS_BAD_INPUT;
  return mfail(m, m->net.eval_pairs(first, count, abs_err));
}

ls_status ls_learn_collect(ls_handle* h, ls_mlp* m, int nsteps, int* steps_done) {
  if (!h || !m || nsteps < 0) return LS_BAD_INPUT;
  if (!h->solver) return fail(h, LS_NOT_READY, "call ls_setup first");
  std::string r = h->solver->set_collect(&m->net);
  if (!r.empty()) return solver_status(h, r);
  r = h->solver->run(nsteps, nullptr, steps_done);
  h->solver->set_collect(nullptr);
  return solver_status(h, r);
}

ls_status ls_batch_set_learned(ls_batch* b, ls_mlp* m, double margin, double support_tol, int reset_mode) {
  if (!b || margin < 0 || support_tol < 0 || reset_mode < 0 || reset_mode > 1) return LS_BAD_INPUT;
  if (!b->solver) return bfail(b, LS_NOT_READY, "call ls_batch_setup first");
  return bsolver_status(b, b->solver->set_learned(m ? &m->net : nullptr, (float)margin, (float)support_tol,
                                                  reset_mode == 0));
}

ls_status ls_set_learned(ls_handle* h, ls_mlp* m, double margin, double support_tol, int reset_mode) {
  if (!h || margin < 0 || support_tol < 0 || reset_mode < 0 || reset_mode > 1) return LS_BAD_INPUT;
  if (!h->solver) return fail(h, LS_NOT_READY, "call ls_setup first");
  return solver_status(h, h->solver->set_learned(m ? &m->net : nullptr, (float)margin, (float)support_tol,
                                                 reset_mode == 0));
}

}  // extern "C"
