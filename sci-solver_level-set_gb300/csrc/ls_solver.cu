// ls_solver.cu -- host orchestration of the device time step.
//
// The reference drives its FIM loop from the host with two synchronous
// device->host copies and a host list update per iteration
// (src/core3d/cuda/redistance3d.cu:85-224).  Here the lists, labels and
// convergence flags stay on the device; the host only launches a fixed
// chunk of FIM iterations (captured once as a CUDA graph) and reads one
// counter per chunk to learn whether the active list has drained.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ls_solver.h"

namespace lsgb {

namespace {
template <typename T>
cudaError_t dalloc(std::vector<void*>& list, T** p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * n);
  if (e == cudaSuccess) list.push_back(*p);
  return e;
}
template <typename T>
cudaError_t upload(std::vector<void*>& list, const T** p, const std::vector<T>& v, cudaStream_t st) {
  T* d = nullptr;
  cudaError_t e = dalloc(list, &d, v.size());
  if (e != cudaSuccess) return e;
  if (!v.empty()) e = cudaMemcpyAsync(d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st);
  *p = d;
  return e;
}

}  // namespace

Solver::~Solver() {
  if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
  if (graph_) cudaGraphDestroy(graph_);
  for (void* p : allocs_) cudaFree(p);
  if (h_counts_) cudaFreeHost(h_counts_);
  if (h_stats_) cudaFreeHost(h_stats_);
  if (h_stage_) cudaFreeHost(h_stage_);
  if (h_snap_) cudaFreeHost(h_snap_);
  if (ev0_) cudaEventDestroy(ev0_);
  if (ev1_) cudaEventDestroy(ev1_);
  for (auto& pe : prof_) {
    cudaEventDestroy(pe.a);
    cudaEventDestroy(pe.b);
  }
  for (cudaEvent_t e : ev_pool_) cudaEventDestroy(e);
  if (stream_) cudaStreamDestroy(stream_);
}

// Two events for one profiled launch, from the pool where it has some.
cudaError_t Solver::prof_begin(ProfEvent& pe, int kind) {
  pe.kind = kind;
  cudaEvent_t ev[2];
  for (int i = 0; i < 2; ++i) {
    if (!ev_pool_.empty()) {
      ev[i] = ev_pool_.back();
      ev_pool_.pop_back();
    } else {
      cudaError_t e = cudaEventCreate(&ev[i]);
      if (e != cudaSuccess) {
        if (i == 1) ev_pool_.push_back(ev[0]);
        return e;
      }
    }
  }
  pe.a = ev[0];
  pe.b = ev[1];
  return cudaSuccess;
}

// A profiled FIM launch: events around it as for the other kernels, and the
// slab-byte counter copied (on the stream, device to device) just before
// and just after it, outside the event pair.
cudaError_t Solver::prof_fim_begin(ProfEvent& pe, int kind) {
  cudaError_t e = prof_begin(pe, kind);
  if (e != cudaSuccess) return e;
  pe.snap = -1;
  if (!d_snap_) {
    long long* d = nullptr;
    e = dalloc(allocs_, &d, (size_t)2 * kSnapCap);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&h_snap_, sizeof(long long) * 2 * kSnapCap);
    if (e != cudaSuccess) return e;
    d_snap_ = d;
  }
  if (nsnap_ < kSnapCap) {
    pe.snap = nsnap_++;
    e = cudaMemcpyAsync(d_snap_ + 2 * pe.snap, s_.stats + 7, sizeof(long long), cudaMemcpyDeviceToDevice, stream_);
    if (e != cudaSuccess) return e;
  }
  return cudaEventRecord(pe.a, stream_);
}

cudaError_t Solver::prof_fim_end(ProfEvent& pe) {
  cudaError_t e = cudaEventRecord(pe.b, stream_);
  if (e == cudaSuccess && pe.snap >= 0)
    e = cudaMemcpyAsync(d_snap_ + 2 * pe.snap + 1, s_.stats + 7, sizeof(long long), cudaMemcpyDeviceToDevice,
                        stream_);
  prof_.push_back(pe);
  return e;
}

// Adds the pending launch times to the stats (keep_times) or drops them, and
// returns their events to the pool; FIM launches also go to the launch log
// with their slab bytes.
void Solver::fold_prof(bool keep_times) {
  bool snaps = false;
  if (keep_times && nsnap_ > 0)
    snaps = cudaMemcpyAsync(h_snap_, d_snap_, sizeof(long long) * 2 * nsnap_, cudaMemcpyDeviceToHost, stream_) ==
                cudaSuccess &&
            cudaStreamSynchronize(stream_) == cudaSuccess;
  nsnap_ = 0;
  for (auto& pe : prof_) {
    float ms = 0;
    if (keep_times && cudaEventSynchronize(pe.b) == cudaSuccess &&
        cudaEventElapsedTime(&ms, pe.a, pe.b) == cudaSuccess) {
      if (pe.kind <= 1 && launch_log_.size() < kLaunchLogCap)
        launch_log_.push_back(
            {pe.kind, (double)ms, (snaps && pe.snap >= 0) ? h_snap_[2 * pe.snap + 1] - h_snap_[2 * pe.snap] : -1});
      switch (pe.kind) {
        case 0: st_.ms_sweep += ms; st_.n_sweep++; break;
        case 1: st_.ms_check += ms; st_.n_check++; break;
        case 2: st_.ms_schedule += ms; st_.n_schedule++; break;
        case 3: st_.ms_seed += ms; st_.n_seed++; break;
        case 4: st_.ms_narrowband += ms; st_.n_narrowband++; break;
        case 5: st_.ms_update += ms; st_.n_update++; break;
      }
    }
    ev_pool_.push_back(pe.a);
    ev_pool_.push_back(pe.b);
  }
  prof_.clear();
}

std::string Solver::check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return "";
  status_ = 4;
  return std::string(what) + ": " + cudaGetErrorString(e);
}

#define LS_TRY(expr, what)                         \
  do {                                             \
    std::string _m = check((expr), (what));        \
    if (!_m.empty()) return _m;                    \
  } while (0)

std::string Solver::init(const Layout& L, const SolverConfig& cfg, const float* vel) {
  lay_ = &L;
  cfg_ = cfg;
  K_ = cfg.bit_exact ? &kernels_exact() : &kernels_fast();
  if (L.lep > 1024) { status_ = 2; return "a patch has more than 1024 element copies"; }
  // active-list entries carry the visited-ahead mark above the patch id
  if (L.nparts >= kPrevisited) return "too many patches";
  LS_TRY(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream");
  {
    int dev = 0;
    LS_TRY(cudaGetDevice(&dev), "device");
    if (cudaDeviceGetAttribute(&pageable_, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) pageable_ = 0;
    if (cfg.host_staging) pageable_ = 0;
  }
  LS_TRY(cudaEventCreate(&ev0_), "event");
  LS_TRY(cudaEventCreate(&ev1_), "event");
  const int nv = L.nv, np = L.nparts;
  const long long full = L.full;
  const int d1 = L.dim + 1;

  // per-copy arrays
  std::vector<ushort4> conn(full);
  for (long long c = 0; c < full; ++c)
    conn[c] = make_ushort4(L.conn_local[c * 4], L.conn_local[c * 4 + 1], L.conn_local[c * 4 + 2],
                           L.conn_local[c * 4 + 3]);
  const int nc = L.dim == 3 ? 6 : 3;
  std::vector<float> lc((size_t)nc * full), sig((size_t)3 * full, 0.f);
  // FIM frame: without the reference's semantics, lengths are divided by
  // the mesh scale (mean edge length unless given) so that the local
  // solver's polynomial terms are O(1) in FP32 whatever the caller's units.
  const bool ref = cfg.ref_compat != 0;
  const double scale = ref ? 1.0 : (cfg.length_scale > 0 ? cfg.length_scale : L.mean_edge);
  // batches: each mesh has its own FIM frame
  const bool batch = !L.patch_mesh.empty();
  const int nmesh = batch ? (int)L.mesh_edge.size() : 1;
  std::vector<double> mscale(nmesh, scale);
  std::vector<double> copy_scale;
  if (batch) {
    if ((int)cfg.mesh_dt.size() != nmesh || (int)cfg.mesh_bandwidth.size() != nmesh ||
        (int)cfg.mesh_curv.size() != nmesh || (int)cfg.mesh_length_scale.size() != nmesh) {
      status_ = 1;
      return "per-mesh parameters missing";
    }
    for (int k = 0; k < nmesh; ++k)
      mscale[k] = ref ? 1.0 : (cfg.mesh_length_scale[k] > 0 ? cfg.mesh_length_scale[k] : L.mesh_edge[k]);
    copy_scale.resize(full);
    for (int p = 0; p < np; ++p)
      for (int c = L.ele_offsets[p]; c < L.ele_offsets[p + 1]; ++c) copy_scale[c] = mscale[L.patch_mesh[p]];
  }
  mesh_scale_ = mscale;
  for (long long c = 0; c < full; ++c) {
    const double cs = batch ? copy_scale[c] : scale;
    const int e = L.ele_permute[c];
    if (L.dim == 3) {
      float P[4][3], Lc[6];
      for (int k = 0; k < 4; ++k)
        for (int j = 0; j < 3; ++j) P[k][j] = L.xyz_p[(size_t)j * nv + L.conn[c * 4 + k]];
      tet_local_coords(P, Lc);
      for (int i = 0; i < 6; ++i) lc[i * full + c] = ref ? Lc[i] : (float)((double)Lc[i] / cs);
      if (vel)
        for (int j = 0; j < 3; ++j) sig[j * full + c] = vel[(size_t)e * 3 + j];
    } else {
      double P[3][3], Lc[3], sg[2], vv[3] = {0, 0, 0};
      for (int k = 0; k < 3; ++k)
        for (int j = 0; j < 3; ++j) P[k][j] = L.xyz_p[(size_t)j * nv + L.conn[c * 3 + k]];
      if (vel)
        for (int j = 0; j < 3; ++j) vv[j] = vel[(size_t)e * 3 + j];
      tri_local_coords(P, vv, Lc, sg);
      for (int i = 0; i < 3; ++i) lc[i * full + c] = (float)(ref ? Lc[i] : Lc[i] / cs);
      sig[c] = (float)sg[0];
      sig[full + c] = (float)sg[1];
    }
  }
  // per-patch algorithmic bytes of one FIM visit: owned DT read + DT_out
  // write + seed flags, ghost ids + ghost DT, connectivity (8 B) and local
  // coordinates (4 B each) per copy, 3 patch offsets pairs
  std::vector<int> pbytes(np);
  for (int p = 0; p < np; ++p) {
    const long long nvp = L.vert_offsets[p + 1] - L.vert_offsets[p];
    const long long ngp = L.ghost_offsets[p + 1] - L.ghost_offsets[p];
    const long long nep = L.ele_offsets[p + 1] - L.ele_offsets[p];
    pbytes[p] = (int)(nvp * (4 + 4 + 1) + ngp * (4 + 4) + nep * (8 + 4 * nc) + 24);
  }
  std::vector<int> ipermute(L.vert_ipermute);

  m_.dim = L.dim; m_.nv = nv; m_.nparts = np; m_.full = full;
  std::vector<void*>& A = allocs_;
  LS_TRY(upload(A, &m_.vert_off, L.vert_offsets, stream_), "upload");
  LS_TRY(upload(A, &m_.ele_off, L.ele_offsets, stream_), "upload");
  LS_TRY(upload(A, &m_.ghost_off, L.ghost_offsets, stream_), "upload");
  LS_TRY(upload(A, &m_.ghost_ids, L.ghost_ids, stream_), "upload");
  LS_TRY(upload(A, &m_.conn, conn, stream_), "upload");
  LS_TRY(upload(A, &m_.lc, lc, stream_), "upload");
  LS_TRY(upload(A, &m_.sig, sig, stream_), "upload");
  LS_TRY(upload(A, &m_.vslot_off, L.vslot_off, stream_), "upload");
  LS_TRY(upload(A, &m_.vslot, L.vslot, stream_), "upload");
  LS_TRY(upload(A, &m_.padj_off, L.padj_off, stream_), "upload");
  LS_TRY(upload(A, &m_.padj, L.padj, stream_), "upload");
  LS_TRY(upload(A, &m_.xyz, L.xyz_p, stream_), "upload");
  LS_TRY(upload(A, &m_.ipermute, ipermute, stream_), "upload");
  m_.capped = nullptr;
  m_.slot_cap = ref_slot_cap(L.dim);
  if (ref && L.any_capped) LS_TRY(upload(A, &m_.capped, L.slot_capped, stream_), "upload");
  m_.patch_mesh = nullptr;
  m_.mesh_par = nullptr;
  m_.geo_m = nullptr;
  m_.geo_h = nullptr;
  if (batch) {
    std::vector<float4> mp(nmesh);
    for (int k = 0; k < nmesh; ++k)
      mp[k] = make_float4((float)(cfg.mesh_bandwidth[k] / mscale[k]), (float)mscale[k], (float)cfg.mesh_dt[k],
                          (float)cfg.mesh_curv[k]);
    LS_TRY(upload(A, &m_.patch_mesh, L.patch_mesh, stream_), "upload");
    LS_TRY(upload(A, &m_.mesh_par, mp, stream_), "upload");
  }
  // step state
  LS_TRY(dalloc(A, &s_.phi, nv), "alloc");
  LS_TRY(dalloc(A, &s_.phi_out, nv), "alloc");
  LS_TRY(dalloc(A, &s_.DT, nv), "alloc");
  LS_TRY(dalloc(A, &s_.DT_out, nv), "alloc");
  LS_TRY(dalloc(A, &s_.seed, nv), "alloc");
  LS_TRY(dalloc(A, &s_.sign, nv), "alloc");
  LS_TRY(dalloc(A, &s_.blabel, np), "alloc");
  LS_TRY(dalloc(A, &s_.bcon, np), "alloc");
  LS_TRY(dalloc(A, &s_.bmin, np), "alloc");
  LS_TRY(dalloc(A, &s_.list0, np), "alloc");
  LS_TRY(dalloc(A, &s_.list1, np), "alloc");
  LS_TRY(dalloc(A, &s_.newlist, np), "alloc");
  LS_TRY(dalloc(A, &s_.nblist, np), "alloc");
  LS_TRY(dalloc(A, &s_.counts, 8), "alloc");
  LS_TRY(dalloc(A, &s_.stats, 9), "alloc");
  LS_TRY(dalloc(A, &s_.ctl, 4), "alloc");
  LS_TRY(dalloc(A, &s_.sched, 4), "alloc");
  LS_TRY(dalloc(A, &s_.gbar, kGridBarrierWords), "alloc");
  LS_TRY(cudaMemsetAsync(s_.gbar, 0, sizeof(unsigned) * kGridBarrierWords, stream_), "memset");
  LS_TRY(dalloc(A, &d_tmp_, nv), "alloc");
  LS_TRY(cudaMemsetAsync(s_.counts, 0, sizeof(int) * 8, stream_), "memset");
  LS_TRY(cudaMemsetAsync(s_.stats, 0, sizeof(unsigned long long) * 9, stream_), "memset");
  LS_TRY(cudaMemsetAsync(s_.ctl, 0, sizeof(int) * 4, stream_), "memset");
  LS_TRY(cudaMemsetAsync(s_.sched, 0, sizeof(int) * 4, stream_), "memset");
  LS_TRY(cudaMemsetAsync(s_.phi, 0, sizeof(float) * nv, stream_), "memset");
  LS_TRY(cudaMallocHost((void**)&h_counts_, sizeof(int) * 12), "pinned");
  LS_TRY(cudaMallocHost((void**)&h_stats_, sizeof(unsigned long long) * 9), "pinned");
  LS_TRY(cudaMallocHost((void**)&h_stage_, sizeof(float) * nv), "pinned");

  // parameters (FIM quantities in the FIM frame)
  sp_.largenum = (float)cfg.largenum;
  sp_.bandwidth = (float)(cfg.bandwidth / scale);
  sp_.scale = (float)scale;
  sp_.tau = (cfg.fp64_flagged && L.dim == 3) ? (float)cfg.fp64_tau : 0.f;
  sp_.xdiv = (cfg.bit_exact && ref) ? 1 : 0;
  sp_.ctas = (cfg.fim_ctas >= 2 && cfg.fim_ctas <= 7) ? cfg.fim_ctas : 5;
  sp_.tol = (float)cfg.smallnum;
  sp_.eps_h64 = cfg.smallnum;
  sp_.eps_h = (float)sp_.eps_h64;
  sp_.dt = (float)cfg.dt;
  sp_.curv_coeff = (float)cfg.curv_coeff;
  sp_.niter = cfg.niter > 0 ? cfg.niter : (L.dim == 3 ? 5 : 10);
  sp_.ref_compat = ref ? 1 : 0;
  sp_.update_kind = cfg.update_kind;
  sp_.lvp = L.lvp;
  sp_.lgp = L.lgp;
  sp_.lep = L.lep;
  sp_.max_fim_iters = cfg.max_fim_iters;
  sp_.spin_limit = cfg.spin_limit != 0 ? cfg.spin_limit : (1 << 22);
  (void)d1;
  LS_TRY(K_->configure(m_, sp_, L_), "configure");
  if (L_.pair_block > 0) {
    // the two-copies-per-thread sweep stages precomputed per-copy geometry
    // (metric terms and heights, 64 bytes a copy) instead of the 24 bytes of
    // local coordinates it would otherwise turn into them on every visit
    float4* geo = nullptr;
    LS_TRY(dalloc(A, &geo, (size_t)4 * (size_t)full), "alloc");
    m_.geo_m = geo;
    m_.geo_h = geo + 3 * full;
    LS_TRY(K_->geometry(m_, geo, geo + 3 * full, L_, stream_), "geometry");
    for (int p = 0; p < np; ++p) {
      const long long nep = L.ele_offsets[p + 1] - L.ele_offsets[p];
      pbytes[p] += (int)(nep * (64 - 4 * nc));
    }
  }
  LS_TRY(upload(A, &m_.patch_bytes, pbytes, stream_), "upload");
  // the persistent FIM loop where the chosen sweep kernel has that form
  persistent_ = cfg_.persistent && L_.persist_grid > 0;
  if (cfg_.graph_chunk < 2) cfg_.graph_chunk = 2;
  if (cfg_.graph_chunk & 1) cfg_.graph_chunk++;
  if (cfg_.use_graph) {
    std::string r = build_graph();
    if (!r.empty()) return r;
  }
  LS_TRY(cudaStreamSynchronize(stream_), "init sync");
  return "";
}

// Step control kernels (host orchestration, same for both kernel builds).
namespace {
// End of one FIM loop body (graph_chunk iterations): continue while the
// active list is not empty, at most max_bodies bodies per step; the cap
// sets ctl[1] so that the host reports a timeout.
__global__ void k_loop_cond(const int* counts, int* ctl, cudaGraphConditionalHandle h, int max_bodies) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const int b = ++ctl[0];
    const bool more = counts[0] > 0 && ctl[3] == 0;  // a FIM kernel wait that ran out ends the loop
    if (more && b >= max_bodies) ctl[1] = 1;
    cudaGraphSetConditional(h, (more && b < max_bodies) ? 1u : 0u);
  }
}
// After the narrowband: the next step's seed search is restricted to it
// when it is not empty.
__global__ void k_step_tail(const int* counts, int* ctl) {
  if (threadIdx.x == 0 && blockIdx.x == 0) ctl[2] = counts[3] > 0 ? 1 : 0;
}
}  // namespace

// One time step as one graph: seed part, a while node running FIM loop
// bodies of graph_chunk iterations until the active list drains (or the
// iteration cap), then narrowband and update.  The host launches it and
// reads the counters once per step.
// The persistent form: the whole step is one captured sequence (seed part,
// the cooperative FIM launch, narrowband and update), no conditional node.
// Returns false when the runtime will not capture the cooperative launch (the
// step then launches kernel by kernel).
bool Solver::build_persistent_graph(std::string* err) {
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return false;
  cudaError_t e = step_persistent_launches(-1);
  cudaError_t e2 = cudaStreamEndCapture(stream_, &g);
  if (e != cudaSuccess || e2 != cudaSuccess || !g) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();  // clear the capture failure
    return false;
  }
  cudaError_t e3 = cudaGraphInstantiate(&graph_exec_, g, 0);
  graph_ = g;
  if (e3 != cudaSuccess) {
    *err = std::string("graph instantiate: ") + cudaGetErrorString(e3);
    graph_exec_ = nullptr;
    return false;
  }
  return true;
}

// One step of the persistent form, launch by launch (use_all < 0: the seed
// kernel decides from the step-control flag, as in a graph).
cudaError_t Solver::step_persistent_launches(int use_all) {
  cudaError_t err = cudaMemsetAsync(s_.counts, 0, sizeof(int) * 3, stream_);
  if (err == cudaSuccess) err = cudaMemsetAsync(s_.counts + 4, 0, sizeof(int), stream_);
  if (err == cudaSuccess) err = cudaMemsetAsync(s_.ctl, 0, sizeof(int) * 2, stream_);
  if (err == cudaSuccess) err = cudaMemsetAsync(s_.ctl + 3, 0, sizeof(int), stream_);
  if (err == cudaSuccess) err = cudaMemsetAsync(s_.gbar, 0, sizeof(unsigned) * kGridBarrierWords, stream_);
  // the patch-draw counters are zero after every complete launch; a launch
  // abandoned on a barrier timeout can leave them set
  if (err == cudaSuccess) err = cudaMemsetAsync(s_.sched, 0, sizeof(int) * 2, stream_);
  if (err == cudaSuccess) err = K_->reset(m_, s_, sp_, L_, stream_);
  if (err == cudaSuccess) err = cudaMemsetAsync(s_.blabel, 0, sizeof(int) * m_.nparts, stream_);
  if (err == cudaSuccess) err = K_->seed(m_, s_, use_all, sp_.scale, L_, stream_);
  if (err == cudaSuccess) err = cudaMemsetAsync(s_.counts + 3, 0, sizeof(int), stream_);
  if (err == cudaSuccess) err = K_->fim_persistent(m_, s_, sp_, L_, stream_);
  if (err == cudaSuccess) err = K_->narrowband(m_, s_, sp_, L_, stream_);
  if (err == cudaSuccess) {
    k_step_tail<<<1, 32, 0, stream_>>>(s_.counts, s_.ctl);
    err = cudaGetLastError();
  }
  if (cfg_.update_kind != 2)
    for (int it = 0; it < cfg_.inside_niter && err == cudaSuccess; ++it) err = K_->update(m_, s_, sp_, L_, stream_);
  return err;
}

std::string Solver::build_graph() {
  if (persistent_) {
    std::string err;
    if (build_persistent_graph(&err)) return "";
    if (!err.empty()) return err;
    return "";  // no graph: the persistent step launches kernel by kernel
  }
  const int chunk = cfg_.graph_chunk;
  const int max_bodies = (cfg_.max_fim_iters + chunk - 1) / chunk;
  cudaGraph_t pre = nullptr, post = nullptr;
  cudaError_t err = cudaSuccess;
  // seed part
  LS_TRY(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "capture begin");
  err = cudaMemsetAsync(s_.counts, 0, sizeof(int) * 3, stream_);
  if (err == cudaSuccess) err = cudaMemsetAsync(s_.counts + 4, 0, sizeof(int), stream_);
  if (err == cudaSuccess) err = cudaMemsetAsync(s_.ctl, 0, sizeof(int) * 2, stream_);
  if (err == cudaSuccess) err = cudaMemsetAsync(s_.ctl + 3, 0, sizeof(int), stream_);
  if (err == cudaSuccess) err = K_->reset(m_, s_, sp_, L_, stream_);
  if (err == cudaSuccess) err = cudaMemsetAsync(s_.blabel, 0, sizeof(int) * m_.nparts, stream_);
  if (err == cudaSuccess) err = K_->seed(m_, s_, -1, sp_.scale, L_, stream_);
  if (err == cudaSuccess) err = cudaMemsetAsync(s_.counts + 3, 0, sizeof(int), stream_);
  cudaError_t e2 = cudaStreamEndCapture(stream_, &pre);
  LS_TRY(err, "capture seed part");
  LS_TRY(e2, "capture end");
  // narrowband + update part
  LS_TRY(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "capture begin");
  err = K_->narrowband(m_, s_, sp_, L_, stream_);
  if (err == cudaSuccess) {
    k_step_tail<<<1, 32, 0, stream_>>>(s_.counts, s_.ctl);
    err = cudaGetLastError();
  }
  if (cfg_.update_kind != 2)
    for (int it = 0; it < cfg_.inside_niter && err == cudaSuccess; ++it) err = K_->update(m_, s_, sp_, L_, stream_);
  e2 = cudaStreamEndCapture(stream_, &post);
  LS_TRY(err, "capture update part");
  LS_TRY(e2, "capture end");

  LS_TRY(cudaGraphCreate(&graph_, 0), "graph create");
  cudaGraphNode_t npre, nloop, npost;
  LS_TRY(cudaGraphAddChildGraphNode(&npre, graph_, nullptr, 0, pre), "graph child");
  cudaGraphConditionalHandle hc;
  LS_TRY(cudaGraphConditionalHandleCreate(&hc, graph_, 1, cudaGraphCondAssignDefault), "conditional handle");
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = hc;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  LS_TRY(cudaGraphAddNode(&nloop, graph_, &npre, nullptr, 1, &cp), "graph while node");
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  LS_TRY(cudaStreamBeginCaptureToGraph(stream_, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
         "capture body");
  err = cudaSuccess;
  for (int i = 0; i < chunk && err == cudaSuccess; ++i) {
    const int cur = i & 1;
    err = K_->sweep(m_, s_, sp_, cur, false, L_, stream_);
    if (err == cudaSuccess) err = K_->schedule(m_, s_, sp_, cur, L_, stream_);
    if (err == cudaSuccess) err = K_->sweep(m_, s_, sp_, cur, true, L_, stream_);
  }
  if (err == cudaSuccess) {
    k_loop_cond<<<1, 32, 0, stream_>>>(s_.counts, s_.ctl, hc, max_bodies);
    err = cudaGetLastError();
  }
  e2 = cudaStreamEndCapture(stream_, &body);
  LS_TRY(err, "capture body launch");
  LS_TRY(e2, "capture body end");
  LS_TRY(cudaGraphAddChildGraphNode(&npost, graph_, &nloop, 1, post), "graph child");
  cudaGraphDestroy(pre);
  cudaGraphDestroy(post);
  LS_TRY(cudaGraphInstantiate(&graph_exec_, graph_, 0), "graph instantiate");
  return "";
}

std::string Solver::fim_loop(const StepParams& sp) {
  long long launched = 0;
  auto prof = [&](int kind, auto&& fn) -> cudaError_t {
    if (!cfg_.profile) return fn();
    ProfEvent pe;
    cudaError_t e = prof_fim_begin(pe, kind);
    if (e != cudaSuccess) return e;
    e = fn();
    cudaError_t e2 = prof_fim_end(pe);
    return e != cudaSuccess ? e : e2;
  };
  // a wait of the FIM kernels that runs out sets ctl[3] (read at every sync)
  LS_TRY(cudaMemsetAsync(s_.ctl + 3, 0, sizeof(int), stream_), "memset");
  while (true) {
    for (int i = 0; i < cfg_.graph_chunk; ++i) {
      const int cur = i & 1;
      LS_TRY(prof(0, [&] { return K_->sweep(m_, s_, sp, cur, false, L_, stream_); }), "sweep");
      LS_TRY(prof(2, [&] { return K_->schedule(m_, s_, sp, cur, L_, stream_); }), "schedule");
      LS_TRY(prof(1, [&] { return K_->sweep(m_, s_, sp, cur, true, L_, stream_); }), "check");
    }
    launched += cfg_.graph_chunk;
    st_.kernel_launches += 3LL * cfg_.graph_chunk;
    LS_TRY(cudaMemcpyAsync(h_counts_, s_.counts, sizeof(int) * 8, cudaMemcpyDeviceToHost, stream_), "d2h");
    LS_TRY(cudaMemcpyAsync(h_counts_ + 8, s_.ctl, sizeof(int) * 4, cudaMemcpyDeviceToHost, stream_), "d2h");
    LS_TRY(cudaStreamSynchronize(stream_), "fim sync");
    if (h_counts_[11]) {
      status_ = 3;
      return "a geometry slab copy wait of the FIM kernel timed out";
    }
    if (h_counts_[0] == 0) break;
    if (launched >= cfg_.max_fim_iters) {
      status_ = 3;
      return "FIM did not converge within max_fim_iters iterations";
    }
  }
  return "";
}

std::string Solver::one_step(bool* empty_nb) {
  *empty_nb = false;
  auto prof = [&](int kind, auto&& fn) -> cudaError_t {
    if (!cfg_.profile) return fn();
    ProfEvent pe;
    cudaError_t e = prof_begin(pe, kind);
    if (e != cudaSuccess) return e;
    cudaEventRecord(pe.a, stream_);
    e = fn();
    cudaEventRecord(pe.b, stream_);
    prof_.push_back(pe);
    return e;
  };
  if (net_ || collect_) return learned_step(empty_nb);
  if (graph_exec_ && !cfg_.profile) {
    LS_TRY(cudaGraphLaunch(graph_exec_, stream_), "graph launch");
    LS_TRY(cudaMemcpyAsync(h_counts_, s_.counts, sizeof(int) * 8, cudaMemcpyDeviceToHost, stream_), "d2h");
    LS_TRY(cudaMemcpyAsync(h_counts_ + 8, s_.ctl, sizeof(int) * 4, cudaMemcpyDeviceToHost, stream_), "d2h");
    LS_TRY(cudaStreamSynchronize(stream_), "step sync");
    const int bodies = h_counts_[8];
    st_.kernel_launches += persistent_ ? 5LL + (cfg_.update_kind != 2 ? 2LL * cfg_.inside_niter : 0)
                                       : 5LL + (3LL * cfg_.graph_chunk + 1) * bodies +
                                             (cfg_.update_kind != 2 ? 2LL * cfg_.inside_niter : 0);
    if (h_counts_[11]) {
      status_ = 3;
      return h_counts_[11] == 1 ? "a grid barrier wait of the persistent FIM kernel timed out"
                                : "a geometry slab copy wait of the FIM kernel timed out";
    }
    if (h_counts_[9]) {
      status_ = 3;
      return "FIM did not converge within max_fim_iters iterations";
    }
    have_nb_ = h_counts_[3] != 0;
    *empty_nb = !have_nb_;
    return "";
  }
  const int use_all = have_nb_ ? 0 : 1;
  if (persistent_) {
    // the persistent step launch by launch (profiled: the FIM loop kernel's
    // time is recorded as the sweep time)
    ProfEvent pe{};
    if (cfg_.profile) LS_TRY(prof_fim_begin(pe, 0), "event");
    LS_TRY(step_persistent_launches(use_all), "persistent step");
    if (cfg_.profile) LS_TRY(prof_fim_end(pe), "event");
    LS_TRY(cudaMemcpyAsync(h_counts_, s_.counts, sizeof(int) * 8, cudaMemcpyDeviceToHost, stream_), "d2h");
    LS_TRY(cudaMemcpyAsync(h_counts_ + 8, s_.ctl, sizeof(int) * 4, cudaMemcpyDeviceToHost, stream_), "d2h");
    LS_TRY(cudaStreamSynchronize(stream_), "step sync");
    st_.kernel_launches += 5LL + (cfg_.update_kind != 2 ? 2LL * cfg_.inside_niter : 0);
    if (h_counts_[11]) {
      status_ = 3;
      return h_counts_[11] == 1 ? "a grid barrier wait of the persistent FIM kernel timed out"
                                : "a geometry slab copy wait of the FIM kernel timed out";
    }
    if (h_counts_[9]) {
      status_ = 3;
      return "FIM did not converge within max_fim_iters iterations";
    }
    have_nb_ = h_counts_[3] != 0;
    *empty_nb = !have_nb_;
    return "";
  }
  LS_TRY(cudaMemsetAsync(s_.counts, 0, sizeof(int) * 3, stream_), "memset");
  LS_TRY(cudaMemsetAsync(s_.counts + 4, 0, sizeof(int), stream_), "memset");
  LS_TRY(K_->reset(m_, s_, sp_, L_, stream_), "reset");
  LS_TRY(cudaMemsetAsync(s_.blabel, 0, sizeof(int) * m_.nparts, stream_), "memset");
  LS_TRY(prof(3, [&] { return K_->seed(m_, s_, use_all, sp_.scale, L_, stream_); }), "seed");
  LS_TRY(cudaMemsetAsync(s_.counts + 3, 0, sizeof(int), stream_), "memset");
  st_.kernel_launches += 4;  // reset, seed, narrowband, step tail
  std::string r = fim_loop(sp_);
  if (!r.empty()) return r;
  LS_TRY(prof(4, [&] { return K_->narrowband(m_, s_, sp_, L_, stream_); }), "narrowband");
  k_step_tail<<<1, 32, 0, stream_>>>(s_.counts, s_.ctl);
  LS_TRY(cudaGetLastError(), "step tail");
  LS_TRY(cudaMemcpyAsync(h_counts_, s_.counts, sizeof(int) * 8, cudaMemcpyDeviceToHost, stream_), "d2h");
  LS_TRY(cudaStreamSynchronize(stream_), "nb sync");
  if (h_counts_[3] == 0) {
    *empty_nb = true;
    have_nb_ = false;
    return "";
  }
  have_nb_ = true;
  if (cfg_.update_kind != 2) {
    for (int it = 0; it < cfg_.inside_niter; ++it) {
      LS_TRY(prof(5, [&] { return K_->update(m_, s_, sp_, L_, stream_); }), "update");
      st_.kernel_launches += 2;  // update, copy-back
    }
  }
  return "";
}

// ---------------------------------------------------------------------------
// Learned warm start.

std::string Solver::learn_buffers() {
  if (X_) return "";
  const Layout& L = *lay_;
  const int nv = m_.nv, d1 = m_.dim + 1;
  // 1-ring from the element copies (each element once), sorted and unique
  std::vector<std::vector<int>> ring(nv);
  std::vector<char> seen(L.ne, 0);
  for (long long c = 0; c < L.full; ++c) {
    const int e = L.ele_permute[c];
    if (seen[e]) continue;
    seen[e] = 1;
    for (int a = 0; a < d1; ++a)
      for (int b = 0; b < d1; ++b)
        if (a != b) ring[L.conn[c * d1 + a]].push_back(L.conn[c * d1 + b]);
  }
  std::vector<int> off(nv + 1, 0), adj;
  for (int v = 0; v < nv; ++v) {
    auto& r = ring[v];
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
    off[v + 1] = off[v] + (int)r.size();
  }
  adj.reserve(off[nv]);
  for (int v = 0; v < nv; ++v) adj.insert(adj.end(), ring[v].begin(), ring[v].end());
  std::vector<void*>& A = allocs_;
  const int* d_off = nullptr;
  const int* d_adj = nullptr;
  LS_TRY(upload(A, &d_off, off, stream_), "upload");
  LS_TRY(upload(A, &d_adj, adj, stream_), "upload");
  adj_off_ = const_cast<int*>(d_off);
  adj_ = const_cast<int*>(d_adj);
  LS_TRY(dalloc(A, &lr_.vlist, nv), "alloc");
  LS_TRY(dalloc(A, &lr_.cnt, 4), "alloc");
  LS_TRY(dalloc(A, &lr_.pred, nv), "alloc");
  LS_TRY(dalloc(A, &lr_.warm, nv), "alloc");
  LS_TRY(dalloc(A, &lr_.target, nv), "alloc");
  LS_TRY(dalloc(A, &X_, (size_t)nv * 128), "alloc");
  lr_.vinv_h = nullptr;
  if (m_.patch_mesh) {
    // a batch: features and targets in units of each vertex's own mesh
    std::vector<float> vinv(nv, 1.f);
    for (int p = 0; p < m_.nparts; ++p)
      for (int v = L.vert_offsets[p]; v < L.vert_offsets[p + 1]; ++v)
        vinv[v] = (float)(1.0 / mesh_scale_[L.patch_mesh[p]]);
    const float* d = nullptr;
    LS_TRY(upload(A, &d, vinv, stream_), "upload");
    lr_.vinv_h = d;
  }
  LS_TRY(cudaStreamSynchronize(stream_), "sync");
  return "";
}

std::string Solver::set_learned(mlp::Net* net, float margin, float tol, bool whole_patch) {
  support_patch_ = whole_patch;
  if (net) {
    std::string r = learn_buffers();
    if (!r.empty()) return r;
  }
  net_ = net;
  margin_ = margin;
  if (tol > 0.f) support_tol_ = tol;
  return "";
}

std::string Solver::set_collect(mlp::Net* net) {
  if (net) {
    std::string r = learn_buffers();
    if (!r.empty()) return r;
  }
  collect_ = net;
  return "";
}

// One time step with the warm start and / or pair collection, launch by
// launch (the support rounds are decided on the host).
std::string Solver::learned_step(bool* empty_nb) {
  *empty_nb = false;
  const bool prev = have_nb_;
  const bool warm = net_ && prev;
  int nb_prev = 0;
  LS_TRY(cudaMemsetAsync(s_.counts, 0, sizeof(int) * 3, stream_), "memset");
  LS_TRY(cudaMemsetAsync(s_.counts + 4, 0, sizeof(int), stream_), "memset");
  LS_TRY(K_->reset(m_, s_, sp_, L_, stream_), "reset");
  if (prev) {
    LS_TRY(cudaMemcpyAsync(h_counts_, s_.counts, sizeof(int) * 8, cudaMemcpyDeviceToHost, stream_), "d2h");
    LS_TRY(cudaStreamSynchronize(stream_), "sync");
    nb_prev = h_counts_[3];
    LS_TRY(cudaMemsetAsync(lr_.cnt, 0, sizeof(int) * 4, stream_), "memset");
    LS_TRY(K_->learn(LEARN_NB_VERTICES, m_, s_, sp_, lr_, nb_prev, 0.f, L_, stream_), "warm set");
    mlp::k_features<<<L_.flat_grid, 256, 0, stream_>>>(0, lr_.vlist, lr_.cnt, adj_off_, adj_, m_.xyz, m_.nv, s_.phi,
                                                        1.f / sp_.scale, lr_.vinv_h, X_);
    LS_TRY(cudaGetLastError(), "features");
    st_.kernel_launches += 2;
    if (warm) {
      std::string r = net_->forward_dev(X_, 0, lr_.cnt, m_.nv, lr_.pred, nullptr, stream_);
      if (!r.empty()) return r;
      LS_TRY(K_->learn(LEARN_WARM, m_, s_, sp_, lr_, 0, margin_, L_, stream_), "warm apply");
      st_.kernel_launches += 2;
    }
  }
  LS_TRY(cudaMemsetAsync(s_.blabel, 0, sizeof(int) * m_.nparts, stream_), "memset");
  if (warm) LS_TRY(K_->learn(LEARN_SEED_WARM, m_, s_, sp_, lr_, 0, 0.f, L_, stream_), "seed");
  else LS_TRY(K_->seed(m_, s_, prev ? 0 : 1, sp_.scale, L_, stream_), "seed");
  LS_TRY(cudaMemsetAsync(s_.counts + 3, 0, sizeof(int), stream_), "memset");
  st_.kernel_launches += 2;
  std::string r = fim_loop(sp_);
  if (!r.empty()) return r;
  if (warm) {
    // support rounds: reset unsupported warm values, FIM again, until none
    const int max_rounds = 16;
    bool clean = false;
    for (int round = 0; round < max_rounds; ++round) {
      LS_TRY(cudaMemsetAsync(s_.counts, 0, sizeof(int) * 3, stream_), "memset");
      LS_TRY(K_->learn(LEARN_SUPPORT, m_, s_, sp_, lr_, support_patch_ ? 1 : 0, support_tol_, L_, stream_),
             "support");
      LS_TRY(cudaMemcpyAsync(h_counts_, s_.counts, sizeof(int) * 8, cudaMemcpyDeviceToHost, stream_), "d2h");
      LS_TRY(cudaStreamSynchronize(stream_), "sync");
      st_.kernel_launches += 1;
      st_.support_rounds++;
      if (h_counts_[0] == 0) {
        clean = true;
        break;
      }
      r = fim_loop(sp_);
      if (!r.empty()) return r;
    }
    if (!clean) {
      // plain FIM from the seeds: the fallback
      st_.learned_fallbacks++;
      LS_TRY(cudaMemsetAsync(s_.counts, 0, sizeof(int) * 3, stream_), "memset");
      LS_TRY(cudaMemcpyAsync(s_.counts + 3, &nb_prev, sizeof(int), cudaMemcpyHostToDevice, stream_), "h2d");
      LS_TRY(K_->reset(m_, s_, sp_, L_, stream_), "reset");
      LS_TRY(cudaMemsetAsync(s_.blabel, 0, sizeof(int) * m_.nparts, stream_), "memset");
      LS_TRY(K_->seed(m_, s_, 0, sp_.scale, L_, stream_), "seed");
      LS_TRY(cudaMemsetAsync(s_.counts + 3, 0, sizeof(int), stream_), "memset");
      r = fim_loop(sp_);
      if (!r.empty()) return r;
    }
    LS_TRY(K_->learn(LEARN_MOVED, m_, s_, sp_, lr_, 0, 1e-3f, L_, stream_), "moved");
    st_.kernel_launches += 1;
  }
  LS_TRY(K_->narrowband(m_, s_, sp_, L_, stream_), "narrowband");
  k_step_tail<<<1, 32, 0, stream_>>>(s_.counts, s_.ctl);
  LS_TRY(cudaGetLastError(), "step tail");
  st_.kernel_launches += 2;
  if (collect_ && prev) {
    LS_TRY(K_->learn(LEARN_TARGETS, m_, s_, sp_, lr_, 0, 1.f / sp_.scale, L_, stream_), "targets");
    st_.kernel_launches += 1;
    long long added = 0;
    r = collect_->append_pairs(X_, lr_.target, lr_.cnt, m_.nv, stream_, &added);
    if (!r.empty()) return r;
    st_.pairs_collected += added;
  }
  LS_TRY(cudaMemcpyAsync(h_counts_, s_.counts, sizeof(int) * 8, cudaMemcpyDeviceToHost, stream_), "d2h");
  LS_TRY(cudaMemcpyAsync(h_counts_ + 8, lr_.cnt, sizeof(int) * 4, cudaMemcpyDeviceToHost, stream_), "d2h");
  LS_TRY(cudaStreamSynchronize(stream_), "sync");
  if (warm) {
    st_.warm_vertices += h_counts_[8];
    st_.unsupported_resets += h_counts_[9];
    st_.moved_vertices += h_counts_[10];
  }
  if (h_counts_[3] == 0) {
    *empty_nb = true;
    have_nb_ = false;
    return "";
  }
  have_nb_ = true;
  if (cfg_.update_kind != 2) {
    for (int it = 0; it < cfg_.inside_niter; ++it) {
      LS_TRY(K_->update(m_, s_, sp_, L_, stream_), "update");
      st_.kernel_launches += 2;
    }
  }
  return "";
}

// The work counters and the profiled launch times are read from the device
// when a caller asks for them (stats), not after every step: a step through
// host buffers then ends with its own result copy and no second round trip.
void Solver::pull_stats() {
  if (cudaMemcpyAsync(h_stats_, s_.stats, sizeof(unsigned long long) * 9, cudaMemcpyDeviceToHost, stream_) !=
          cudaSuccess ||
      cudaStreamSynchronize(stream_) != cudaSuccess)
    return;
  stats_stale_ = false;
  st_.patch_visits = (long long)h_stats_[0];
  st_.check_visits = (long long)h_stats_[1];
  st_.nb_vertex_updates = (long long)h_stats_[2];
  st_.nb_patch_vertices = (long long)h_stats_[3];
  st_.nb_patches = (long long)h_stats_[4];
  st_.fim_iters = (long long)h_stats_[5];
  st_.sweep_slab_bytes = (long long)h_stats_[7];
  st_.flagged_copies = (long long)h_stats_[6];
  st_.early_visits = (long long)h_stats_[8];
  fold_prof(true);
}

std::string Solver::run(int nsteps, float* history, int* steps_done) {
  int done = 0;
  if (history) {
    LS_TRY(K_->unpermute(m_, s_.phi, d_tmp_, L_, stream_), "unpermute");
    LS_TRY(cudaMemcpyAsync(h_stage_, d_tmp_, sizeof(float) * m_.nv, cudaMemcpyDeviceToHost, stream_), "d2h");
    LS_TRY(cudaStreamSynchronize(stream_), "sync");
    std::memcpy(history, h_stage_, sizeof(float) * m_.nv);
  }
  LS_TRY(cudaEventRecord(ev0_, stream_), "event");
  for (int s = 0; s < nsteps; ++s) {
    bool empty = false;
    std::string r = one_step(&empty);
    if (!r.empty()) return r;
    if (cfg_.profile) fold_prof(true);
    if (empty) break;
    done++;
    if (history) {
      LS_TRY(K_->unpermute(m_, s_.phi, d_tmp_, L_, stream_), "unpermute");
      LS_TRY(cudaMemcpyAsync(h_stage_, d_tmp_, sizeof(float) * m_.nv, cudaMemcpyDeviceToHost, stream_), "d2h");
      LS_TRY(cudaStreamSynchronize(stream_), "sync");
      std::memcpy(history + (size_t)(s + 1) * m_.nv, h_stage_, sizeof(float) * m_.nv);
    }
  }
  LS_TRY(cudaEventRecord(ev1_, stream_), "event");
  LS_TRY(cudaEventSynchronize(ev1_), "event sync");
  float ms = 0;
  cudaEventElapsedTime(&ms, ev0_, ev1_);
  st_.ms_total += ms;
  st_.steps_run += done;
  if (steps_done) *steps_done = done;
  stats_stale_ = true;
  return "";
}

std::string Solver::step_host(const float* phi_in, float* phi_out) {
  const int nv = m_.nv;
  if (pageable_) {
    // the GPU reads and writes the caller's pageable host arrays directly
    // (coherent access over the CPU-GPU link): the permutation kernels read
    // and write the caller's side in its order (coalesced) and scatter or
    // gather on the device side, with no staging copy on either side
    LS_TRY(K_->permute(m_, phi_in, s_.phi, L_, stream_), "permute in");
  } else {
    std::memcpy(h_stage_, phi_in, sizeof(float) * nv);
    LS_TRY(cudaMemcpyAsync(d_tmp_, h_stage_, sizeof(float) * nv, cudaMemcpyHostToDevice, stream_), "h2d");
    LS_TRY(K_->permute(m_, d_tmp_, s_.phi, L_, stream_), "permute");
  }
  st_.kernel_launches += 2;  // permute, unpermute
  bool empty = false;
  std::string r = one_step(&empty);
  if (!r.empty()) return r;
  if (cfg_.profile) fold_prof(true);
  if (pageable_) {
    LS_TRY(K_->unpermute(m_, s_.phi, phi_out, L_, stream_), "unpermute out");
    LS_TRY(cudaStreamSynchronize(stream_), "sync");
  } else {
    LS_TRY(K_->unpermute(m_, s_.phi, d_tmp_, L_, stream_), "unpermute");
    LS_TRY(cudaMemcpyAsync(h_stage_, d_tmp_, sizeof(float) * nv, cudaMemcpyDeviceToHost, stream_), "d2h");
    LS_TRY(cudaStreamSynchronize(stream_), "sync");
    std::memcpy(phi_out, h_stage_, sizeof(float) * nv);
  }
  if (!empty) st_.steps_run++;
  stats_stale_ = true;
  return "";
}

std::string Solver::eikonal(const int* seeds, const float* values, int nseeds, float* out) {
  if (m_.patch_mesh) {
    status_ = 1;
    return "the standalone eikonal solve takes one mesh, not a batch";
  }
  const Layout& L = *lay_;
  const int nv = m_.nv, np = m_.nparts;
  const float LN = sp_.largenum;
  std::vector<float> dt(nv, LN);
  std::vector<uint8_t> sd(nv, 0);
  std::vector<int> act;
  for (int i = 0; i < nseeds; ++i) {
    const int v = L.vert_ipermute[seeds[i]];
    const float a = values[i];
    dt[v] = (a >= LN) ? LN : a / sp_.scale;
    sd[v] = 1;
  }
  // first active list: the patches one of whose element copies holds a seed
  // (the list the seed kernel makes at the start of a time step)
  const int d1 = m_.dim + 1;
  for (int p = 0; p < np; ++p) {
    bool hit = false;
    for (int c = L.ele_offsets[p]; c < L.ele_offsets[p + 1] && !hit; ++c)
      for (int k = 0; k < d1; ++k) hit |= sd[L.conn[(size_t)c * d1 + k]] != 0;
    if (hit) act.push_back(p);
  }
  int counts[8] = {(int)act.size(), 0, 0, 0, 0, 0, 0, 0};
  LS_TRY(cudaMemcpyAsync(s_.DT, dt.data(), sizeof(float) * nv, cudaMemcpyHostToDevice, stream_), "h2d");
  LS_TRY(cudaMemcpyAsync(s_.seed, sd.data(), nv, cudaMemcpyHostToDevice, stream_), "h2d");
  if (!act.empty())
    LS_TRY(cudaMemcpyAsync(s_.list0, act.data(), sizeof(int) * act.size(), cudaMemcpyHostToDevice, stream_), "h2d");
  LS_TRY(cudaMemcpyAsync(s_.counts, counts, sizeof(counts), cudaMemcpyHostToDevice, stream_), "h2d");
  LS_TRY(cudaMemsetAsync(s_.blabel, 0, sizeof(int) * np, stream_), "memset");
  LS_TRY(cudaMemsetAsync(s_.ctl + 2, 0, sizeof(int), stream_), "memset");
  StepParams sp = sp_;
  // no narrowband limit: every converged patch that the front has reached
  // (minimum below LARGENUM) activates its neighbours
  sp.bandwidth = LN;
  std::string r = fim_loop(sp);
  if (!r.empty()) return r;
  if (cfg_.profile) fold_prof(true);
  LS_TRY(cudaMemcpyAsync(dt.data(), s_.DT, sizeof(float) * nv, cudaMemcpyDeviceToHost, stream_), "d2h");
  LS_TRY(cudaStreamSynchronize(stream_), "sync");
  for (int v = 0; v < nv; ++v) out[L.vert_permute[v]] = (dt[v] >= LN) ? LN : dt[v] * sp_.scale;
  have_nb_ = false;  // the step state was overwritten
  stats_stale_ = true;
  return "";
}

std::string Solver::set_phi(const float* phi_orig) {
  std::memcpy(h_stage_, phi_orig, sizeof(float) * m_.nv);
  LS_TRY(cudaMemcpyAsync(d_tmp_, h_stage_, sizeof(float) * m_.nv, cudaMemcpyHostToDevice, stream_), "h2d");
  LS_TRY(K_->permute(m_, d_tmp_, s_.phi, L_, stream_), "permute");
  LS_TRY(cudaMemsetAsync(s_.ctl + 2, 0, sizeof(int), stream_), "memset");
  LS_TRY(cudaStreamSynchronize(stream_), "sync");
  have_nb_ = false;
  return "";
}

std::string Solver::get_phi(float* phi_orig) {
  LS_TRY(K_->unpermute(m_, s_.phi, d_tmp_, L_, stream_), "unpermute");
  LS_TRY(cudaMemcpyAsync(h_stage_, d_tmp_, sizeof(float) * m_.nv, cudaMemcpyDeviceToHost, stream_), "d2h");
  LS_TRY(cudaStreamSynchronize(stream_), "sync");
  std::memcpy(phi_orig, h_stage_, sizeof(float) * m_.nv);
  return "";
}

std::string Solver::narrowband(unsigned char* flags) {
  LS_TRY(cudaMemcpyAsync(h_counts_, s_.counts, sizeof(int) * 8, cudaMemcpyDeviceToHost, stream_), "d2h");
  LS_TRY(cudaStreamSynchronize(stream_), "sync");
  const int n = h_counts_[3];
  std::vector<int> nb(n > 0 ? n : 1);
  if (n > 0) LS_TRY(cudaMemcpy(nb.data(), s_.nblist, sizeof(int) * n, cudaMemcpyDeviceToHost), "d2h");
  std::memset(flags, 0, m_.nparts);
  for (int i = 0; i < n; ++i) flags[nb[i]] = 1;
  return "";
}

std::string Solver::active_patches(std::vector<int>& out) {
  LS_TRY(cudaMemcpyAsync(h_counts_, s_.counts, sizeof(int) * 8, cudaMemcpyDeviceToHost, stream_), "d2h");
  LS_TRY(cudaStreamSynchronize(stream_), "sync");
  out.assign(h_counts_[0], 0);
  if (h_counts_[0] > 0) LS_TRY(cudaMemcpy(out.data(), s_.list0, sizeof(int) * h_counts_[0], cudaMemcpyDeviceToHost), "d2h");
  for (int& p : out) p &= ~kPrevisited;
  return "";
}

std::string Solver::dt_values(float* dt) {
  LS_TRY(cudaStreamSynchronize(stream_), "sync");
  LS_TRY(cudaMemcpy(dt, s_.DT, sizeof(float) * m_.nv, cudaMemcpyDeviceToHost), "d2h");
  return "";
}

void Solver::stats(SolverStats& s) {
  if (stats_stale_) pull_stats();
  s = st_;
}

void Solver::reset_stats() {
  cudaMemsetAsync(s_.stats, 0, sizeof(unsigned long long) * 9, stream_);
  cudaStreamSynchronize(stream_);
  // launch times recorded before the reset are dropped with the counters
  fold_prof(false);
  launch_log_.clear();
  st_ = SolverStats();
  stats_stale_ = false;
}

}  // namespace lsgb
