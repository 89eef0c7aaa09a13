// ls_solver.h -- device solver behind the C ABI: owns the device copy of the
// patch layout, the step state, the stream and the FIM-iteration graphs.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "ls_device.cuh"
#include "ls_layout.h"
#include "ls_mlp.h"

namespace lsgb {

struct Launch {
  int sms;
  int fim_grid, fim_block, fim_smem;
  int pair_block;  // threads of the two-copies-per-thread sweep kernel (0: not used)
  int persist_grid;  // CTAs of the persistent FIM kernel (all resident; 0: no persistent form here)
  int upd_grid, upd_block, upd_smem;
  int seed_grid;
  int warp_grid;
  int flat_grid;
};

enum { LEARN_NB_VERTICES = 0, LEARN_WARM, LEARN_SEED_WARM, LEARN_SUPPORT, LEARN_MOVED, LEARN_TARGETS };

// One build of the step kernels (fast or bit-exact).
struct KernelSet {
  cudaError_t (*configure)(const DevMesh& m, const StepParams& sp, Launch& L);
  cudaError_t (*reset)(const DevMesh& m, const DevState& s, const StepParams& sp, const Launch& L, cudaStream_t st);
  cudaError_t (*seed)(const DevMesh& m, const DevState& s, int use_all, float scale, const Launch& L, cudaStream_t st);
  cudaError_t (*sweep)(const DevMesh& m, const DevState& s, const StepParams& sp, int cur, bool check,
                       const Launch& L, cudaStream_t st);
  cudaError_t (*schedule)(const DevMesh& m, const DevState& s, const StepParams& sp, int cur, const Launch& L,
                          cudaStream_t st);
  // every FIM iteration of a step in one cooperative launch (L.persist_grid > 0)
  cudaError_t (*fim_persistent)(const DevMesh& m, const DevState& s, const StepParams& sp, const Launch& L,
                                cudaStream_t st);
  cudaError_t (*narrowband)(const DevMesh& m, const DevState& s, const StepParams& sp, const Launch& L,
                            cudaStream_t st);
  cudaError_t (*update)(const DevMesh& m, const DevState& s, const StepParams& sp, const Launch& L, cudaStream_t st);
  cudaError_t (*unpermute)(const DevMesh& m, const float* phi, float* out, const Launch& L, cudaStream_t st);
  cudaError_t (*permute)(const DevMesh& m, const float* in, float* out, const Launch& L, cudaStream_t st);
  // learned warm start / collection kernels (op: LEARN_*)
  cudaError_t (*learn)(int op, const DevMesh& m, const DevState& s, const StepParams& sp, const DevLearn& lr, int arg,
                       float fa, const Launch& L, cudaStream_t st);
  // per-copy geometry records of the two-copies-per-thread sweep (written
  // when L.pair_block > 0; gm: 3 float4 per copy, gh: 1)
  cudaError_t (*geometry)(const DevMesh& m, float4* gm, float4* gh, const Launch& L, cudaStream_t st);
};
const KernelSet& kernels_fast();
const KernelSet& kernels_exact();

struct SolverConfig {
  int update_kind = 0;
  int ref_compat = 0;
  int fp64_flagged = 0;
  int bit_exact = 0;
  int profile = 0;
  int use_graph = 1;
  int niter = 0;
  int inside_niter = 1;
  int max_fim_iters = 100000;
  int graph_chunk = 4;
  int fim_ctas = 3;
  double dt = 1.0;
  double bandwidth = 16.0;
  double curv_coeff = 1.0;
  double smallnum = 1e-5;
  double largenum = 1e9;
  double length_scale = 0.0;
  double fp64_tau = 3.814697265625e-06;  // 2^-18
  int host_staging = 0;  // 1: host arrays go through pinned staging even where the GPU can read pageable memory
  int persistent = 0;    // 1: a step's FIM loop runs as one cooperative launch where the kernel has that form
  int spin_limit = 1 << 22;  // polls of one grid-barrier wait of the persistent kernel (< 0: every FIM
                             // kernel wait gives up at its first check)
  // batches (Layout::patch_mesh set): per-mesh dt, bandwidth, curvature
  // coefficient and FIM length scale (<= 0: the mesh's mean edge)
  std::vector<double> mesh_dt, mesh_bandwidth, mesh_curv, mesh_length_scale;
};

struct SolverStats {
  long long steps_run = 0;
  long long fim_iters = 0, patch_visits = 0, check_visits = 0;
  long long nb_vertex_updates = 0, nb_patch_vertices = 0, nb_patches = 0, flagged_copies = 0;
  double ms_total = 0;
  double ms_sweep = 0, ms_check = 0, ms_schedule = 0, ms_seed = 0, ms_narrowband = 0, ms_update = 0;
  long long n_sweep = 0, n_check = 0, n_schedule = 0, n_seed = 0, n_narrowband = 0, n_update = 0;
  long long sweep_slab_bytes = 0;
  long long kernel_launches = 0;
  // learned warm start
  long long warm_vertices = 0, unsupported_resets = 0, support_rounds = 0, moved_vertices = 0;
  long long learned_fallbacks = 0, pairs_collected = 0;
  long long early_visits = 0;
};

// One profiled FIM launch: 0 sweep (or the persistent FIM loop), 1 check;
// device time; algorithmic slab bytes (-1 when not recorded).
struct LaunchRec {
  int kind;
  double ms;
  long long bytes;
};

class Solver {
 public:
  Solver() = default;
  ~Solver();
  // Upload the layout and the per-copy data; phi0 / vel in the caller's order.
  std::string init(const Layout& L, const SolverConfig& cfg, const float* vel);
  std::string set_phi(const float* phi_orig);          // host, caller order
  std::string get_phi(float* phi_orig);                // host, caller order
  // Run nsteps; history (optional) gets phi after each step (host, caller order).
  std::string run(int nsteps, float* history, int* steps_done);
  std::string step_host(const float* phi_in, float* phi_out);
  // Distance from arbitrary seed vertices (caller order), whole mesh, no
  // narrowband limit; out: nv floats in the caller's order.
  std::string eikonal(const int* seeds, const float* values, int nseeds, float* out);
  std::string narrowband(unsigned char* flags);
  std::string active_patches(std::vector<int>& out);
  std::string dt_values(float* dt_new_order);
  void stats(SolverStats& s);  // reads the device counters if a step ran since the last read
  void reset_stats();
  // FIM launches of the profiled steps since the last reset_stats (oldest
  // first, at most kLaunchLogCap kept)
  const std::vector<LaunchRec>& launch_log() {
    if (stats_stale_) pull_stats();
    return launch_log_;
  }
  static constexpr size_t kLaunchLogCap = 1u << 20;
  int status_code() const { return status_; }
  void set_profile(bool on) { cfg_.profile = on ? 1 : 0; }
  // Learned warm start: each step's FIM starts from |network prediction| +
  // margin (FIM frame) on the previous narrowband, followed by support checks
  // (tolerance tol) until no warm value is left unsupported; net = null turns
  // it off.  Collection: steps record (features, post-redistance phi / h)
  // pairs of the previous narrowband's vertices into net's pair buffer.
  std::string set_learned(mlp::Net* net, float margin, float tol, bool whole_patch);
  std::string set_collect(mlp::Net* net);

 private:
  std::string check(cudaError_t e, const char* what);
  std::string one_step(bool* empty_nb);
  std::string learned_step(bool* empty_nb);
  std::string learn_buffers();
  std::string fim_loop(const StepParams& sp);
  std::string build_graph();
  bool build_persistent_graph(std::string* err);
  cudaError_t step_persistent_launches(int use_all);
  bool persistent_ = false;        // the step's FIM loop is one cooperative launch
  std::vector<double> mesh_scale_;  // FIM length unit of each mesh (one entry for a single mesh)
  void pull_stats();
  bool stats_stale_ = false;  // device counters changed since the last pull_stats
  // event pairs around the launches of profiled steps (cfg_.profile); kind 0
  // sweep, 1 check, 2 schedule, 3 seed, 4 narrowband, 5 update.  Each
  // profiled step folds its pairs into the stats when it ends and returns
  // the events to a pool, so the number of events stays that of one step.
  struct ProfEvent {
    cudaEvent_t a, b;
    int kind;
    int snap = -1;  // FIM launches: slot of the slab-byte counter snapshots around the launch
  };
  std::vector<ProfEvent> prof_;
  std::vector<LaunchRec> launch_log_;
  std::vector<cudaEvent_t> ev_pool_;
  cudaError_t prof_begin(ProfEvent& pe, int kind);
  // profiled FIM launches: the device's slab-byte counter (stats[7]) copied
  // before and after each launch into d_snap_ (slots of 2, at most kSnapCap
  // launches between two folds), read back when the times are folded
  static constexpr int kSnapCap = 4096;
  long long* d_snap_ = nullptr;
  long long* h_snap_ = nullptr;
  int nsnap_ = 0;
  cudaError_t prof_fim_begin(ProfEvent& pe, int kind);
  cudaError_t prof_fim_end(ProfEvent& pe);
  void fold_prof(bool keep_times);

  const Layout* lay_ = nullptr;
  const KernelSet* K_ = nullptr;
  SolverConfig cfg_;
  DevMesh m_{};
  DevState s_{};
  StepParams sp_{};
  Launch L_{};
  cudaStream_t stream_ = nullptr;
  cudaGraphExec_t graph_exec_ = nullptr;
  cudaGraph_t graph_ = nullptr;
  std::vector<void*> allocs_;
  int* h_counts_ = nullptr;           // pinned mirror of s_.counts [0..7] and s_.ctl [8..11]
  unsigned long long* h_stats_ = nullptr;
  float* h_stage_ = nullptr;          // pinned nv floats
  float* d_tmp_ = nullptr;            // nv floats (caller-order staging)
  bool have_nb_ = false;              // previous narrowband valid (seed search restricted)
  int pageable_ = 0;                  // the GPU can access pageable host memory directly
  int status_ = 0;
  SolverStats st_;
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
  // learned warm start
  mlp::Net* net_ = nullptr;      // warm start on when set
  mlp::Net* collect_ = nullptr;  // pair collection on when set
  float margin_ = 0.f, support_tol_ = 5e-4f;
  bool support_patch_ = true;       // reset whole patches on an unsupported vertex
  DevLearn lr_{};
  int* adj_off_ = nullptr;       // vertex 1-ring CSR (product numbering)
  int* adj_ = nullptr;
  __nv_bfloat16* X_ = nullptr;   // features of the warm set
};

}  // namespace lsgb
