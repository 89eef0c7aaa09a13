/*
 * lsgb300.h -- C ABI of the GB300-native narrowband level-set time step.
 *
 * This is the drop-in boundary for the hot path of GPUTUM Level-Set
 * (HongLi15/SCI-Solver_Level-Set): the narrowband time step on partitioned
 * triangle / tetrahedral patches (seed -> fast-iterative-method redistance ->
 * advection or mean-curvature update).  Plain C types only; the caller owns
 * every array it passes and may free it after the call returns.  A handle is
 * not thread-safe; each handle owns one CUDA stream on the current device.
 * Every entry point returns an ls_status; ls_last_error() gives the reason.
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   LevelSet::LevelSet / ~LevelSet            src/LevelSet.cu:4-33
 *   LevelSet public parameters                src/LevelSet.h:49-60
 *   LevelSet::initializeMesh                  src/LevelSet.cu:111-144
 *   LevelSet::initializeVertices              src/LevelSet.cu:52-80
 *   LevelSet::initializeAdvection             src/LevelSet.cu:82-109
 *   meshFIM3d::Partition_METIS / GraphPartition_Square (partition input)
 *                                             src/core3d/cuda/meshFIM3d.cu:269-421
 *   meshFIM3d::InitPatches / InitPatches2 / GenerateBlockNeighbors
 *                                             src/core3d/cuda/meshFIM3d.cu:423-570
 *   LevelSet::solveLevelSet -> meshFIM3d::GenerateData (per-step loop)
 *                                             src/LevelSet.cu:146-243,
 *                                             src/core3d/cuda/meshFIM3d.cu:572-690
 *   redistance3d::FindSeedPoint / ReInitTsign / GenerateData
 *                                             src/core3d/cuda/redistance3d.cu:10-274
 *   meshFIM3d::updateT_single_stage_d (advection)
 *                                             src/core3d/cuda/meshFIM3d.cu:83-99
 *   meshFIM3d::updateT_single_stage (curvature; host-only in the reference)
 *                                             src/core3d/cuda/meshFIM3d.cu:103-267
 *   LevelSet::getResultAtIteration / numIterations
 *                                             src/LevelSet.cu:35-38
 *   2D twins                                  src/core2d/cuda/meshFIM2d.cu:93-128,676-863,
 *                                             src/core2d/cuda/redistance.cu:10-339
 */
#ifndef LSGB300_H
#define LSGB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum ls_status {
  LS_OK = 0,
  LS_BAD_INPUT = 1,         /* wrong sizes / indices / order of calls       */
  LS_PATCH_TOO_LARGE = 2,   /* a patch exceeds 1024 element copies          */
  LS_DEVICE_TIMEOUT = 3,    /* the FIM loop exceeded max_fim_iters          */
  LS_CUDA_ERROR = 4,        /* a CUDA call failed                           */
  LS_NOT_READY = 5,         /* ls_setup has not run                         */
  LS_NO_MEMORY = 6          /* device or host allocation failed             */
} ls_status;

/* Update applied after the redistance of each step. */
enum { LS_UPDATE_ADVECT = 0, LS_UPDATE_CURVATURE = 1, LS_UPDATE_NONE = 2 };

/* Flags. */
enum {
  /* Reproduce the reference's arithmetic choices: absolute SMALLNUM in the
   * tet solver and convergence test, patch-constant velocity (3D), the 2D
   * velocity replaced by (phi0, phi1)/|grad phi|, and the reference host
   * curvature formula (sigma = (1,0,1) gate, no mass-lumping factor). */
  LS_REF_COMPAT = 1u << 0,
  /* Precision form: a tet local solve whose quadratic discriminant cancels
   * in FP32 (|q^2 - 4pr| <= fp64_threshold * (q^2 + |4pr|)) is repeated in
   * FP64; all other arithmetic stays FP32. */
  LS_FP64_FLAGGED = 1u << 1,
  /* Record per-kernel CUDA-event timings (ls_get_stats). */
  LS_PROFILE = 1u << 2,
  /* Do not run the time step as one CUDA graph (launch kernel by kernel;
   * the host checks the active list every graph_chunk FIM iterations). */
  LS_NO_GRAPH = 1u << 3,
  /* Use the bit-exact kernel build (no FMA contraction; every float
   * operation individually rounded in the reference's order).  Slower;
   * reproduces the CPU restatement of the reference bit for bit. */
  LS_BITEXACT = 1u << 4,
  /* ls_step_host: stage host arrays through pinned buffers even where the
   * GPU can access pageable host memory directly (the default there). */
  LS_HOST_STAGING = 1u << 5,
  /* Run every FIM iteration of a time step in one cooperative (all CTAs
   * resident) launch, the sweep, schedule and check passes separated by
   * grid-wide barriers, instead of three launches per iteration.  Same
   * results.  Applies where the step's sweep kernel has a persistent form
   * (the two-copies-per-thread tet sweep; the one-copy sweep of up to 384
   * threads); elsewhere it is ignored.  A barrier wait that exceeds
   * barrier_wait_limit polls abandons the step with LS_DEVICE_TIMEOUT. */
  LS_PERSISTENT = 1u << 6
};

typedef struct ls_params {
  /* reference LevelSet fields (src/LevelSet.h:51-58, defaults LevelSet.cu:4-22) */
  int num_steps;          /* numSteps_         (10)   */
  double time_step;       /* timeStep_         (1.0)  */
  int inside_iterations;  /* insideIterations_ (1)    */
  int block_size;         /* blockSize_        (16)   structured partition block side */
  int side_lengths;       /* sideLengths_      (1)    structured partition side       */
  double bandwidth;       /* bandwidth_        (16.0) */
  int metis_size;         /* metisSize_        (16)   target vertices per graph patch */
  int partition_type;     /* partitionType_    (0)    1 structured blocks; otherwise patches
                           * of metis_size vertices: 2 recursive coordinate bisection,
                           * any other value (the reference's METIS path) recursive
                           * graph bisection (ls_partition_graph) */
  int verbose;            /* verbose_          (0)    */
  /* extensions */
  int update_kind;        /* LS_UPDATE_*       (ADVECT) */
  double curv_coeff;      /* curvature coefficient (1.0) */
  unsigned flags;         /* LS_* flags        (0)    */
  int fim_sweeps;         /* sweeps per patch visit (0 -> 5 in 3D, 10 in 2D) */
  int max_fim_iters;      /* FIM iterations per step before LS_DEVICE_TIMEOUT (0 -> 100000) */
  double smallnum;        /* 0 -> 1e-5 */
  double largenum;        /* 0 -> 1e9  */
  double length_scale;    /* FIM length unit when not LS_REF_COMPAT (0 -> mean edge length) */
  double fp64_threshold;  /* LS_FP64_FLAGGED: discriminant cancellation threshold tau (0 -> 2^-18) */
  int graph_chunk;        /* FIM iterations per loop body of the step graph (0 -> 4, rounded up to even) */
  int fim_ctas_per_sm;    /* FIM CTAs per SM for patches of <= 384 copies: 2, 3 or 4 with one element copy
                             per thread; 5 or 6: two copies per thread, five CTAs per SM (64 registers) or
                             six (56 registers); 7: the same kernel with one copy per thread, three CTAs
                             per SM (shorter visits when the lists are short) (tetrahedra without the
                             precision form; others run 3) (0 -> 5) */
  int barrier_wait_limit; /* LS_PERSISTENT: polls (about 0.25 us apart) one grid-barrier wait may take
                             before the step is abandoned with LS_DEVICE_TIMEOUT (0 -> 4194304, about a
                             second).  The FIM kernel's wait for its geometry slab copies is bounded by
                             about a second of SM clock cycles.  Negative: every such wait gives up at
                             its first check (a setting for testing the timeout paths) */
} ls_params;

typedef struct ls_stats {
  int steps_run;
  long long fim_iters;          /* FIM outer iterations, all steps          */
  long long patch_visits;       /* patch sweeps (NITER sweeps each)         */
  long long check_visits;       /* neighbour checks (one sweep each)        */
  long long nb_vertex_updates;  /* sum over steps of #{v : |phi(v)| <= w}   */
  long long nb_patch_vertices;  /* sum over steps of sum_{p in NB} nv_p     */
  long long nb_patches;         /* sum over steps of |NB|                   */
  long long flagged_copies;     /* local solves repeated in FP64 (precision form) */
  double ms_total;              /* device time of ls_step / ls_solve calls  */
  /* LS_PROFILE only: per-kernel device time (ms) and launches */
  double ms_sweep, ms_check, ms_schedule, ms_seed, ms_narrowband, ms_update;
  long long n_sweep, n_check, n_schedule, n_seed, n_narrowband, n_update;
  long long sweep_slab_bytes;   /* algorithmic bytes read+written by the FIM patch kernel (visits and checks) */
  long long kernel_launches;    /* kernels launched (graph kernels included) */
  /* learned warm start (ls_set_learned) */
  long long warm_vertices;      /* vertices started from the network's prediction */
  long long unsupported_resets; /* warm values below their local-solve support, reset */
  long long support_rounds;     /* support checks run */
  long long moved_vertices;     /* warm vertices the FIM moved by more than 1e-3 h */
  long long learned_fallbacks;  /* steps redone as plain FIM after 16 support rounds */
  long long pairs_collected;    /* training pairs recorded (ls_learn_collect) */
  long long early_visits;       /* patch visits run by the neighbour check that activated the patch
                                   (fast build, tetrahedra; counted in patch_visits too) */
} ls_stats;

typedef struct ls_handle ls_handle;

ls_status ls_default_params(ls_params* p);
/* LevelSet(bool isTriMesh, ...): src/LevelSet.cu:4-22 */
ls_status ls_create(ls_handle** h, int is_tri);
/* ~LevelSet: src/LevelSet.cu:24-33 */
ls_status ls_destroy(ls_handle* h);
ls_status ls_set_params(ls_handle* h, const ls_params* p);
ls_status ls_get_params(ls_handle* h, ls_params* p);
/* initializeMesh: xyz nv*3 floats, elems ne*(3|4) ints (0-based). */
ls_status ls_set_mesh(ls_handle* h, const float* xyz, int nv, const int* elems, int ne);
/* initializeMesh from a file (src/LevelSet.cu:111-144): tetgen .node/.ele
 * (basename or either file) for tet handles, ASCII PLY for triangle handles
 * (polygons are split into triangle fans).  Tets with negative signed
 * volume get their last two vertices swapped (TetMesh::reorient, called at
 * src/LevelSet.cu:139). */
ls_status ls_load_mesh(ls_handle* h, const char* filename);
ls_status ls_get_mesh_info(ls_handle* h, int* nv, int* ne);
ls_status ls_get_mesh(ls_handle* h, float* xyz, int* elems);
/* writeVTK for one phi (meshFIM3d.cu:48-81): legacy VTK unstructured grid,
 * POINT_DATA "traveltime". */
ls_status ls_write_vtk(ls_handle* h, const char* path, const float* phi);
/* Partition input (replaces Partition_METIS / GraphPartition_Square):
 * npart nv ints in [0, nparts).  Optional; ls_setup partitions otherwise. */
ls_status ls_set_partition(ls_handle* h, const int* npart, int nparts);
/* initializeVertices: phi nv floats in the caller's vertex order. */
ls_status ls_set_phi(ls_handle* h, const float* phi);
/* initializeAdvection: vel ne*3 floats, one vector per element. */
ls_status ls_set_velocity(ls_handle* h, const float* vel);
/* Host part of the preprocessing only (partition if not given, default phi
 * and velocity, patch layout); no device work.  ls_setup calls it. */
ls_status ls_prepare(ls_handle* h);
/* Preprocessing of GenerateData (meshFIM3d.cu:592-629): partition (if not
 * given), patch layout, device upload.  Allocates all device memory. */
ls_status ls_setup(ls_handle* h);
/* GenerateData's time loop (meshFIM3d.cu:639-678): nsteps steps from the
 * current phi.  history (optional): (nsteps+1)*nv floats, row 0 = phi at
 * entry, row s = phi after step s (caller's vertex order), copied to the host
 * after every step as the reference does.  Stops early when the narrowband
 * is empty (meshFIM3d.cu:655-659); *steps_done reports the steps run. */
ls_status ls_solve(ls_handle* h, int nsteps, float* history, int* steps_done);
/* Device-resident steps: no host copies of phi. */
ls_status ls_step(ls_handle* h, int nsteps, int* steps_done);
/* End-to-end step through host buffers: phi_in (nv floats, host) is copied
 * to the device, one step runs, phi_out (host) receives the result. */
ls_status ls_step_host(ls_handle* h, const float* phi_in, float* phi_out);
/* Standalone eikonal solve (the fast iterative method of the redistance,
 * without the narrowband limit): distance from the given seed vertices
 * (caller order, seed values >= 0) over the whole mesh, unit speed.  dist:
 * nv floats, LARGENUM where unreached.  Overwrites the step state: the next
 * step searches seeds in every patch. */
ls_status ls_eikonal(ls_handle* h, const int* seeds, const float* values, int nseeds, float* dist);
/* Current phi in the caller's vertex order. */
ls_status ls_get_phi(ls_handle* h, float* phi);
/* Work counters and profiled kernel times since the last ls_reset_stats.
 * The device-side counters are read here (one small copy and a wait on the
 * handle's stream when a step ran since the previous read), not after every
 * step. */
ls_status ls_get_stats(ls_handle* h, ls_stats* s);
/* Zeroes the counters and drops profiled kernel times not yet read. */
ls_status ls_reset_stats(ls_handle* h);
/* Per-launch record of the FIM patch kernel (no counterpart in the
 * reference, whose host loop times nothing): for every sweep and check
 * launch of the profiled steps (LS_PROFILE / ls_set_profile) since the last
 * ls_reset_stats, oldest first, its kind (0 sweep, or the whole FIM loop of
 * a step with LS_PERSISTENT; 1 neighbour check), its device time in ms
 * (CUDA events on the handle's stream) and its algorithmic slab bytes (the
 * per-visit bytes of every patch visit and check it ran; -1 past 4,096
 * launches in one step).  Copies min(cap, available) records into the
 * caller's arrays (any of them may be NULL) and the number available into
 * *n.  At most 2^20 records are kept. */
ls_status ls_get_launch_log(ls_handle* h, int cap, int* kinds, double* ms, long long* bytes, int* n);
/* Turn per-kernel CUDA-event timing on or off for the following steps
 * (kernels are then launched one by one instead of from the graph). */
ls_status ls_set_profile(ls_handle* h, int on);
/* Narrowband of the last step: one byte per patch. */
ls_status ls_get_narrowband(ls_handle* h, unsigned char* flags);
/* Diagnostics: the current FIM active list (patch ids, at most cap) and,
 * if dt is given, the FIM distance values in the layout's vertex order
 * (nv floats, FIM frame units). */
ls_status ls_debug_active(ls_handle* h, int* list, int cap, int* count, float* dt);
/* info[0..9] = nparts, full, lep, lvp, lgp, lim, nadj, nv, ne, dim */
ls_status ls_get_layout_info(ls_handle* h, long long* info);
/* Reference-format layout arrays (LS_REF_* below) for bit-exact checks. */
ls_status ls_get_layout(ls_handle* h, int which, void* dst);
const char* ls_last_error(ls_handle* h);
const char* ls_version(void);

/* Layout array selectors for ls_get_layout (meshFIM3d members). */
enum {
  LS_REF_ELE_PERMUTE = 0,          /* int[full]           ele_permute          */
  LS_REF_ELE_OFFSETS = 1,          /* int[nparts+1]       m_ele_offsets_d      */
  LS_REF_VERT_PERMUTE = 2,         /* int[nv]             m_vert_permute_d     */
  LS_REF_VERT_OFFSETS = 3,         /* int[nparts+1]       m_vert_offsets_d     */
  LS_REF_ELE_AFTER_PERMUTE = 4,    /* int[(d+1)*full]     m_ele_after_permute_d*/
  LS_REF_MEM_LOCATIONS = 5,        /* int[(d+1)*full]     m_mem_locations      */
  LS_REF_MEM_LOCATION_OFFSETS = 6, /* int[nv+1]           m_mem_location_offsets */
  LS_REF_BLOCK_XADJ = 7,           /* int[nparts+1]       m_block_xadj_d       */
  LS_REF_BLOCK_ADJNCY = 8,         /* int[nadj]           m_block_adjncy_d     */
  LS_REF_LOCAL_COORDS = 9,         /* float[6|3 * full]   m_ele_local_coords_d */
  LS_REF_VERT_IPERMUTE = 10        /* int[nv]             vert_ipermute        */
};

/* Narrowband selection without any device allocation.  No counterpart in
 * the reference: it is the solver's narrowband kernel (narrowband patches,
 * phi = +-DT * scale, vertex-update count) for callers that cannot call
 * cudaMalloc -- host applications that own all device memory through their
 * own pool, or that run under a fixed device-memory budget, so that an
 * allocation inside the call would take memory already handed out or fail.
 * All pointers except `counts` are device pointers owned by the caller:
 *   vert_offsets  nparts+1 ints, patch ranges of the vertices (layout
 *                 order); must start at 0, never decrease and end at most at
 *                 nv (the offsets live on the device and are not checked:
 *                 other values make the kernel read and write outside dt,
 *                 sign and phi)
 *   dt            nv floats, FIM distances in the FIM frame (any value;
 *                 the patch minimum compares them as floats, -0.0 and
 *                 negative values included)
 *   sign          nv bytes, 1 where phi >= 0 before the redistance
 *   phi           nv floats, output: +-DT * scale (+-DT where DT >= largenum)
 *   nb_flags      nparts bytes, output: 1 for narrowband patches
 *   counts        host, 3 long longs, output: narrowband patches, vertex
 *                 updates (DT <= bandwidth), vertices of narrowband patches
 * stream is a cudaStream_t (NULL = default stream); the call synchronises it.
 * Scratch (the compact patch list and the counters) is a file-scope device
 * array of LS_NOALLOC_MAX_PATCHES + 64 ints (about 4 MB), held by every GPU
 * that loads the library until exit; nparts above the limit is rejected
 * with LS_BAD_INPUT.  The first call on a device looks up the array's device
 * address (make it before any stream capture).  The array is shared by all
 * calls and keeps the last call's contents (counters are cleared per call):
 * calls that overlap on the GPU race. */
#define LS_NOALLOC_MAX_PATCHES (1 << 20)
ls_status ls_narrowband_noalloc(int nv, int nparts, const int* vert_offsets, const float* dt,
                                const unsigned char* sign, float bandwidth, float scale, float largenum,
                                float* phi, unsigned char* nb_flags, long long* counts, void* stream);

/* Partitioners.  Structured blocks: GraphPartition_Square semantics
 * (meshFIM3d.cu:316-326, meshFIM2d.cu:346-353) on an x-fastest lattice of
 * side nside (3D: nside^3 vertices, 2D: nside^2), block side block. */
ls_status ls_partition_structured(int dim, int nside, int block, int nv, int* npart, int* nparts);
/* Graph partition stand-in for METIS_PartGraphKway (meshFIM3d.cu:354-421):
 * recursive coordinate bisection into ceil(nv / target) parts (3D) or
 * max(2, nv / target) parts (2D, meshFIM2d.cu:380-382). */
ls_status ls_partition_rcb(int dim, const float* xyz, int nv, int target, int* npart, int* nparts);
/* Graph partition from the mesh connectivity alone (no counterpart in the
 * reference, which calls METIS_PartGraphKway): recursive bisection of the
 * vertex graph by breadth-first level structures from pseudo-peripheral
 * vertices, then greedy boundary refinement that lowers the edge cut within
 * a 3 % size tolerance; same part counts as ls_partition_rcb. */
ls_status ls_partition_graph(int dim, const int* elems, int ne, int nv, int target, int* npart, int* nparts);
/* Mesh edges whose vertices lie in different parts. */
ls_status ls_edge_cut(int dim, const int* elems, int ne, int nv, const int* npart, long long* cut);

/* Autotuner (no counterpart in the reference): times trial_steps steps (after
 * one warm-up step, from the handle's phi0) for each candidate patch size --
 * structured block side 2, 3, 4 (3D) / 4, 5, 6, 8 (2D) when
 * partition_type = 1, patch target size (metis_size) 8, 16, 27, 32, 64 (3D)
 * / 16, 25, 36, 64 (2D) for the graph and RCB partitioners, or only the
 * caller's partition when ls_set_partition was
 * used -- and each FIM setting of fim_ctas_per_sm (2-4; tetrahedra also 5-7;
 * patches of up to 384 element copies), picks the highest narrowband
 * vertex-updates/s, writes it
 * into the handle's parameters (block_size or metis_size,
 * fim_ctas_per_sm) and leaves the handle set up at phi0 with it. */
#define LS_TUNE_MAX_TRIALS 32
typedef struct ls_tune_trial {
  int patch_size;       /* block side or RCB target; 0 = the caller's partition */
  int fim_ctas_per_sm;
  double ms_per_step;
  double updates_per_s;
} ls_tune_trial;
typedef struct ls_tune_report {
  int ntrials;
  int best;             /* index into trials */
  ls_tune_trial trials[LS_TUNE_MAX_TRIALS];
} ls_tune_report;
ls_status ls_autotune(ls_handle* h, int trial_steps, ls_tune_report* rep);

/* Batches of independent meshes (no counterpart in the reference, which
 * solves one mesh per LevelSet and process).  Each member is a handle with
 * its mesh, partition, phi0, velocity and parameters set; ls_batch_add
 * prepares it (ls_prepare) and copies what the batch needs, so the handle
 * may be destroyed afterwards.  The members' patch layouts are merged into
 * one patch set: every FIM iteration, narrowband and update launch covers
 * all members at once, each with its own time step, bandwidth, curvature
 * coefficient and FIM length unit.  Members must share the update kind, the
 * flags (LS_PROFILE aside), fim_sweeps, inside_iterations, smallnum,
 * largenum and fp64_threshold; the first member's graph_chunk,
 * max_fim_iters and fim_ctas_per_sm apply.  A step of the batch is one step
 * of every member; solving stops early only when every member's narrowband
 * is empty, and a member whose narrowband empties earlier keeps the
 * +-LARGENUM values that its empty redistance leaves. */
typedef struct ls_batch ls_batch;
ls_status ls_batch_create(ls_batch** b);
ls_status ls_batch_destroy(ls_batch* b);
const char* ls_batch_last_error(ls_batch* b);
/* index: position of the member (0, 1, ...) */
ls_status ls_batch_add(ls_batch* b, ls_handle* h, int* index);
ls_status ls_batch_setup(ls_batch* b);
ls_status ls_batch_solve(ls_batch* b, int nsteps, int* steps_done);
/* Autotuner of a batch (no counterpart in the reference): as ls_autotune,
 * over the whole batch -- each member laid out again with each candidate
 * patch size (when every member uses the library's partitioner of one
 * type; a caller's partition is kept), each FIM setting timed on the merged
 * patch set for trial_steps steps after one warm-up step -- and leaves the
 * batch set up with the best, every member at its phi0.  Replaces the
 * batch's solver (call it before ls_batch_solve, or ls_batch_setup again
 * after it). */
ls_status ls_batch_autotune(ls_batch* b, int trial_steps, ls_tune_report* rep);
/* phi of one member, in that member's vertex order */
ls_status ls_batch_get_phi(ls_batch* b, int index, float* phi);
ls_status ls_batch_get_stats(ls_batch* b, ls_stats* s);
ls_status ls_batch_reset_stats(ls_batch* b);
ls_status ls_batch_set_profile(ls_batch* b, int on);
/* merged layout (host only; same info[10] and LS_REF_* arrays as
 * ls_get_layout_info / ls_get_layout) */
ls_status ls_batch_get_layout_info(ls_batch* b, long long* info);
ls_status ls_batch_get_layout(ls_batch* b, int which, void* dst);

/* The learned warm start's network (no counterpart in the reference): a
 * 128-128-128-128-1 ReLU MLP with BF16 weights and activations and FP32
 * accumulation on the tcgen05 tensor cores, trained on the GPU (forward,
 * backward and Adam kernels).  Input: 128 features per sample (32 1-ring
 * slots x (dx, dy, dz, phi) / h, slot 0 the vertex itself); output: the
 * signed distance / h after the FIM redistance.  Parameters, fp32, in the
 * order W1 W2 W3 (128 x 128 each, [out][in]), b1 b2 b3 (128 each), w4
 * (128), b4 (1): ls_mlp_num_params() floats.  Loss 1/(2n) sum (y - t)^2. */
typedef struct ls_mlp ls_mlp;
ls_status ls_mlp_create(ls_mlp** m, unsigned long long seed);
ls_status ls_mlp_destroy(ls_mlp* m);
const char* ls_mlp_last_error(ls_mlp* m);
int ls_mlp_num_params(void);
ls_status ls_mlp_set_params(ls_mlp* m, const float* params);
ls_status ls_mlp_get_params(ls_mlp* m, float* params);
/* x: n x 128 floats (rounded to BF16), y: n outputs */
ls_status ls_mlp_predict(ls_mlp* m, const float* x, int n, float* y);
/* gradients of the loss over one batch of n samples (all parameters, same
 * order as the parameters) and the loss */
ls_status ls_mlp_gradients(ls_mlp* m, const float* x, const float* t, int n, float* grad, float* loss);
/* Adam (beta 0.9 / 0.999, eps 1e-8) over epochs passes of the n samples in
 * batches of `batch`; loss = mean batch loss of the last epoch */
ls_status ls_mlp_train(ls_mlp* m, const float* x, const float* t, int n, int epochs, int batch, float lr,
                       float* loss);

/* Training pairs held by the network on the device: (features of a vertex
 * of the previous step's narrowband patches before the redistance, its
 * signed distance / h after it).  ls_learn_collect runs nsteps steps of h
 * (its state advances as with ls_step) recording the pairs of each step
 * into m's pair buffer (capacity ls_mlp_reserve_pairs, 4 Mi pairs by
 * default; overflow is dropped).  ls_mlp_train_pairs shuffles the pairs
 * once and runs Adam over them. */
ls_status ls_mlp_reserve_pairs(ls_mlp* m, long long capacity);
ls_status ls_mlp_clear_pairs(ls_mlp* m);
ls_status ls_mlp_num_pairs(ls_mlp* m, long long* n);
ls_status ls_mlp_train_pairs(ls_mlp* m, int epochs, int batch, float lr, unsigned long long seed, float* loss);
ls_status ls_learn_collect(ls_handle* h, ls_mlp* m, int nsteps, int* steps_done);
/* The network's error on pairs of its buffer (no counterpart in the
 * reference): |prediction - target| in units of h for the pairs [first,
 * first + count), e.g. pairs collected after training from a run the
 * network was not trained on. */
ls_status ls_mlp_eval_pairs(ls_mlp* m, long long first, long long count, float* abs_err);
/* Learned warm start for the steps of h (m = NULL turns it off): the FIM of
 * each step starts the previous narrowband's vertices at |prediction| +
 * margin (units of h, the FIM length unit) instead of LARGENUM, with all
 * those patches active; afterwards every reached vertex whose value lies
 * more than support_tol (units of h; 0 -> 5e-4) below all local solves of
 * its elements is reset to LARGENUM -- with every other non-seed vertex of
 * its patch (reset_mode 0) or alone (reset_mode 1) -- and the FIM runs
 * again, until no such vertex is left (at most 16 rounds, then the step's
 * redistance is redone as plain FIM).  The network is not owned by h and
 * must outlive its use.  Batches: ls_batch_set_learned.  Steps run
 * launch by launch. */
ls_status ls_set_learned(ls_handle* h, ls_mlp* m, double margin, double support_tol, int reset_mode);
/* The learned warm start for the steps of a batch (no counterpart in the
 * reference): as ls_set_learned, with every mesh's features, predictions,
 * margin and tolerances in units of that mesh's own h. */
ls_status ls_batch_set_learned(ls_batch* b, ls_mlp* m, double margin, double support_tol, int reset_mode);

#ifdef __cplusplus
}
#endif
#endif
