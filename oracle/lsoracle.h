/*
 * lsoracle.h -- CPU oracle for the narrowband level-set time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA
 * product path is compared against.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline / reference legs may load it.  The product
 * library never links, loads or calls it.
 *
 * It restates, in plain C, the algorithm of GPUTUM Level-Set
 * (HongLi15/SCI-Solver_Level-Set) for one time step:
 *   layout build   src/core3d/cuda/meshFIM3d.cu:423-570 (+ K2..K8 kernels in
 *                  src/core3d/include/meshFIM_kernels.h:410-659), 2D twin in
 *                  src/core2d/cuda/meshFIM2d.cu:447-607
 *   seeding        src/core3d/include/redistance_kernels3d.h:623-770
 *   FIM schedule   src/core3d/cuda/redistance3d.cu:67-274
 *   patch sweep    src/core3d/include/redistance_kernels3d.h:287-621
 *   local solvers  src/core3d/include/redistance_kernels3d.h:124-285 (tet),
 *                  src/core2d/include/redistance_kernels.h:287-334 (tri)
 *   advection      src/core3d/include/meshFIM_kernels.h:36-408,
 *                  src/core2d/include/meshFIM2d_kernels.h:37-362
 *   curvature      src/core3d/cuda/meshFIM3d.cu:103-267 (host function)
 *   step order     src/core3d/cuda/meshFIM3d.cu:639-678
 *
 * Two arithmetic instantiations exist: 32 (the reference's FP32 3D
 * arithmetic, including its float->double promotions) and 64 (all double;
 * this is the reference's own precision for 2D and the FP64 error oracle
 * for 3D).
 *
 * Parity pins: the local solvers and the host curvature update are checked
 * against the reference's own code compiled from its sources into
 * oracle/_ref (see oracle/build_ref.py) through golden vectors committed in
 * tests/golden/.  The reference ships no golden vectors of its own.
 */
#ifndef LSORACLE_H
#define LSORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  LSO_OK = 0,
  LSO_BAD_INPUT = 1,
  LSO_PATCH_TOO_LARGE = 2,
  LSO_TIMEOUT = 3,
  LSO_NOMEM = 4
};

enum { LSO_ADVECT = 0, LSO_CURVATURE = 1, LSO_NONE = 2 };

typedef struct lso_params {
  int dim;            /* 2 (triangles) or 3 (tetrahedra) */
  int precision;      /* 32 or 64 */
  int ref_compat;     /* 1: reference semantics; 0: corrected semantics */
  int update_kind;    /* LSO_ADVECT / LSO_CURVATURE / LSO_NONE */
  int niter;          /* sweeps per patch visit; 0 -> 5 (3D) / 10 (2D) */
  int inside_niter;   /* update passes per step; 0 -> 1 */
  int max_fim_iters;  /* cap on FIM outer iterations per step; 0 -> 100000 */
  int nthreads;       /* OpenMP threads; 0 -> runtime default */
  double dt;
  double bandwidth;
  double curv_coeff;  /* epsilon of the curvature update */
  double smallnum;    /* 0 -> 1e-5 */
  double largenum;    /* 0 -> 1e9 */
  double length_scale;/* non-ref mode: FIM length unit; 0 -> mean edge */
  double fp64_tau;    /* precision form: FP64 redo of cancelled tet solves (0 = off) */
} lso_params;

typedef struct lso_stats {
  int steps_run;
  int status;
  long long fim_iters;
  long long patch_visits;
  long long check_visits;
  long long nb_vertex_updates;   /* sum over steps of #{v : DT(v) <= w} */
  long long nb_patch_vertices;   /* sum over steps of sum_{p in NB} nv_p */
  long long nb_patches;          /* sum over steps of |NB| */
  double seconds;
} lso_stats;

typedef struct lso_layout lso_layout;

/* Layout arrays retrievable with lso_layout_copy (reference formats). */
enum {
  LSO_L_ELE_PERMUTE = 0,      /* int[full]   original element of each copy */
  LSO_L_ELE_OFFSETS = 1,      /* int[nparts+1] */
  LSO_L_VERT_PERMUTE = 2,     /* int[nv]     new -> old vertex id */
  LSO_L_VERT_OFFSETS = 3,     /* int[nparts+1] */
  LSO_L_ELE_AFTER_PERMUTE = 4,/* int[(d+1)*full] SoA k*full+c, new ids */
  LSO_L_MEM_LOCATIONS = 5,    /* int[(d+1)*full] */
  LSO_L_MEM_LOCATION_OFFSETS = 6, /* int[nv+1] */
  LSO_L_BLOCK_XADJ = 7,       /* int[nparts+1] */
  LSO_L_BLOCK_ADJNCY = 8,     /* int[nadj] */
  LSO_L_LOCAL_COORDS = 9,     /* float[6*full] (3D) / float[3*full] (2D) */
  LSO_L_VERT_IPERMUTE = 10    /* int[nv]     old -> new vertex id */
};

/* info[0..7] = nparts, full, lep, lvp, lim, nadj, nv, ne */
int lso_layout_build(int dim, int nv, const float* xyz, int ne,
                     const int* elems, const int* npart, int nparts,
                     lso_layout** out);
void lso_layout_info(const lso_layout* lo, long long* info);
int lso_layout_copy(const lso_layout* lo, int which, void* dst);
void lso_layout_free(lso_layout* lo);

/* Full solve: nsteps time steps from phi0 (original vertex order).
 * hist: (nsteps+1)*nv floats, snapshot 0 = phi0 (may be NULL).
 * nb_sets: nsteps*nparts bytes, 1 if the patch is in the step's narrowband
 * (may be NULL).  iters: nsteps ints, FIM outer iterations per step (may be
 * NULL).  vel: ne*3 floats per original element (may be NULL = zero). */
int lso_solve(const lso_layout* lo, const lso_params* prm, const float* phi0,
              const float* vel, int nsteps, float* hist,
              unsigned char* nb_sets, int* iters, lso_stats* st);

/* Update pass only (advection / curvature) over the given narrowband patch
 * list, on phi in original order; result in phi_out (original order). */
int lso_update_only(const lso_layout* lo, const lso_params* prm,
                    const float* phi, const float* vel, const int* nb_list,
                    int nnb, float* phi_out);

/* Local solvers, exposed for pinning against the reference. */
/* FP32 solve that falls back to the FP64 solve when a discriminant
 * q^2 - 4pr cancels: |q^2 - 4pr| <= tau * (q^2 + |4pr|).  *flagged set to 1
 * when the fallback ran. */
float lso_tet_solve_f32_flagged(float TA, float TB, float TC, float ACAC, float ACBC,
                                float ACCD, float BCBC, float BCCD, float CDCD,
                                double eps_h, float largenum, float tau, int* flagged);
float lso_tet_solve_f32(float TA, float TB, float TC, float ACAC, float ACBC,
                        float ACCD, float BCBC, float BCCD, float CDCD,
                        double eps_h, float largenum);
double lso_tet_solve_f64(double TA, double TB, double TC, double ACAC,
                         double ACBC, double ACCD, double BCBC, double BCCD,
                         double CDCD, double eps_h, double largenum);
double lso_tri_solve_f64(double TA, double TB, double LenAB, double LenBC,
                         double LenAC, double largenum);
float lso_tri_solve_f32(float TA, float TB, float LenAB, float LenBC,
                        float LenAC, float largenum);

/* Synthetic inputs used by the tests when checking the oracle alone. */
int lso_version(void);

#ifdef __cplusplus
}
#endif
#endif
