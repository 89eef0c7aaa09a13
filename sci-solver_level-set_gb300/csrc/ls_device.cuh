// ls_device.cuh -- device-side local eikonal solvers and shared types.
//
// The tet and triangle local solvers evaluate the same closed-form updates
// as GPUTUM Level-Set's localSolverTet1Levelset
// (src/core3d/include/redistance_kernels3d.h:124-285) and localSolverTri
// (src/core2d/include/redistance_kernels.h:287-334): three face (edge-pair)
// quadratics plus the interior quadratic for a tet, the two-root law-of-
// cosines update for a triangle, each candidate accepted only when its
// barycentric coordinates lie in [0,1].  tet_solve keeps the formulas term
// for term, so that the bit-exact build reproduces the reference's FP32
// arithmetic (the reference's `/ (2.0 * p)` divisions, evaluated there in
// double and rounded to float, give the same correctly rounded float
// quotient as an IEEE float division).  The fast build's tet sweeps use
// tet_solve_wave instead: the same candidates and validity rules, with the
// stationary points found without the reference's cancelling discriminants,
// so that FP32 stays at the reference's FP64 result.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace lsgb {

// Device view of the patch layout.
struct DevMesh {
  int dim, nv, nparts;
  long long full;
  const int* vert_off;       // nparts+1
  const int* ele_off;        // nparts+1
  const int* ghost_off;      // nparts+1
  const int* ghost_ids;      // ghosts (new vertex ids)
  const ushort4* conn;       // full: slab-local vertex indices
  const float* lc;           // SoA [6|3][full] local coordinates
  const float* sig;          // SoA [3][full] per-copy velocity (2D: projected, 2 rows)
  const int* vslot_off;      // nv+1
  const uint16_t* vslot;     // owned-vertex slots (copy_local*4 + k)
  // per copy: corners beyond the reference's per-vertex slot limit, set only
  // with the reference's semantics on meshes that have such corners (null
  // otherwise): they stay private to their copy in the FIM sweep and are
  // left out of the update's sums (Layout::slot_capped)
  const uint8_t* capped;
  int slot_cap;              // the limit: 32 (tetrahedra) or 16 (triangles)
  const int* padj_off;       // nparts+1
  const int* padj;           // patch adjacency
  const float* xyz;          // SoA [3][nv]
  const int* ipermute;       // old -> new vertex id
  const int* patch_bytes;    // per patch: algorithmic bytes of one FIM visit
  // batches of independent meshes: mesh of each patch and per-mesh
  // parameters {bandwidth in the FIM frame, FIM frame scale, dt, curvature
  // coefficient}; null for a single mesh (StepParams hold them)
  const int* patch_mesh;
  const float4* mesh_par;
  // per copy, precomputed once per mesh for the two-copies-per-thread tet
  // sweep (null otherwise): the 11 metric terms of copy_metric as three
  // float4 (geo_m[3c .. 3c+2], last lane a second copy of CDCD) and the
  // heights of A, B, C, D over their opposite faces (geo_h[c]); a patch's
  // copies are contiguous, so its records are two contiguous slabs, staged
  // by bulk asynchronous copies
  const float4* geo_m;
  const float4* geo_h;
};

// Bandwidth (FIM frame), FIM frame scale, dt and curvature coefficient of
// patch p.
struct PatchPar {
  float bw, scale, dt, cc;
};

// Device step state.
struct DevState {
  float* phi;
  float* phi_out;
  float* DT;
  float* DT_out;
  uint8_t* seed;    // per vertex: 1 = seed point of this step
  uint8_t* sign;    // per vertex: 1 = phi >= 0 before redistance
  int* blabel;      // per patch: 0 far, 1 active (host FIM labels of the reference)
  int* bcon;        // per patch: 1 = converged
  float* bmin;      // per patch: min DT after the visit
  int* list0;       // active list, even iterations
  int* list1;       // active list, odd iterations
  int* newlist;     // neighbour candidates of this iteration
  int* nblist;      // narrowband patches
  int* counts;      // [0] list0, [1] list1, [2] newlist, [3] nblist, [4] fim iters (step)
  unsigned long long* stats;  // [0] visits [1] checks [2] nb verts [3] nb patch verts [4] nb patches [5] fim iters [6] flagged copies solved [7] FIM slab bytes [8] visits run by checks
  int* ctl;         // step control: [0] FIM loop bodies run this step, [1] iteration cap hit,
                    // [2] previous narrowband valid (seed search restricted to it), [3] a wait of a
                    // FIM kernel timed out and the launch was abandoned (1: grid barrier of the
                    // persistent kernel, 2: geometry slab copy); cleared at every step start
  int* sched;       // dynamic patch assignment of the sweep kernels: [0] next list entry of a
                    // sweep, [1] of a check; zero between launches (the launch's last draw
                    // resets it)
  unsigned* gbar;   // persistent FIM kernel (kGridBarrierWords, zeroed per launch): [0] grid-barrier
                    // arrivals since the launch started, [2 + smid] CTAs on SM smid
};
constexpr int kGridBarrierWords = 2 + 1024;

// Learned warm start / training-pair collection buffers (null when off).
struct DevLearn {
  int* vlist;     // warm-set vertices (owned vertices of the previous narrowband patches)
  int* cnt;       // [0] warm-set size, [1] unsupported vertices reset, [2] vertices moved beyond
                  // the tolerance, [3] patches re-activated by the support check
  float* pred;    // network output per warm-set vertex (signed distance / h)
  float* warm;    // per vertex: warm-start value in the FIM frame
  float* target;  // collection: signed distance / h after the redistance, per warm-set vertex
  const float* vinv_h;  // batches: per vertex, 1 / its mesh's FIM length unit (null for one mesh)
};

struct StepParams {
  float largenum;
  float bandwidth;   // in the FIM frame (divided by scale)
  float scale;       // FIM frame length unit (1 with the reference's semantics)
  float tau;         // precision form: discriminant cancellation threshold
  int xdiv;          // interior division in double (bit-exact build, reference semantics)
  int ctas;          // FIM CTAs per SM for patches of up to 384 copies (2, 3, 4; 5: two copies per thread)
  float tol;       // convergence threshold on oldT - newT
  float eps_h;     // denominator offset of the interior tet update
  double eps_h64;
  float dt;
  float curv_coeff;
  int niter;       // sweeps per visit
  int ref_compat;
  int update_kind; // 0 advect, 1 curvature
  int lvp, lgp, lep;
  int max_fim_iters;  // persistent FIM kernel: iteration cap of one step
  int spin_limit;     // polls of one grid-barrier wait of the persistent FIM kernel before it gives up;
                      // < 0: every wait of the FIM kernels (grid barrier, geometry slab copy) gives up
                      // at its first check (the setting that tests the timeout paths)
};

__device__ __forceinline__ PatchPar patch_par(const DevMesh& m, const StepParams& sp, int p) {
  if (m.patch_mesh) {
    const float4 q = __ldg(&m.mesh_par[__ldg(&m.patch_mesh[p])]);
    return PatchPar{q.x, q.y, q.z, q.w};
  }
  return PatchPar{sp.bandwidth, sp.scale, sp.dt, sp.curv_coeff};
}


enum { LS_FAR = 0, LS_ACTIVE = 1 };

// Mark on an active-list entry: the patch was already visited by the
// neighbour check that activated it (k_fim_pair); the sweep skips it and the
// schedule masks the mark off.
constexpr int kPrevisited = 1 << 30;

template <typename R>
__device__ __forceinline__ R rmin(R a, R b) { return fmin(a, b); }
template <typename R>
__device__ __forceinline__ R rmax(R a, R b) { return fmax(a, b); }
template <>
__device__ __forceinline__ float rmin<float>(float a, float b) { return fminf(a, b); }

// Unit-speed tet update of vertex D from face ABC given the metric terms of
// the edge vectors AC, BC, CD (R = float or double).  Every expression keeps
// the reference's operand order and association, so that a build without
// FMA contraction reproduces the reference arithmetic bit for bit.
//
// XDIV: the reference evaluates the interior barycentric coordinate
// `(s * l1 + t) / (h + SMALLNUM)` with a double SMALLNUM, i.e. in double;
// XDIV = true reproduces that (used only by the bit-exact build with the
// reference's semantics), XDIV = false divides in R.
//
// `tau` > 0 turns on the conditioning check of the precision form: `ill` is
// set when a discriminant q^2 - 4pr cancels, |q^2 - 4pr| <= tau (q^2 + |4pr|),
// i.e. when FP32 has lost about log2(1/tau) bits of it.
// Roots of p x^2 + q x + r given sq = sqrt(q^2 - 4pr).  The reference's
// form (-q +- sq) / 2p, or, for the precision form, the cancellation-free
// pair s / p, r / s with s = -(q + sign(q) sq) / 2 (the same two roots; also
// right when p = 0).
template <typename R, bool STABLE>
__device__ __forceinline__ void roots(R p, R q, R r, R sq, R& ra, R& rb) {
  if (STABLE) {
    const R sh = -(q + (q >= R(0) ? sq : -sq)) * R(0.5);
    ra = sh / p;
    rb = r / sh;
  } else {
    ra = (-q + sq) / (R(2) * p);
    rb = (-q - sq) / (R(2) * p);
  }
}

template <typename R, bool XDIV, bool CHK = true, bool LB = false>
__device__ __forceinline__ R tet_solve(R TA, R TB, R TC, R ACAC, R ACBC, R ACCD, R BCBC, R BCCD,
                                       R CDCD, R eps_h, double eps_h64, R LN, R tau, bool& ill,
                                       R cutoff = R(0)) {
  if (TA >= LN && TB >= LN && TC >= LN) return LN;
  // precision form (CHK): a quadratic is flagged only when all its arrival
  // times are below LARGENUM -- with one at LARGENUM its candidates lie at or
  // above the edge candidates computed separately (equal values, e.g. two
  // LARGENUMs, make the discriminant vanish identically)
  if (CHK || LB) {
    // precision form: a solve whose candidates cannot fall below `cutoff`
    // (the target's current value) is skipped -- every candidate is at
    // least min(TA, TB, TC) plus D's height over the plane ABC (Gram
    // determinants of AC, BC, CD; taken x 0.999)
    const R det2 = ACAC * BCBC - ACBC * ACBC;
    const R det3 = ACAC * (BCBC * CDCD - BCCD * BCCD) - ACBC * (ACBC * CDCD - BCCD * ACCD) +
                   ACCD * (ACBC * BCCD - BCBC * ACCD);
    const R lb = rmin(rmin(TA, TB), TC) + R(0.999) * sqrt(fmax(det3 / det2, R(0)));
    if (lb >= cutoff) return LN;
  }
  const R two = R(2), four = R(4), one = R(1), zero = R(0);
  R p, q, r, lambda1, lambda2, lambda3, delta, TE;
  R FaceTAC = LN, FaceTAB = LN, FaceTBC = LN, TD = LN;
  const R TAC = TC - TA, TBC = TC - TB, TAB = TB - TA;

  // face BC (lambda1 = 0)
  p = BCBC * TBC * TBC - BCBC * BCBC;
  q = (BCCD + BCCD) * TBC * TBC - two * BCBC * BCCD;
  r = TBC * TBC * CDCD - BCCD * BCCD;
  delta = q * q - four * p * r;
  if (CHK && rmax(TB, TC) < LN) ill |= (fabs(delta) <= tau * (q * q + fabs(four * p * r)));
  if (delta >= zero) {
    const R sq = sqrt(delta);
    R ra, rb;
    roots<R, CHK>(p, q, r, sq, ra, rb);
    lambda1 = zero;
    lambda2 = ra;
    lambda3 = one - lambda1 - lambda2;
    if (lambda2 >= zero && lambda2 <= one) {
      TE = TB * lambda2 + TC * lambda3;
      FaceTBC = rmin(FaceTBC, TE + sqrt((lambda2 * BCBC + BCCD) * lambda2 + (lambda2 * BCCD + CDCD)));
    }
    lambda2 = rb;
    lambda3 = one - lambda1 - lambda2;
    if (lambda2 >= zero && lambda2 <= one) {
      TE = TB * lambda2 + TC * lambda3;
      FaceTBC = rmin(FaceTBC, TE + sqrt((lambda2 * BCBC + BCCD) * lambda2 + (lambda2 * BCCD + CDCD)));
    }
  }
  FaceTBC = rmin(FaceTBC, rmin(TB + sqrt((BCBC + BCCD) + (BCCD + CDCD)), TC + sqrt(CDCD)));

  // face AB (lambda3 = 0)
  const R gammax = ACAC - ACBC, gammay = ACBC - BCBC, gammaz = ACCD - BCCD;
  p = (TAB * TAB * ACAC - gammax * gammax) + (BCBC * TAB * TAB - gammay * gammay) -
      ((ACBC + ACBC) * TAB * TAB - two * gammax * gammay);
  q = -(BCBC * TAB * TAB - gammay * gammay) * two + ((ACBC + ACBC) * TAB * TAB - two * gammax * gammay) +
      ((ACCD + ACCD) * TAB * TAB - two * gammax * gammaz) - ((BCCD + BCCD) * TAB * TAB - two * gammay * gammaz);
  r = (TAB * TAB * BCBC - gammay * gammay) + ((BCCD + BCCD) * TAB * TAB - two * gammay * gammaz) +
      (TAB * TAB * CDCD - gammaz * gammaz);
  delta = q * q - four * p * r;
  if (CHK && rmax(TA, TB) < LN) ill |= (fabs(delta) <= tau * (q * q + fabs(four * p * r)));
  if (delta >= zero) {
    const R sq = sqrt(delta);
    R ra, rb;
    roots<R, CHK>(p, q, r, sq, ra, rb);
#pragma unroll
    for (int sgn = 0; sgn < 2; ++sgn) {
      lambda1 = sgn ? rb : ra;
      lambda2 = one - lambda1;
      if (lambda1 >= zero && lambda1 <= one) {
        TE = TA * lambda1 + TB * lambda2;
        FaceTAB = rmin(FaceTAB, TE + sqrt((lambda1 * ACAC + lambda2 * ACBC + ACCD) * lambda1 +
                                          (lambda1 * ACBC + lambda2 * BCBC + BCCD) * lambda2 +
                                          (lambda1 * ACCD + lambda2 * BCCD + CDCD)));
      }
    }
  }
  FaceTAB = rmin(FaceTAB, rmin(TB + sqrt((BCBC + BCCD) + (BCCD + CDCD)), TA + sqrt((ACAC + ACCD) + (ACCD + CDCD))));

  // face AC (lambda2 = 0)
  p = ACAC * TAC * TAC - ACAC * ACAC;
  q = (ACCD + ACCD) * TAC * TAC - two * ACAC * ACCD;
  r = TAC * TAC * CDCD - ACCD * ACCD;
  delta = q * q - four * p * r;
  if (CHK && rmax(TA, TC) < LN) ill |= (fabs(delta) <= tau * (q * q + fabs(four * p * r)));
  if (delta >= zero) {
    const R sq = sqrt(delta);
    R ra, rb;
    roots<R, CHK>(p, q, r, sq, ra, rb);
#pragma unroll
    for (int sgn = 0; sgn < 2; ++sgn) {
      lambda1 = sgn ? rb : ra;
      lambda3 = one - lambda1 - zero;
      if (lambda1 >= zero && lambda1 <= one) {
        TE = TA * lambda1 + TC * lambda3;
        FaceTAC = rmin(FaceTAC, TE + sqrt((lambda1 * ACAC + ACCD) * lambda1 + (lambda1 * ACCD + CDCD)));
      }
    }
  }
  FaceTAC = rmin(FaceTAC, rmin(TA + sqrt((ACAC + ACCD) + (ACCD + CDCD)), TC + sqrt(CDCD)));

  // interior of face ABC
  const R s = TAC * ACBC - TBC * ACAC;
  const R t = TAC * BCCD - TBC * ACCD;
  const R h = -(TAC * BCBC - TBC * ACBC);
  p = (TAC * TAC * ACAC - ACAC * ACAC) * h * h + (BCBC * TAC * TAC - ACBC * ACBC) * s * s +
      ((ACBC + ACBC) * TAC * TAC - two * ACAC * ACBC) * s * h;
  q = (BCBC * TAC * TAC - ACBC * ACBC) * two * s * t + ((ACBC + ACBC) * TAC * TAC - two * ACAC * ACBC) * t * h +
      ((ACCD + ACCD) * TAC * TAC - two * ACAC * ACCD) * h * h + ((BCCD + BCCD) * TAC * TAC - two * ACBC * ACCD) * s * h;
  r = (TAC * TAC * BCBC - ACBC * ACBC) * t * t + ((BCCD + BCCD) * TAC * TAC - two * ACBC * ACCD) * t * h +
      (TAC * TAC * CDCD - ACCD * ACCD) * h * h;
  delta = q * q - four * p * r;
  if (CHK && rmax(rmax(TA, TB), TC) < LN) ill |= (fabs(delta) <= tau * (q * q + fabs(four * p * r)));
  if (delta >= zero) {
    const R sq = sqrt(delta);
    R ra, rb;
    roots<R, CHK>(p, q, r, sq, ra, rb);
#pragma unroll
    for (int sgn = 0; sgn < 2; ++sgn) {
      lambda1 = sgn ? rb : ra;
      if (XDIV)
        lambda2 = (R)((double)(s * lambda1 + t) / ((double)h + eps_h64));
      else
        lambda2 = (s * lambda1 + t) / (h + eps_h);
      lambda3 = one - lambda1 - lambda2;
      if (lambda1 >= zero && lambda1 <= one && lambda2 >= zero && lambda2 <= one && lambda3 >= zero &&
          lambda3 <= one) {
        TE = TA * lambda1 + TB * lambda2 + TC * lambda3;
        TD = rmin(TD, TE + sqrt((lambda1 * ACAC + lambda2 * ACBC + ACCD) * lambda1 +
                                (lambda1 * ACBC + lambda2 * BCBC + BCCD) * lambda2 +
                                (lambda1 * ACCD + lambda2 * BCCD + CDCD)));
      }
    }
  }
  TD = rmin(TD, rmin(FaceTBC, rmin(FaceTAB, FaceTAC)));
  return TD;
}

// The same tet update with predicated candidates instead of branches (fast
// build): every quadratic's roots and candidate distances are evaluated and
// the invalid ones masked, so the lanes of a warp stay converged through the
// solve.  A negative discriminant gives NaN roots, which fail every range
// test, and a candidate whose distance is not a number is dropped by fminf,
// so neither needs a guard.  Valid candidates use the same expressions as
// tet_solve; CHK adds
// the precision form's flags and cancellation-free roots (as tet_solve with
// CHK, without its lower-bound skip, which the caller has applied).
template <bool CHK = false>
__device__ __forceinline__ float tet_solve_pred(float TA, float TB, float TC, float ACAC, float ACBC, float ACCD,
                                                float BCBC, float BCCD, float CDCD, float eps_h, float LN,
                                                float tau = 0.f, bool* ill = nullptr) {
  if (TA >= LN && TB >= LN && TC >= LN) return LN;
  float FaceTAC = LN, FaceTAB = LN, FaceTBC = LN, TD = LN;
  const float TAC = TC - TA, TBC = TC - TB, TAB = TB - TA;
  float p, q, r, delta;
  // face BC (lambda1 = 0)
  p = BCBC * TBC * TBC - BCBC * BCBC;
  q = (BCCD + BCCD) * TBC * TBC - 2.f * BCBC * BCCD;
  r = TBC * TBC * CDCD - BCCD * BCCD;
  delta = q * q - 4.f * p * r;
  if (CHK && fmaxf(TB, TC) < LN && fabsf(delta) <= tau * (q * q + fabsf(4.f * p * r))) *ill = true;
  {
    const float sq = sqrtf(delta);  // NaN when delta < 0: every root test fails
    float ra, rb;
    roots<float, CHK>(p, q, r, sq, ra, rb);
#pragma unroll
    for (int sgn = 0; sgn < 2; ++sgn) {
      const float l2 = sgn ? rb : ra;
      const float l3 = 1.f - l2;
      const float c = TB * l2 + TC * l3 + sqrtf((l2 * BCBC + BCCD) * l2 + (l2 * BCCD + CDCD));
      if (l2 >= 0.f && l2 <= 1.f) FaceTBC = fminf(FaceTBC, c);
    }
  }
  FaceTBC = fminf(FaceTBC, fminf(TB + sqrtf((BCBC + BCCD) + (BCCD + CDCD)), TC + sqrtf(CDCD)));
  // face AB (lambda3 = 0)
  const float gammax = ACAC - ACBC, gammay = ACBC - BCBC, gammaz = ACCD - BCCD;
  p = (TAB * TAB * ACAC - gammax * gammax) + (BCBC * TAB * TAB - gammay * gammay) -
      ((ACBC + ACBC) * TAB * TAB - 2.f * gammax * gammay);
  q = -(BCBC * TAB * TAB - gammay * gammay) * 2.f + ((ACBC + ACBC) * TAB * TAB - 2.f * gammax * gammay) +
      ((ACCD + ACCD) * TAB * TAB - 2.f * gammax * gammaz) - ((BCCD + BCCD) * TAB * TAB - 2.f * gammay * gammaz);
  r = (TAB * TAB * BCBC - gammay * gammay) + ((BCCD + BCCD) * TAB * TAB - 2.f * gammay * gammaz) +
      (TAB * TAB * CDCD - gammaz * gammaz);
  delta = q * q - 4.f * p * r;
  if (CHK && fmaxf(TA, TB) < LN && fabsf(delta) <= tau * (q * q + fabsf(4.f * p * r))) *ill = true;
  {
    const float sq = sqrtf(delta);  // NaN when delta < 0: every root test fails
    float ra, rb;
    roots<float, CHK>(p, q, r, sq, ra, rb);
#pragma unroll
    for (int sgn = 0; sgn < 2; ++sgn) {
      const float l1 = sgn ? rb : ra;
      const float l2 = 1.f - l1;
      const float c = TA * l1 + TB * l2 +
                      sqrtf((l1 * ACAC + l2 * ACBC + ACCD) * l1 + (l1 * ACBC + l2 * BCBC + BCCD) * l2 +
                            (l1 * ACCD + l2 * BCCD + CDCD));
      if (l1 >= 0.f && l1 <= 1.f) FaceTAB = fminf(FaceTAB, c);
    }
  }
  FaceTAB = fminf(FaceTAB, fminf(TB + sqrtf((BCBC + BCCD) + (BCCD + CDCD)), TA + sqrtf((ACAC + ACCD) + (ACCD + CDCD))));
  // face AC (lambda2 = 0)
  p = ACAC * TAC * TAC - ACAC * ACAC;
  q = (ACCD + ACCD) * TAC * TAC - 2.f * ACAC * ACCD;
  r = TAC * TAC * CDCD - ACCD * ACCD;
  delta = q * q - 4.f * p * r;
  if (CHK && fmaxf(TA, TC) < LN && fabsf(delta) <= tau * (q * q + fabsf(4.f * p * r))) *ill = true;
  {
    const float sq = sqrtf(delta);  // NaN when delta < 0: every root test fails
    float ra, rb;
    roots<float, CHK>(p, q, r, sq, ra, rb);
#pragma unroll
    for (int sgn = 0; sgn < 2; ++sgn) {
      const float l1 = sgn ? rb : ra;
      const float l3 = 1.f - l1;
      const float c = TA * l1 + TC * l3 + sqrtf((l1 * ACAC + ACCD) * l1 + (l1 * ACCD + CDCD));
      if (l1 >= 0.f && l1 <= 1.f) FaceTAC = fminf(FaceTAC, c);
    }
  }
  FaceTAC = fminf(FaceTAC, fminf(TA + sqrtf((ACAC + ACCD) + (ACCD + CDCD)), TC + sqrtf(CDCD)));
  // interior of face ABC
  const float s = TAC * ACBC - TBC * ACAC;
  const float t = TAC * BCCD - TBC * ACCD;
  const float h = -(TAC * BCBC - TBC * ACBC);
  p = (TAC * TAC * ACAC - ACAC * ACAC) * h * h + (BCBC * TAC * TAC - ACBC * ACBC) * s * s +
      ((ACBC + ACBC) * TAC * TAC - 2.f * ACAC * ACBC) * s * h;
  q = (BCBC * TAC * TAC - ACBC * ACBC) * 2.f * s * t + ((ACBC + ACBC) * TAC * TAC - 2.f * ACAC * ACBC) * t * h +
      ((ACCD + ACCD) * TAC * TAC - 2.f * ACAC * ACCD) * h * h + ((BCCD + BCCD) * TAC * TAC - 2.f * ACBC * ACCD) * s * h;
  r = (TAC * TAC * BCBC - ACBC * ACBC) * t * t + ((BCCD + BCCD) * TAC * TAC - 2.f * ACBC * ACCD) * t * h +
      (TAC * TAC * CDCD - ACCD * ACCD) * h * h;
  delta = q * q - 4.f * p * r;
  if (CHK && fmaxf(fmaxf(TA, TB), TC) < LN && fabsf(delta) <= tau * (q * q + fabsf(4.f * p * r))) *ill = true;
  {
    const float sq = sqrtf(delta);  // NaN when delta < 0: every root test fails
    float ra, rb;
    roots<float, CHK>(p, q, r, sq, ra, rb);
#pragma unroll
    for (int sgn = 0; sgn < 2; ++sgn) {
      const float l1 = sgn ? rb : ra;
      const float l2 = (s * l1 + t) / (h + eps_h);
      const float l3 = 1.f - l1 - l2;
      const float c = TA * l1 + TB * l2 + TC * l3 +
                      sqrtf((l1 * ACAC + l2 * ACBC + ACCD) * l1 + (l1 * ACBC + l2 * BCBC + BCCD) * l2 +
                            (l1 * ACCD + l2 * BCCD + CDCD));
      if (l1 >= 0.f && l1 <= 1.f && l2 >= 0.f && l2 <= 1.f && l3 >= 0.f && l3 <= 1.f) TD = fminf(TD, c);
    }
  }
  return fminf(TD, fminf(FaceTBC, fminf(FaceTAB, FaceTAC)));
}

// l in [+0, 1] as one unsigned compare of the bits (negative values, -0.0
// and NaN fail).  A candidate rejected for l = -0.0 sits at the side's end
// point, where the edge candidate gives the same value.
__device__ __forceinline__ bool in_unit(float l) { return __float_as_uint(l) <= 0x3f800000u; }

// Tet update of D from the face ABC in FP32 without the quadratics (fast
// build).  It returns the same quantity as tet_solve -- the least T_lin(x) +
// |x - D| over the face, T_lin interpolating TA, TB, TC, with the reference's
// candidates (three edges, three sides, the face interior) and its validity
// rules -- but finds each stationary point from the planar wave that passes
// through the known values instead of from a squared equation.  For a side
// PQ with f = Q - P, w = D - P and u = TQ - TP, the point P + l f with
//   l = (f.w - |f x w| u / sqrt(|f|^2 - u^2)) / |f|^2
// is where the characteristic through D meets the side (none when |u| >=
// |f|), and its distance to D is |f x w| / sqrt(|f|^2 - u^2) (the same
// quantity the reference evaluates at that point, without a square root of
// its own).  For the interior, the in-plane gradient g solves the 2x2 Gram
// system of AC, BC; the characteristic leaves the plane at sqrt(1 - |g|^2),
// so the weight of A is the foot point's first barycentric minus (hD /
// sqrt(1 - |g|^2)) times g's first coefficient (hD: D's height over ABC),
// and the weight of B comes from the reference's own relation l2 = (s l1 +
// t) / (h + eps_h), so that its SMALLNUM offset acts as in the reference; the
// candidate is evaluated at that point as the reference does.  The
// reference's quadratic also has the mirror root (the foot point plus the
// same offset), taken too: where h is small the offset moves the first
// root's point by far more than rounding, and the mirror's point can then be
// the better one.  The reference's discriminants q^2 -
// 4pr vanish analytically whenever two arrival times along a side are equal,
// so in FP32 they come out as rounding noise of either sign (a negative one
// drops the candidate: errors up to ~0.3 h); none of the quantities here
// cancel, and the result stays within ~5e-5 h of the reference's solver run
// in FP64.  Invalid points come out as NaN or out of range and fail the
// range tests.
// Evaluation: sm_100 issues one FP32x2 instruction (add, multiply, fused
// multiply-add, each lane rounded as the scalar operation) for two lanes, so
// the independent halves run as pairs -- edges AD and BD, sides BC and AC
// (both from C), the two interior roots -- with the square roots, side AB
// and the interior's set-up per lane.
// Arguments as tet_solve, plus hD.
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

__device__ __forceinline__ float tet_solve_wave(float TA, float TB, float TC, float ACAC, float ACBC, float ACCD,
                                                float BCBC, float BCCD, float CDCD, float hD, float eps_h, float LN) {
  if (TA >= LN && TB >= LN && TC >= LN) return LN;
  // edges AD, BD (lanes x, y) and CD
  const float2 d2 = __fadd2_rn(__fadd2_rn(f2(ACAC, BCBC), f2(ACCD, BCCD)), __fadd2_rn(f2(ACCD, BCCD), f2(CDCD, CDCD)));
  const float2 ed = __fadd2_rn(f2(TA, TB), f2(sqrtf(d2.x), sqrtf(d2.y)));
  float best = fminf(fminf(ed.x, ed.y), TC + sqrtf(CDCD));
  // sides: x = lam Q + (1 - lam) P with |Q - P|^2 = ff, (Q - P).(D - P) = fw,
  // |D - P|^2 = ww and u = T_Q - T_P.  At the stationary point of
  // T_P + lam u + |x - D| the distance is r = sqrt(ff ww - fw^2) /
  // sqrt(ff - u^2) (no root when ff <= u^2: the rsqrt is then NaN or inf and
  // the candidate is rejected) and lam = (fw - u r) / ff.
  {  // sides BC (lane x: P = C, Q = B) and AC (lane y: P = C, Q = A)
    const float2 fw = f2(-BCCD, -ACCD), ff = f2(BCBC, ACAC);
    const float2 u = __fadd2_rn(f2(TB, TA), f2(-TC, -TC));
    const float2 G = __ffma2_rn(ff, f2(CDCD, CDCD), __fmul2_rn(fw, f2(BCCD, ACCD)));  // ff ww - fw^2
    const float2 q = __ffma2_rn(u, f2(-u.x, -u.y), ff);                              // ff - u^2
    const float2 r = __fmul2_rn(f2(sqrtf(G.x), sqrtf(G.y)), f2(rsqrtf(q.x), rsqrtf(q.y)));
    const float2 lam = __fmul2_rn(__ffma2_rn(f2(-u.x, -u.y), r, fw), f2(1.f / ff.x, 1.f / ff.y));
    const float2 c = __fadd2_rn(__ffma2_rn(lam, u, f2(TC, TC)), r);
    if (in_unit(lam.x)) best = fminf(best, c.x);
    if (in_unit(lam.y)) best = fminf(best, c.y);
  }
  {  // side AB (P = B, Q = A)
    const float u = TA - TB;
    const float ff = (BCBC - ACBC) + (ACAC - ACBC), fw = (BCBC + BCCD) - (ACBC + ACCD);
    const float ww = (BCBC + BCCD) + (BCCD + CDCD);
    const float r = sqrtf(ff * ww - fw * fw) * rsqrtf(ff - u * u);
    const float lam = (fw - u * r) / ff;
    if (in_unit(lam)) best = fminf(best, TB + lam * u + r);
  }
  {  // interior of ABC: x = l1 A + l2 B + l3 C
    const float u1 = TA - TC, u2 = TB - TC;
    const float idet = 1.f / (ACAC * BCBC - ACBC * ACBC);
    const float g1 = (BCBC * u1 - ACBC * u2) * idet;  // in-plane gradient, coefficient of -AC
    const float g2 = (ACAC * u2 - ACBC * u1) * idet;  // and of -BC
    const float foot1 = (ACBC * BCCD - BCBC * ACCD) * idet;  // D's foot point, weight of A
    // the point downhill of the foot point (lane x) and its mirror uphill
    // (lane y): the reference's SMALLNUM offset in l2 = (s l1 + t) / (h +
    // eps_h) can move the first point out of the face where h is small, and
    // the mirror's point is then the better one, as in the reference
    const float dl = hD * rsqrtf(1.f - (g1 * u1 + g2 * u2)) * g1;
    const float TAC = TC - TA, TBC = TC - TB;
    const float s = TAC * ACBC - TBC * ACAC, t = TAC * BCCD - TBC * ACCD, h = -(TAC * BCBC - TBC * ACBC);
    const float ih = 1.f / (h + eps_h);
    const float2 l1 = __fadd2_rn(f2(foot1, foot1), f2(-dl, dl));
    const float2 l2 = __fmul2_rn(__ffma2_rn(f2(s, s), l1, f2(t, t)), f2(ih, ih));
    const float2 l3 = __fadd2_rn(__fadd2_rn(f2(1.f, 1.f), f2(-l1.x, -l1.y)), f2(-l2.x, -l2.y));
    // |x - D|^2 as the quadratic form of (l1, l2), and T_lin(x)
    const float2 a1 = __ffma2_rn(l1, f2(ACAC, ACAC), __ffma2_rn(l2, f2(ACBC, ACBC), f2(ACCD, ACCD)));
    const float2 a2 = __ffma2_rn(l1, f2(ACBC, ACBC), __ffma2_rn(l2, f2(BCBC, BCBC), f2(BCCD, BCCD)));
    const float2 a3 = __ffma2_rn(l1, f2(ACCD, ACCD), __ffma2_rn(l2, f2(BCCD, BCCD), f2(CDCD, CDCD)));
    const float2 Q = __ffma2_rn(a1, l1, __ffma2_rn(a2, l2, a3));
    const float2 lin = __ffma2_rn(f2(TA, TA), l1, __ffma2_rn(f2(TB, TB), l2, __fmul2_rn(f2(TC, TC), l3)));
    const float2 c = __fadd2_rn(lin, f2(sqrtf(Q.x), sqrtf(Q.y)));
    if (in_unit(l1.x) && in_unit(l2.x) && in_unit(l3.x)) best = fminf(best, c.x);
    if (in_unit(l1.y) && in_unit(l2.y) && in_unit(l3.y)) best = fminf(best, c.y);
  }
  return best;
}

// Triangle update of C from edge AB (speed 1); the square roots are taken in
// single precision as in the reference, which passes doubles to sqrtf.
template <typename R>
__device__ __forceinline__ R tri_solve(R TA, R TB, R LenAB, R LenBC, R LenAC, R LN) {
  if (TA >= LN && TB >= LN) return LN;
  const R speedI = R(1);
  const R TAB = TB - TA;
  const R a = (speedI * speedI * LenAB * LenAB - TAB * TAB) * LenAB * LenAB;
  const R EdgeTA = TA + LenAC * speedI, EdgeTB = TB + LenBC * speedI;
  R TC1 = LN, TC2 = LN;
  if (a > R(0)) {
    const R cosA = (LenAC * LenAC + LenAB * LenAB - LenBC * LenBC) / (R(2) * LenAC * LenAB);
    const R b = R(2) * LenAB * LenAC * cosA * (TAB * TAB - speedI * speedI * LenAB * LenAB);
    const R delta = R(4) * LenAC * LenAC * a * TAB * TAB * (R(1) - cosA * cosA);
    const R sq = (R)sqrtf((float)delta);
    const R l1 = (-b + sq) / (R(2) * a);
    const R l2 = (-b - sq) / (R(2) * a);
    if (l1 >= R(0) && l1 <= R(1)) {
      const R LenAD = l1 * LenAB;
      const R LenCD = (R)sqrtf((float)(LenAC * LenAC + LenAD * LenAD - R(2) * LenAC * LenAD * cosA));
      TC1 = l1 * TAB + TA + LenCD * speedI;
    }
    if (l2 >= R(0) && l2 <= R(1)) {
      const R LenAD = l2 * LenAB;
      const R LenCD = (R)sqrtf((float)(LenAC * LenAC + LenAD * LenAD - R(2) * LenAC * LenAD * cosA));
      TC2 = l2 * TAB + TA + LenCD * speedI;
    }
    return rmin(TC2, rmin(TC1, rmin(EdgeTA, EdgeTB)));
  }
  return rmin(EdgeTA, EdgeTB);
}

}  // namespace lsgb
