// ls_device.cuh -- device-side local eikonal solvers and shared types.
//
// The tet and triangle local solvers evaluate the same closed-form updates
// as GPUTUM Level-Set's localSolverTet1Levelset
// (src/core3d/include/redistance_kernels3d.h:124-285) and localSolverTri
// (src/core2d/include/redistance_kernels.h:287-334): three face (edge-pair)
// quadratics plus the interior quadratic for a tet, the two-root law-of-
// cosines update for a triangle, each candidate accepted only when its
// barycentric coordinates lie in [0,1].  The formulas are kept term for term
// because the results must agree with the reference within 1e-4 h; the
// arithmetic is FP32 throughout (the reference's `/ (2.0 * p)` divisions,
// evaluated there in double and rounded to float, give the same correctly
// rounded float quotient as an IEEE float division).
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
  const int* padj_off;       // nparts+1
  const int* padj;           // patch adjacency
  const float* xyz;          // SoA [3][nv]
  const int* ipermute;       // old -> new vertex id
  const int* patch_bytes;    // per patch: algorithmic bytes of one FIM visit
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
  unsigned long long* stats;  // [0] visits [1] checks [2] nb verts [3] nb patch verts [4] nb patches [5] fim iters [6] flagged copies solved [7] sweep slab bytes
};

struct StepParams {
  float largenum;
  float bandwidth;   // in the FIM frame (divided by scale)
  float scale;       // FIM frame length unit (1 with the reference's semantics)
  float tau;         // precision form: discriminant cancellation threshold
  float tol;       // convergence threshold on oldT - newT
  float eps_h;     // denominator offset of the interior tet update
  double eps_h64;
  float dt;
  float curv_coeff;
  int niter;       // sweeps per visit
  int ref_compat;
  int update_kind; // 0 advect, 1 curvature
  int lvp, lgp, lep;
};

enum { LS_FAR = 0, LS_ACTIVE = 1 };

template <typename R>
__device__ __forceinline__ R rmin(R a, R b) { return fmin(a, b); }
template <>
__device__ __forceinline__ float rmin<float>(float a, float b) { return fminf(a, b); }

// Unit-speed tet update of vertex D from face ABC given the metric terms of
// the edge vectors AC, BC, CD (R = float or double).
//
// `tau` > 0 turns on the conditioning check of the precision form: `ill` is
// set when a discriminant q^2 - 4pr cancels, |q^2 - 4pr| <= tau (q^2 + |4pr|),
// i.e. when FP32 has lost about log2(1/tau) bits of it.
template <typename R>
__device__ __forceinline__ R tet_solve(R TA, R TB, R TC, R ACAC, R ACBC, R ACCD, R BCBC, R BCCD,
                                       R CDCD, R eps_h, R LN, R tau, bool& ill) {
  if (TA >= LN && TB >= LN && TC >= LN) return LN;
  R p, q, r, l1, l2, l3, delta, TE;
  R FaceTAC = LN, FaceTAB = LN, FaceTBC = LN, TD = LN;
  const R TAC = TC - TA, TBC = TC - TB, TAB = TB - TA;
  const R two = R(2), four = R(4), one = R(1), zero = R(0);

  // face BC (lambda1 = 0)
  p = BCBC * TBC * TBC - BCBC * BCBC;
  q = (BCCD + BCCD) * TBC * TBC - two * BCBC * BCCD;
  r = TBC * TBC * CDCD - BCCD * BCCD;
  delta = q * q - four * p * r;
  ill |= (fabs(delta) <= tau * (q * q + fabs(four * p * r)));
  if (delta >= zero) {
    const R sq = sqrt(delta);
    l2 = (-q + sq) / (two * p);
    l3 = one - zero - l2;
    if (l2 >= zero && l2 <= one) {
      TE = TB * l2 + TC * l3;
      FaceTBC = rmin(FaceTBC, TE + sqrt((l2 * BCBC + BCCD) * l2 + (l2 * BCCD + CDCD)));
    }
    l2 = (-q - sq) / (two * p);
    l3 = one - zero - l2;
    if (l2 >= zero && l2 <= one) {
      TE = TB * l2 + TC * l3;
      FaceTBC = rmin(FaceTBC, TE + sqrt((l2 * BCBC + BCCD) * l2 + (l2 * BCCD + CDCD)));
    }
  }
  FaceTBC = rmin(FaceTBC, rmin(TB + sqrt((BCBC + BCCD) + (BCCD + CDCD)), TC + sqrt(CDCD)));

  // face AB (lambda3 = 0)
  const R gx = ACAC - ACBC, gy = ACBC - BCBC, gz = ACCD - BCCD;
  const R TAB2 = TAB * TAB;
  p = (TAB2 * ACAC - gx * gx) + (BCBC * TAB2 - gy * gy) - ((ACBC + ACBC) * TAB2 - two * gx * gy);
  q = -(BCBC * TAB2 - gy * gy) * two + ((ACBC + ACBC) * TAB2 - two * gx * gy) +
      ((ACCD + ACCD) * TAB2 - two * gx * gz) - ((BCCD + BCCD) * TAB2 - two * gy * gz);
  r = (TAB2 * BCBC - gy * gy) + ((BCCD + BCCD) * TAB2 - two * gy * gz) + (TAB2 * CDCD - gz * gz);
  delta = q * q - four * p * r;
  ill |= (fabs(delta) <= tau * (q * q + fabs(four * p * r)));
  if (delta >= zero) {
    const R sq = sqrt(delta);
#pragma unroll
    for (int sgn = 0; sgn < 2; ++sgn) {
      l1 = (-q + (sgn ? -sq : sq)) / (two * p);
      l2 = one - l1;
      if (l1 >= zero && l1 <= one) {
        TE = TA * l1 + TB * l2;
        FaceTAB = rmin(FaceTAB, TE + sqrt((l1 * ACAC + l2 * ACBC + ACCD) * l1 +
                                          (l1 * ACBC + l2 * BCBC + BCCD) * l2 +
                                          (l1 * ACCD + l2 * BCCD + CDCD)));
      }
    }
  }
  FaceTAB = rmin(FaceTAB, rmin(TB + sqrt((BCBC + BCCD) + (BCCD + CDCD)), TA + sqrt((ACAC + ACCD) + (ACCD + CDCD))));

  // face AC (lambda2 = 0)
  const R TAC2 = TAC * TAC;
  p = ACAC * TAC2 - ACAC * ACAC;
  q = (ACCD + ACCD) * TAC2 - two * ACAC * ACCD;
  r = TAC2 * CDCD - ACCD * ACCD;
  delta = q * q - four * p * r;
  ill |= (fabs(delta) <= tau * (q * q + fabs(four * p * r)));
  if (delta >= zero) {
    const R sq = sqrt(delta);
#pragma unroll
    for (int sgn = 0; sgn < 2; ++sgn) {
      l1 = (-q + (sgn ? -sq : sq)) / (two * p);
      l3 = one - l1 - zero;
      if (l1 >= zero && l1 <= one) {
        TE = TA * l1 + TC * l3;
        FaceTAC = rmin(FaceTAC, TE + sqrt((l1 * ACAC + ACCD) * l1 + (l1 * ACCD + CDCD)));
      }
    }
  }
  FaceTAC = rmin(FaceTAC, rmin(TA + sqrt((ACAC + ACCD) + (ACCD + CDCD)), TC + sqrt(CDCD)));

  // interior of face ABC
  const R s = TAC * ACBC - TBC * ACAC;
  const R t = TAC * BCCD - TBC * ACCD;
  const R h = -(TAC * BCBC - TBC * ACBC);
  const R cA = TAC2 * ACAC - ACAC * ACAC;
  const R cB = BCBC * TAC2 - ACBC * ACBC;
  const R cC = (ACBC + ACBC) * TAC2 - two * ACAC * ACBC;
  const R cD = (ACCD + ACCD) * TAC2 - two * ACAC * ACCD;
  const R cE = (BCCD + BCCD) * TAC2 - two * ACBC * ACCD;
  const R cF = TAC2 * CDCD - ACCD * ACCD;
  p = cA * h * h + cB * s * s + cC * s * h;
  q = cB * two * s * t + cC * t * h + cD * h * h + cE * s * h;
  r = cB * t * t + cE * t * h + cF * h * h;
  delta = q * q - four * p * r;
  ill |= (fabs(delta) <= tau * (q * q + fabs(four * p * r)));
  if (delta >= zero) {
    const R sq = sqrt(delta);
    const R hd = h + eps_h;
#pragma unroll
    for (int sgn = 0; sgn < 2; ++sgn) {
      l1 = (-q + (sgn ? -sq : sq)) / (two * p);
      l2 = (s * l1 + t) / hd;
      l3 = one - l1 - l2;
      if (l1 >= zero && l1 <= one && l2 >= zero && l2 <= one && l3 >= zero && l3 <= one) {
        TE = TA * l1 + TB * l2 + TC * l3;
        TD = rmin(TD, TE + sqrt((l1 * ACAC + l2 * ACBC + ACCD) * l1 + (l1 * ACBC + l2 * BCBC + BCCD) * l2 +
                                (l1 * ACCD + l2 * BCCD + CDCD)));
      }
    }
  }
  TD = rmin(TD, rmin(FaceTBC, rmin(FaceTAB, FaceTAC)));
  return TD;
}

// Triangle update of C from edge AB; square roots in single precision as in
// the reference (which passes doubles to sqrtf).
template <typename R>
__device__ __forceinline__ R tri_solve(R TA, R TB, R LenAB, R LenBC, R LenAC, R LN) {
  if (TA >= LN && TB >= LN) return LN;
  const R TAB = TB - TA;
  const R a = (LenAB * LenAB - TAB * TAB) * LenAB * LenAB;
  const R EdgeTA = TA + LenAC, EdgeTB = TB + LenBC;
  R TC1 = LN, TC2 = LN;
  if (a > R(0)) {
    const R cosA = (LenAC * LenAC + LenAB * LenAB - LenBC * LenBC) / (R(2) * LenAC * LenAB);
    const R b = R(2) * LenAB * LenAC * cosA * (TAB * TAB - LenAB * LenAB);
    const R delta = R(4) * LenAC * LenAC * a * TAB * TAB * (R(1) - cosA * cosA);
    const R sq = (R)sqrtf((float)delta);
    const R l1 = (-b + sq) / (R(2) * a);
    const R l2 = (-b - sq) / (R(2) * a);
    if (l1 >= R(0) && l1 <= R(1)) {
      const R LenAD = l1 * LenAB;
      const R LenCD = (R)sqrtf((float)(LenAC * LenAC + LenAD * LenAD - R(2) * LenAC * LenAD * cosA));
      TC1 = l1 * TAB + TA + LenCD;
    }
    if (l2 >= R(0) && l2 <= R(1)) {
      const R LenAD = l2 * LenAB;
      const R LenCD = (R)sqrtf((float)(LenAC * LenAC + LenAD * LenAD - R(2) * LenAC * LenAD * cosA));
      TC2 = l2 * TAB + TA + LenCD;
    }
    return rmin(TC2, rmin(TC1, rmin(EdgeTA, EdgeTB)));
  }
  return rmin(EdgeTA, EdgeTB);
}

}  // namespace lsgb
