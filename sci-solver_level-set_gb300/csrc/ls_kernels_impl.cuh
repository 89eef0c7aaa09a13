// ls_kernels_impl.cuh -- sm_103a kernels of the narrowband level-set time step.
// Included twice: by ls_kernels.cu (fast build, FMA contraction on) and by
// ls_kernels_exact.cu (compiled with -fmad=false; with the same operand
// order as the CPU oracle it reproduces the oracle bit for bit).
//
// One step (reference order, src/core3d/cuda/meshFIM3d.cu:639-678):
//   k_reset        DT := LARGENUM, seed := 0, sign := (phi >= 0)     (whole mesh)
//   k_seed         seed points and the first active patch list        (K9)
//   FIM iterations, each:
//     sweep        NITER sweeps on every active patch, fused per-patch
//                  convergence AND and min (K11 + K13)
//     k_schedule   copy-back, unconverged patches to the next list,
//                  neighbours of converged patches with min < w to the
//                  candidate list (the host loop of redistance3d.cu:139-181)
//     check        one-sweep probe of the candidates; unconverged ones join
//                  the next list (K12 + K13 + redistance3d.cu:188-222)
//     The sweep and the check are one kernel with a runtime flag: k_fim
//     (bit-exact build and triangles: one element copy per thread, the
//     reference's solves in its order), k_fim_compact (fast build,
//     tetrahedra: the solves that can lower a value listed and run densely,
//     one copy per thread) and k_fim_pair (the same with two copies per
//     thread, the default for patches of up to 384 copies; its checks also
//     run the visits of the patches they activate on long check lists).
//   k_narrowband   patch narrowband, phi := sign * DT, vertex-update count (K14 + K10b)
//   k_update       advection (K16) or mean-curvature update on narrowband patches
//                  (k_update_384: the same for patches of up to 384 copies,
//                  three CTAs per SM)
//   k_copy_phi     phi := phi_out on narrowband patches (K15)
//   k_unpermute    phi in the caller's vertex order (K18)
//
// Patch visits read a contiguous slab: owned vertex values [vs, ve) plus a
// sorted ghost list, 16-bit slab-local connectivity (one 8-byte load per
// element copy), SoA local coordinates.  The per-vertex minimum of the
// reference's gather/broadcast (redistance_kernels3d.h:418-436) is a shared-
// memory atomicMin on the float bit pattern (values are non-negative), and
// ghost values stay private to each element copy, as in the reference.


__device__ __forceinline__ int warp_id_global() {
  return (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
}

// ---------------------------------------------------------------------------
__global__ void k_reset(DevState s, int nv, float LN) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
    s.DT[v] = LN;
    s.seed[v] = 0;
    s.sign[v] = (s.phi[v] < 0.f) ? 0 : 1;
  }
}

// Seed search (redistance_kernels3d.h:623-770): an element copy whose
// vertex values include an exact zero or differ in sign marks those
// vertices as seeds with DT = |phi|; the patch joins list0.
template <int D1>
__global__ void k_seed(DevMesh m, DevState s, int use_all, float scale, int warm) {
  // use_all < 0: decided on the device from the step-control flag
  if (use_all < 0) use_all = s.ctl[2] ? 0 : 1;
  const int count = use_all ? m.nparts : s.counts[3];
  for (int li = blockIdx.x; li < count; li += gridDim.x) {
    const int p = use_all ? li : s.nblist[li];
    const float sc = m.patch_mesh ? __ldg(&m.mesh_par[m.patch_mesh[p]]).y : scale;
    const int vs = m.vert_off[p], nvp = m.vert_off[p + 1] - vs;
    const int gs = m.ghost_off[p];
    const int es = m.ele_off[p], nep = m.ele_off[p + 1] - es;
    int found = 0;
    for (int c = threadIdx.x; c < nep; c += blockDim.x) {
      const ushort4 cv = m.conn[es + c];
      const int idx[4] = {cv.x, cv.y, cv.z, cv.w};
      int gv[D1];
      float val[D1];
      bool allpos = true, allneg = true;
#pragma unroll
      for (int k = 0; k < D1; ++k) {
        gv[k] = idx[k] < nvp ? vs + idx[k] : m.ghost_ids[gs + idx[k] - nvp];
        val[k] = s.phi[gv[k]];
        allpos &= (val[k] >= 0.f);
        allneg &= (val[k] <= 0.f);
      }
      const bool cross = !(allpos || allneg);
#pragma unroll
      for (int k = 0; k < D1; ++k) {
        if (cross || val[k] == 0.f) {
          s.seed[gv[k]] = 1;
          s.DT[gv[k]] = fabsf(val[k]) / sc;
          found = 1;
        }
      }
    }
    found = __syncthreads_or(found);
    if (threadIdx.x == 0 && (found || warm)) {
      const int pos = atomicAdd(&s.counts[0], 1);
      s.list0[pos] = p;
    }
  }
}

// ---------------------------------------------------------------------------
// FIM patch visit.  CHECK = false: NITER sweeps, writes DT_out and the patch
// convergence / minimum / label (kernel_update_values + run_reduction_
// bandwidth).  CHECK = true: one sweep, no value writes; unconverged
// candidates are appended to the next list (kernel_run_check_neghbor +
// run_reduction3d + redistance3d.cu:214-222).
// Solves of one element copy (Jacobi: all from the values at sweep start).
// With the precision form (tau > 0) a solve whose discriminant cancelled is
// repeated in FP64; `nflag` counts those repeats.
// Fast build: a tet solve whose candidates provably cannot fall below the
// target's current value (min(TA, TB, TC) + 0.999 x D's height over the
// base plane >= T_D) is skipped -- in exact arithmetic it cannot change
// min(T_D, r).  The bit-exact build keeps every solve (the reference's
// arithmetic, including FP32 candidates that fall below that bound).
#ifdef LS_KERNELS_EXACT
constexpr bool kLbSkip = false;
#else
constexpr bool kLbSkip = true;
#endif

// The four solves of one element copy from the values at the sweep start
// (Jacobi within the element), each kept only where it lowers its target.
// Precision-form tets use solve_copy_flags and the deferred FP64 repeats
// instead.
template <int D1, bool XDIV>
__device__ __forceinline__ void solve_copy(const float* Mt, const float T[4], float out[4], float eps_h,
                                           double eps_h64, float LN) {
  if (D1 == 4) {
    const float ACAC = Mt[0], ACBC = Mt[1], ACCD = Mt[2], BCBC = Mt[3], BCCD = Mt[4];
    const float CDCD = Mt[5], ADAD = Mt[6], ADBD = Mt[7], ADCD = Mt[8], BDBD = Mt[9], CDBD = Mt[10];
    const float TA = T[0], TB = T[1], TC = T[2], TD = T[3];
    bool d = false;
    const float r3 = tet_solve<float, XDIV, false, kLbSkip>(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, eps_h,
                                                           eps_h64, LN, 0.f, d, TD);
    const float r0 = tet_solve<float, XDIV, false, kLbSkip>(TB, TD, TC, BCBC, -BCCD, -ACBC, CDCD, ACCD, ACAC, eps_h,
                                                           eps_h64, LN, 0.f, d, TA);
    const float r1 = tet_solve<float, XDIV, false, kLbSkip>(TA, TD, TC, ACAC, -ACCD, -ACBC, CDCD, BCCD, BCBC, eps_h,
                                                           eps_h64, LN, 0.f, d, TB);
    const float r2 = tet_solve<float, XDIV, false, kLbSkip>(TA, TB, TD, ADAD, ADBD, -ADCD, BDBD, -CDBD, CDCD, eps_h,
                                                           eps_h64, LN, 0.f, d, TC);
    out[3] = fminf(TD, r3);
    out[0] = fminf(TA, r0);
    out[1] = fminf(TB, r1);
    out[2] = fminf(TC, r2);
  } else {
    const float LenAB = Mt[0], LenBC = Mt[1], LenCA = Mt[2];
    const float TA = T[0], TB = T[1], TC = T[2];
    out[2] = fminf(TC, tri_solve<float>(TA, TB, LenAB, LenBC, LenCA, LN));
    out[0] = fminf(TA, tri_solve<float>(TB, TC, LenBC, LenCA, LenAB, LN));
    out[1] = fminf(TB, tri_solve<float>(TC, TA, LenCA, LenAB, LenBC, LN));
    out[3] = LN;
  }
}

// Precision form, deferred: the FP32 solves of one tet copy with their
// ill-conditioning flags (the FP64 repeats run later, compacted over the CTA).
template <bool XDIV>
__device__ __forceinline__ void solve_copy_flags(const float* Mt, const float T[4], float r[4], bool ill[4],
                                                 float eps_h, double eps_h64, float LN, float tau) {
  const float ACAC = Mt[0], ACBC = Mt[1], ACCD = Mt[2], BCBC = Mt[3], BCCD = Mt[4];
  const float CDCD = Mt[5], ADAD = Mt[6], ADBD = Mt[7], ADCD = Mt[8], BDBD = Mt[9], CDBD = Mt[10];
  const float TA = T[0], TB = T[1], TC = T[2], TD = T[3];
  ill[0] = ill[1] = ill[2] = ill[3] = false;
  r[3] = tet_solve<float, XDIV, true>(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, eps_h, eps_h64, LN, tau, ill[3], TD);
  r[0] = tet_solve<float, XDIV, true>(TB, TD, TC, BCBC, -BCCD, -ACBC, CDCD, ACCD, ACAC, eps_h, eps_h64, LN, tau, ill[0], TA);
  r[1] = tet_solve<float, XDIV, true>(TA, TD, TC, ACAC, -ACCD, -ACBC, CDCD, BCCD, BCBC, eps_h, eps_h64, LN, tau, ill[1], TB);
  r[2] = tet_solve<float, XDIV, true>(TA, TB, TD, ADAD, ADBD, -ADCD, BDBD, -CDBD, CDCD, eps_h, eps_h64, LN, tau, ill[2], TC);
}

// The FP64 repeat of solve k of a tet copy (same argument order as above).
__device__ __noinline__ float solve_k_fp64(const float* Mt, const float T[4], int k, double eps_h64, float LN) {
  const float ACAC = Mt[0], ACBC = Mt[1], ACCD = Mt[2], BCBC = Mt[3], BCCD = Mt[4];
  const float CDCD = Mt[5], ADAD = Mt[6], ADBD = Mt[7], ADCD = Mt[8], BDBD = Mt[9], CDBD = Mt[10];
  const float TA = T[0], TB = T[1], TC = T[2], TD = T[3];
  const double L64 = LN;
  bool d = false;
  double r;
  switch (k) {
    case 3: r = tet_solve<double, false, false>(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, eps_h64, eps_h64, L64, 0.0, d); break;
    case 0: r = tet_solve<double, false, false>(TB, TD, TC, BCBC, -BCCD, -ACBC, CDCD, ACCD, ACAC, eps_h64, eps_h64, L64, 0.0, d); break;
    case 1: r = tet_solve<double, false, false>(TA, TD, TC, ACAC, -ACCD, -ACBC, CDCD, BCCD, BCBC, eps_h64, eps_h64, L64, 0.0, d); break;
    default: r = tet_solve<double, false, false>(TA, TB, TD, ADAD, ADBD, -ADCD, BDBD, -CDBD, CDCD, eps_h64, eps_h64, L64, 0.0, d); break;
  }
  return (float)r;
}

// One deferred FP64 solve: the copy (CTA-local index << 2 | solve) and its
// four values at the start of the sweep; res = min(T_k, FP64 result).
struct DeferredSolve {
  int code;
  float t[4];
  float res;
};
constexpr int kDeferCap = 1024;
// words of k_fim_pair's shared seed mask (owned vertices per patch it covers: 32 x words)
constexpr int kSeedMaskWords = 32;

template <int D1>
__device__ __forceinline__ void copy_metric(const DevMesh& m, long long c, float* Mt) {
  const long long F = m.full;
  if (D1 == 4) {
    float L[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) L[i] = __ldg(m.lc + i * F + c);
    // redistance_kernels3d.h:381-396
    const float ACBC = L[1] * (L[1] - L[0]) + L[2] * L[2];
    const float BCCD = (L[1] - L[0]) * (L[3] - L[1]) + L[2] * (L[4] - L[2]);
    const float ACCD = L[1] * (L[3] - L[1]) + L[2] * (L[4] - L[2]);
    const float ADBD = L[3] * (L[3] - L[0]) + L[4] * L[4] + L[5] * L[5];
    const float ACAD = L[1] * L[3] + L[2] * L[4];
    const float BCBD = (L[1] - L[0]) * (L[3] - L[0]) + L[2] * L[4];
    const float ADBC = ACBC + BCCD;
    const float ACBD = ACBC + ACCD;
    const float CDBD = ADBD - ACBD;
    const float ADCD = ADBD - ADBC;
    const float CDCD = ADCD - ACCD;
    Mt[0] = ACAD - ACCD;   // ACAC
    Mt[1] = ACBC;
    Mt[2] = ACCD;
    Mt[3] = BCBD - BCCD;   // BCBC
    Mt[4] = BCCD;
    Mt[5] = CDCD;
    Mt[6] = ADCD + ACAD;   // ADAD
    Mt[7] = ADBD;
    Mt[8] = ADCD;
    Mt[9] = BCBD + CDBD;   // BDBD
    Mt[10] = CDBD;
  } else {
    const float c0 = __ldg(m.lc + c), c1 = __ldg(m.lc + F + c), c2 = __ldg(m.lc + 2 * F + c);
    Mt[0] = fabsf(c0);
    Mt[1] = sqrtf(c2 * c2 + (c1 - c0) * (c1 - c0));
    Mt[2] = sqrtf(c1 * c1 + c2 * c2);
  }
}

// The neighbour check and the sweep are one kernel with a runtime flag: both
// must evaluate a patch's first sweep with the same instructions, otherwise
// differently contracted FMAs could make the check report a drop of more
// than the tolerance that the following visit never applies, and two
// patches could re-activate each other without end.
// vb: the CTA's index in the patch assignment (blockIdx.x, or the spread
// index of the persistent kernel)
template <int D1, bool XDIV, bool PREC>
__device__ __forceinline__ void fim_copy_pass(const DevMesh& m, const DevState& s, const StepParams& sp, int cur,
                                              int check, int vb) {
  const bool CHECK = check != 0;
  extern __shared__ float smem[];
  float* sT = smem;                       // owned + ghost values
  float* sOld = smem + sp.lvp + sp.lgp;   // owned values at the start of the last sweep
  __shared__ unsigned s_min;
  __shared__ int s_qn;  // deferred FP64 solves queued in this sweep (precision form)
  DeferredSolve* sQ = reinterpret_cast<DeferredSolve*>(smem + 2 * sp.lvp + sp.lgp);
  if (PREC && threadIdx.x == 0) s_qn = 0;
  const int* list = CHECK ? s.newlist : (cur ? s.list1 : s.list0);
  const int count = CHECK ? s.counts[2] : s.counts[cur];
  const int nxt = cur ^ 1;
  int* nlist = nxt ? s.list1 : s.list0;
  if (!CHECK && blockIdx.x == 0 && threadIdx.x == 0) {
    // the next list and the candidate list are filled by the following kernels
    s.counts[nxt] = 0;
    s.counts[2] = 0;
    if (count > 0) {
      s.counts[4] += 1;
      atomicAdd(&s.stats[5], 1ull);
    }
    atomicAdd(&s.stats[0], (unsigned long long)count);
  }
  if (CHECK && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&s.stats[1], (unsigned long long)count);
  const int niter = CHECK ? 1 : sp.niter;
  const int tid = threadIdx.x;
  for (int li = vb; li < count; li += gridDim.x) {
    const int p = list[li] & ~kPrevisited;  // re-visiting is harmless: same inputs, same results
    const int vs = m.vert_off[p], nvp = m.vert_off[p + 1] - vs;
    const int gs = m.ghost_off[p], ngp = m.ghost_off[p + 1] - gs;
    const int es = m.ele_off[p], nep = m.ele_off[p + 1] - es;
    for (int i = tid; i < nvp + ngp; i += blockDim.x)
      sT[i] = s.DT[i < nvp ? vs + i : __ldg(m.ghost_ids + gs + i - nvp)];
    if (tid == 0) s_min = 0x7f800000u;
    __syncthreads();
    const bool act = tid < nep;
    int idx[4] = {0, 0, 0, 0};
    float T[4] = {0.f, 0.f, 0.f, 0.f};
    float Mt[11];
    int nflag = 0;
    // corners whose value is the vertex's: owned, and within the reference's
    // per-vertex slot limit where that applies (others stay private)
    unsigned shared_k = 0u;
    if (act) {
      const ushort4 cv = m.conn[es + tid];
      idx[0] = cv.x; idx[1] = cv.y; idx[2] = cv.z; idx[3] = cv.w;
      const unsigned capm = m.capped ? (unsigned)m.capped[es + tid] : 0u;
#pragma unroll
      for (int k = 0; k < D1; ++k)
        if (idx[k] < nvp && !((capm >> k) & 1u)) shared_k |= 1u << k;
#pragma unroll
      for (int k = 0; k < D1; ++k) T[k] = sT[idx[k]];
      copy_metric<D1>(m, (long long)es + tid, Mt);
    }
#pragma unroll 1
    for (int it = 0; it < niter; ++it) {
      if (it == niter - 1) {
        for (int i = tid; i < nvp; i += blockDim.x) sOld[i] = sT[i];
        __syncthreads();
      }
      int qpos[4] = {-1, -1, -1, -1};
      if (act) {
        float nw[4];
        if constexpr (PREC && D1 == 4) {
          // FP32 solves; flagged ones go to the CTA's queue for one
          // compacted FP64 pass after the sweep (inline if the queue is full)
          float rr[4];
          bool ill[4];
          solve_copy_flags<XDIV>(Mt, T, rr, ill, sp.eps_h, sp.eps_h64, sp.largenum, sp.tau);
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            if (ill[k]) {
              const int pos = atomicAdd(&s_qn, 1);
              if (pos < kDeferCap) {
                DeferredSolve& e = sQ[pos];
                e.code = (tid << 2) | k;
                e.t[0] = T[0]; e.t[1] = T[1]; e.t[2] = T[2]; e.t[3] = T[3];
                qpos[k] = pos;
                rr[k] = sp.largenum;
              } else {
                rr[k] = solve_k_fp64(Mt, T, k, sp.eps_h64, sp.largenum);
                nflag++;
              }
            }
            nw[k] = fminf(T[k], rr[k]);
          }
        } else {
          solve_copy<D1, XDIV>(Mt, T, nw, sp.eps_h, sp.eps_h64, sp.largenum);
        }
#pragma unroll
        for (int k = 0; k < D1; ++k) {
          if ((shared_k >> k) & 1u) atomicMin(reinterpret_cast<int*>(&sT[idx[k]]), __float_as_int(nw[k]));
          else T[k] = nw[k];
        }
      }
      __syncthreads();
      if constexpr (PREC && D1 == 4) {
        const int nq = min(s_qn, kDeferCap);
        for (int i = tid; i < nq; i += blockDim.x) {
          DeferredSolve& e = sQ[i];
          const int cl = e.code >> 2, k = e.code & 3;
          float Mq[11];
          copy_metric<D1>(m, (long long)es + cl, Mq);
          const float res = fminf(e.t[k], solve_k_fp64(Mq, e.t, k, sp.eps_h64, sp.largenum));
          const ushort4 cv = m.conn[es + cl];
          const int tk = k == 0 ? cv.x : k == 1 ? cv.y : k == 2 ? cv.z : cv.w;
          const bool capped_k = m.capped && ((m.capped[es + cl] >> k) & 1u);
          if (tk < nvp && !capped_k) atomicMin(reinterpret_cast<int*>(&sT[tk]), __float_as_int(res));
          else e.res = res;
          nflag++;
        }
        __syncthreads();
        if (act) {
#pragma unroll
          for (int k = 0; k < 4; ++k)
            if (qpos[k] >= 0 && !((shared_k >> k) & 1u)) T[k] = sQ[qpos[k]].res;
        }
        if (tid == 0) s_qn = 0;
      }
      if (act) {
#pragma unroll
        for (int k = 0; k < D1; ++k)
          if ((shared_k >> k) & 1u) T[k] = sT[idx[k]];
      }
      __syncthreads();
    }
    int con = 1;
    for (int i = tid; i < nvp; i += blockDim.x) {
      const int v = vs + i;
      const float nt = sT[i];
      float outv;
      if (!s.seed[v]) {
        if (!CHECK) s.DT_out[v] = nt;
        con &= (sOld[i] - nt < sp.tol) ? 1 : 0;
        outv = nt;
      } else {
        outv = s.DT[v];
      }
      if (!CHECK) atomicMin(&s_min, __float_as_uint(outv));
    }
    if (D1 == 4 && sp.tau > 0.f) {
      nflag = __reduce_add_sync(0xffffffffu, nflag);
      if ((tid & 31) == 0 && nflag) atomicAdd(&s.stats[6], (unsigned long long)nflag);
    }
    con = __syncthreads_and(con);
    if (tid == 0) {
      if (!CHECK) {
        atomicAdd(&s.stats[7], (unsigned long long)__ldg(m.patch_bytes + p));
        s.bcon[p] = con;
        s.bmin[p] = __uint_as_float(s_min);
        s.blabel[p] = con ? LS_FAR : LS_ACTIVE;
      } else {
        // a check reads the visit's slab but writes no DT_out
        atomicAdd(&s.stats[7], (unsigned long long)(__ldg(m.patch_bytes + p) - 4 * nvp));
        if (!con) {
          const int pos = atomicAdd(&s.counts[nxt], 1);
          nlist[pos] = p;
        } else {
          s.blabel[p] = LS_FAR;
        }
      }
    }
    __syncthreads();
  }
}

template <int D1, int MAXT, bool XDIV, int MINB, bool PREC>
__global__ void __launch_bounds__(MAXT, MINB) k_fim(DevMesh m, DevState s, StepParams sp, int cur, int check) {
  fim_copy_pass<D1, XDIV, PREC>(m, s, sp, cur, check, blockIdx.x);
}

// Patch assignment of the sweep kernels: CTA b takes list entry b first
// (consecutive CTA ids sit on different SMs, so a short list spreads over the
// whole GPU), then draws entries gridDim.x, gridDim.x + 1, ... from the launch
// kind's counter, so that CTAs that drew cheap patches take more.  Only CTAs
// that had a first entry draw, each until its first miss: the draws number
// max(count - gridDim.x, 0) + min(count, gridDim.x), and the last of them
// (value count - 1) resets the counter for the next launch of the kind.
__device__ __forceinline__ int draw_patch(int* next, int count) {
  const int v = atomicAdd(next, 1);
  if (v == count - 1) atomicExch(next, 0);
  return (int)gridDim.x + v;
}

// Fast-build FIM patch visit for tetrahedra with compacted solves.  Same
// visit semantics as k_fim (Jacobi within an element, private ghost values,
// per-vertex minimum, convergence on the last sweep), reorganised so that
// the warps only run solves that can change something: at the start of each
// sweep every element copy tests its four solves with the lower bound of
// solve_copy (min of the three other values + 0.999 x height >= own value
// -> cannot lower it) and appends the others to a CTA list; all threads
// then run the listed solves densely, one solve per thread at a time.
// Shared memory per CTA (stride MAXT): metric [11], heights [4], copy
// values at the sweep start [4], ghost results [4], connectivity, list.
template <int MAXT, int MINB, bool PREC>
__global__ void __launch_bounds__(MAXT, MINB) k_fim_compact(DevMesh m, DevState s, StepParams sp, int cur,
                                                            int check) {
  const bool CHECK = check != 0;
  extern __shared__ float smem[];
  float* sT = smem;                       // owned + ghost values
  float* sOld = smem + sp.lvp + sp.lgp;   // owned values at the start of the last sweep
  float* sM = smem + ((2 * sp.lvp + sp.lgp + 3) & ~3);  // [11][MAXT] metric (16-byte aligned)
  float* sH = sM + 11 * MAXT;             // [4][MAXT] heights of A, B, C, D
  float* sTc = sH + 4 * MAXT;             // [4][MAXT] copy values at the sweep start
  float* sR = sTc + 4 * MAXT;             // [4][MAXT] results for ghost targets
  ushort4* sC = reinterpret_cast<ushort4*>(sR + 4 * MAXT);  // [MAXT] connectivity
  int* sItem = reinterpret_cast<int*>(sC + MAXT);           // [4 * MAXT] listed solves (copy << 2 | k)
  int* sRep = sItem + 4 * MAXT;  // precision form: [4 * MAXT] solves to repeat in FP64
  __shared__ int s_rep;
  __shared__ unsigned s_min;
  __shared__ int s_n[2];  // listed solves, by sweep parity (reset one sweep ahead)
  __shared__ int s_li;    // list entry of the next patch
  const int* list = CHECK ? s.newlist : (cur ? s.list1 : s.list0);
  const int count = CHECK ? s.counts[2] : s.counts[cur];
  const int nxt = cur ^ 1;
  int* nlist = nxt ? s.list1 : s.list0;
  if (!CHECK && blockIdx.x == 0 && threadIdx.x == 0) {
    s.counts[nxt] = 0;
    s.counts[2] = 0;
    if (count > 0) {
      s.counts[4] += 1;
      atomicAdd(&s.stats[5], 1ull);
    }
    atomicAdd(&s.stats[0], (unsigned long long)count);
  }
  if (CHECK && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&s.stats[1], (unsigned long long)count);
  const int niter = CHECK ? 1 : sp.niter;
  const int tid = threadIdx.x;
  // first entry by CTA index, later ones drawn from a counter (draw_patch)
  int* next = s.sched + (CHECK ? 1 : 0);
  if (tid == 0) {
    s_n[0] = s_n[1] = 0;
    s_rep = 0;
    s_li = blockIdx.x;
  }
  __syncthreads();
  int nflag = 0;
  for (int li = s_li; li < count;) {
    const int p = list[li] & ~kPrevisited;  // re-visiting is harmless: same inputs, same results
    const int vs = m.vert_off[p], nvp = m.vert_off[p + 1] - vs;
    const int gs = m.ghost_off[p], ngp = m.ghost_off[p + 1] - gs;
    const int es = m.ele_off[p], nep = m.ele_off[p + 1] - es;
    for (int i = tid; i < nvp + ngp; i += blockDim.x)
      sT[i] = s.DT[i < nvp ? vs + i : __ldg(m.ghost_ids + gs + i - nvp)];
    if (tid == 0) s_min = 0x7f800000u;
    __syncthreads();
    const bool act = tid < nep;
    int idx[4] = {0, 0, 0, 0};
    float T[4] = {0.f, 0.f, 0.f, 0.f};
    float hgt[4] = {0.f, 0.f, 0.f, 0.f};
    if (act) {
      const ushort4 cv = m.conn[es + tid];
      sC[tid] = cv;
      idx[0] = cv.x; idx[1] = cv.y; idx[2] = cv.z; idx[3] = cv.w;
#pragma unroll
      for (int k = 0; k < 4; ++k) T[k] = sT[idx[k]];
      float Mt[11];
      copy_metric<4>(m, (long long)es + tid, Mt);
#pragma unroll
      for (int j = 0; j < 11; ++j) sM[j * MAXT + tid] = Mt[j];
      const float ACAC = Mt[0], ACBC = Mt[1], ACCD = Mt[2], BCBC = Mt[3], BCCD = Mt[4], CDCD = Mt[5];
      const float ADAD = Mt[6], ADBD = Mt[7], BDBD = Mt[9];
      const float det3 = ACAC * (BCBC * CDCD - BCCD * BCCD) - ACBC * (ACBC * CDCD - BCCD * ACCD) +
                         ACCD * (ACBC * BCCD - BCBC * ACCD);
      hgt[0] = sqrtf(fmaxf(det3 / (BCBC * CDCD - BCCD * BCCD), 0.f));  // A over BCD
      hgt[1] = sqrtf(fmaxf(det3 / (ACAC * CDCD - ACCD * ACCD), 0.f));  // B over ACD
      hgt[2] = sqrtf(fmaxf(det3 / (ADAD * BDBD - ADBD * ADBD), 0.f));  // C over ABD
      hgt[3] = sqrtf(fmaxf(det3 / (ACAC * BCBC - ACBC * ACBC), 0.f));  // D over ABC
#pragma unroll
      for (int k = 0; k < 4; ++k) sH[k * MAXT + tid] = hgt[k];
    }
    // vertices of this copy whose value changed in the previous sweep (all
    // on the first): a solve whose three inputs are unchanged returns what
    // it returned before, which cannot lower its target again.
    unsigned chg = 0xFu, ghost = 0u;
    if (act) {
#pragma unroll
      for (int k = 0; k < 4; ++k) ghost |= (idx[k] >= nvp ? 1u : 0u) << k;
    }
#pragma unroll 1
    for (int it = 0; it < niter; ++it) {
      // the owned values at the start of the last sweep (read back by the
      // same thread only; the solves change sT after the listing barrier)
      if (it == niter - 1)
        for (int i = tid; i < nvp; i += blockDim.x) sOld[i] = sT[i];
      // list the solves that can lower their target
      unsigned need = 0;
      if (act) {
#pragma unroll
        for (int k = 0; k < 4; ++k) sTc[k * MAXT + tid] = T[k];
        const float LN = sp.largenum;
        const float m012 = fminf(fminf(T[0], T[1]), T[2]), m013 = fminf(fminf(T[0], T[1]), T[3]);
        const float m023 = fminf(fminf(T[0], T[2]), T[3]), m123 = fminf(fminf(T[1], T[2]), T[3]);
        // apex k: the other three values all LARGENUM -> LARGENUM (as tet_solve)
        // a ghost target's result is only read by later sweeps of the same
        // visit: the last sweep (and a check's only sweep) skips those solves
        const unsigned allow = (it == niter - 1) ? (~ghost & 0xFu) : 0xFu;
        unsigned cand = 0u;
        if (chg & 0xEu) cand |= 1u;
        if (chg & 0xDu) cand |= 2u;
        if (chg & 0xBu) cand |= 4u;
        if (chg & 0x7u) cand |= 8u;
        cand &= allow;
        if ((cand & 1u) && m123 < LN && m123 + 0.999f * hgt[0] < T[0]) need |= 1u;
        if ((cand & 2u) && m023 < LN && m023 + 0.999f * hgt[1] < T[1]) need |= 2u;
        if ((cand & 4u) && m013 < LN && m013 + 0.999f * hgt[2] < T[2]) need |= 4u;
        if ((cand & 8u) && m012 < LN && m012 + 0.999f * hgt[3] < T[3]) need |= 8u;
        const int n = __popc(need);
        if (n) {
          int pos = atomicAdd(&s_n[it & 1], n);
#pragma unroll
          for (int k = 0; k < 4; ++k)
            if (need & (1u << k)) sItem[pos++] = (tid << 2) | k;
        }
      }
      __syncthreads();
      const int nitems = s_n[it & 1];
      // the other parity's counter is idle until the next sweep's listing,
      // which starts after the barrier below
      if (tid == 0) s_n[(it & 1) ^ 1] = 0;
      // nothing listed: this sweep changes nothing, so every later sweep of
      // the visit has the same inputs and lists nothing either; the visit
      // ends here, and the convergence test sees no change, as it would
      // after the remaining empty sweeps (same bits as running them)
      if (nitems == 0 && it < niter - 1) {
        for (int i = tid; i < nvp; i += blockDim.x) sOld[i] = sT[i];
        break;
      }
      for (int i = tid; i < nitems; i += blockDim.x) {
        const int code = sItem[i];
        const int cc = code >> 2, k = code & 3;
        const float TA = sTc[cc], TB = sTc[MAXT + cc], TC = sTc[2 * MAXT + cc], TD = sTc[3 * MAXT + cc];
        const float ACAC = sM[cc], ACBC = sM[MAXT + cc], ACCD = sM[2 * MAXT + cc], BCBC = sM[3 * MAXT + cc];
        const float BCCD = sM[4 * MAXT + cc], CDCD = sM[5 * MAXT + cc], ADAD = sM[6 * MAXT + cc];
        const float ADBD = sM[7 * MAXT + cc], ADCD = sM[8 * MAXT + cc], BDBD = sM[9 * MAXT + cc];
        const float CDBD = sM[10 * MAXT + cc];
        // the permuted arguments of solve k (solve_copy's four calls)
        float a0, a1, a2, g0, g1, g2, g3, g4, g5, own;
        if (k == 3) { a0 = TA; a1 = TB; a2 = TC; g0 = ACAC; g1 = ACBC; g2 = ACCD; g3 = BCBC; g4 = BCCD; g5 = CDCD; own = TD; }
        else if (k == 0) { a0 = TB; a1 = TD; a2 = TC; g0 = BCBC; g1 = -BCCD; g2 = -ACBC; g3 = CDCD; g4 = ACCD; g5 = ACAC; own = TA; }
        else if (k == 1) { a0 = TA; a1 = TD; a2 = TC; g0 = ACAC; g1 = -ACCD; g2 = -ACBC; g3 = CDCD; g4 = BCCD; g5 = BCBC; own = TB; }
        else { a0 = TA; a1 = TB; a2 = TD; g0 = ADAD; g1 = ADBD; g2 = -ADCD; g3 = BDBD; g4 = -CDBD; g5 = CDCD; own = TC; }
        bool ill = false;
        float r;
        if constexpr (PREC)
          r = tet_solve_pred<true>(a0, a1, a2, g0, g1, g2, g3, g4, g5, sp.eps_h, sp.largenum, sp.tau, &ill);
        else
          r = tet_solve_wave(a0, a1, a2, g0, g1, g2, g3, g4, g5, sH[k * MAXT + cc], sp.eps_h, sp.largenum);
        if (PREC && ill) {
          // discriminant cancelled: repeat in FP64 after this pass, densely
          sRep[atomicAdd(&s_rep, 1)] = code;
          continue;
        }
        const float nw = fminf(own, r);
        const ushort4 cv = sC[cc];
        const int tk = k == 0 ? cv.x : k == 1 ? cv.y : k == 2 ? cv.z : cv.w;
        if (tk < nvp) atomicMin(reinterpret_cast<int*>(&sT[tk]), __float_as_int(nw));
        else sR[k * MAXT + cc] = nw;
      }
      __syncthreads();
      if constexpr (PREC) {
        const int nrep = s_rep;
        for (int i = tid; i < nrep; i += blockDim.x) {
          const int code = sRep[i];
          const int cc = code >> 2, k = code & 3;
          float Mq[11], Tq[4];
#pragma unroll
          for (int j = 0; j < 11; ++j) Mq[j] = sM[j * MAXT + cc];
#pragma unroll
          for (int j = 0; j < 4; ++j) Tq[j] = sTc[j * MAXT + cc];
          const float nw = fminf(Tq[k], solve_k_fp64(Mq, Tq, k, sp.eps_h64, sp.largenum));
          const ushort4 cv = sC[cc];
          const int tk = k == 0 ? cv.x : k == 1 ? cv.y : k == 2 ? cv.z : cv.w;
          if (tk < nvp) atomicMin(reinterpret_cast<int*>(&sT[tk]), __float_as_int(nw));
          else sR[k * MAXT + cc] = nw;
          nflag++;
        }
        __syncthreads();
        if (tid == 0) s_rep = 0;
      }
      if (act) {
        chg = 0u;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float old = T[k];
          if (idx[k] < nvp) T[k] = sT[idx[k]];
          else if (need & (1u << k)) T[k] = sR[k * MAXT + tid];
          if (T[k] != old) chg |= 1u << k;
        }
      }
      // no barrier here: the next sweep's solves change sT only after the
      // barrier that follows its listing (Jacobi order is kept)
    }
    __syncthreads();
    if (tid == 0) s_n[0] = s_n[1] = 0;  // read by every thread before the barrier above
    int con = 1;
    for (int i = tid; i < nvp; i += blockDim.x) {
      const int v = vs + i;
      const float nt = sT[i];
      float outv;
      if (!s.seed[v]) {
        if (!CHECK) s.DT_out[v] = nt;
        con &= (sOld[i] - nt < sp.tol) ? 1 : 0;
        outv = nt;
      } else {
        outv = s.DT[v];
      }
      if (!CHECK) atomicMin(&s_min, __float_as_uint(outv));
    }
    con = __syncthreads_and(con);
    if (tid == 0) {
      if (!CHECK) {
        atomicAdd(&s.stats[7], (unsigned long long)__ldg(m.patch_bytes + p));
        s.bcon[p] = con;
        s.bmin[p] = __uint_as_float(s_min);
        s.blabel[p] = con ? LS_FAR : LS_ACTIVE;
      } else {
        // a check reads the visit's slab but writes no DT_out
        atomicAdd(&s.stats[7], (unsigned long long)(__ldg(m.patch_bytes + p) - 4 * nvp));
        if (!con) {
          const int pos = atomicAdd(&s.counts[nxt], 1);
          nlist[pos] = p;
        } else {
          s.blabel[p] = LS_FAR;
        }
      }
    }
    __syncthreads();
    if (tid == 0) s_li = draw_patch(next, count);
    __syncthreads();
    li = s_li;
  }
  if (PREC) {
    nflag = __reduce_add_sync(0xffffffffu, nflag);
    if ((tid & 31) == 0 && nflag) atomicAdd(&s.stats[6], (unsigned long long)nflag);
  }
}

// Local solver of the two-copies-per-thread sweep: the fast build's
// planar-wave solver with the lower-bound skip (kPairWave), or the
// reference's solver in its operand order, every listed solve run (the
// bit-exact build; kPairRefXdiv with the interior division in double, as
// the reference semantics there).
constexpr int kPairWave = 0, kPairRef = 1, kPairRefXdiv = 2;

// Can solve k (listed as a candidate: its inputs changed) lower its target
// T_k?  Not when the three other values are all LARGENUM (the solver returns
// LARGENUM); with the planar-wave solver also not when min of them plus
// 0.999 x the target's height over their face is at least T_k (the lower
// bound of every candidate in exact arithmetic).  The reference solver's
// FP32 candidates can fall below that bound, so the bit-exact build keeps
// those solves.
template <int SOLVER>
__device__ __forceinline__ bool pair_may_lower(unsigned cand, float mn, float hk, float tk, float LN) {
  if (!cand || !(mn < LN)) return false;
  if constexpr (SOLVER == kPairWave) return mn + 0.999f * hk < tk;
  return true;
}

// One listed solve of k_fim_pair: solve k of copy cc from the copy values
// at the sweep start; the result lowers the owned target's shared value or
// becomes the copy's private ghost value.
template <int SOLVER>
__device__ __forceinline__ void pair_solve(int code, const float4* sTc, const float4* sM, const float4* sH,
                                           const ushort4* sC, float* sT, float4* sR, int nvp, const StepParams& sp) {
  const int cc = code >> 2, k = code & 3;
  const float4 tv = sTc[cc];
  const float TA = tv.x, TB = tv.y, TC = tv.z, TD = tv.w;
  // the six metric terms of solve k (k_geometry's record: floats 0-5 for
  // solves 0, 1, 3, floats 6-11 for solve 2), v0 .. v5 = ACAC ACBC ACCD BCBC
  // BCCD CDCD, or ADAD ADBD ADCD BDBD CDBD CDCD
  const float2* mp = reinterpret_cast<const float2*>(sM) + 6 * cc + (k == 2 ? 3 : 0);
  const float2 p0 = mp[0], p1 = mp[1], p2 = mp[2];
  const float v0 = p0.x, v1 = p0.y, v2 = p1.x, v3 = p1.y, v4 = p2.x, v5 = p2.y;
  // the permuted arguments of solve k (solve_copy's four calls)
  float a0, a1, a2, g0, g1, g2, g3, g4, g5, own;
  if (k == 3) { a0 = TA; a1 = TB; a2 = TC; g0 = v0; g1 = v1; g2 = v2; g3 = v3; g4 = v4; g5 = v5; own = TD; }
  else if (k == 0) { a0 = TB; a1 = TD; a2 = TC; g0 = v3; g1 = -v4; g2 = -v1; g3 = v5; g4 = v2; g5 = v0; own = TA; }
  else if (k == 1) { a0 = TA; a1 = TD; a2 = TC; g0 = v0; g1 = -v2; g2 = -v1; g3 = v5; g4 = v4; g5 = v3; own = TB; }
  else { a0 = TA; a1 = TB; a2 = TD; g0 = v0; g1 = v1; g2 = -v2; g3 = v3; g4 = -v4; g5 = v5; own = TC; }
  float r;
  if constexpr (SOLVER == kPairWave) {
    // the target's height: component k of the copy's record, loaded alone
    const float hD = reinterpret_cast<const float*>(sH)[4 * cc + k];
    r = tet_solve_wave(a0, a1, a2, g0, g1, g2, g3, g4, g5, hD, sp.eps_h, sp.largenum);
  } else {
    bool d = false;
    r = tet_solve<float, SOLVER == kPairRefXdiv, false, false>(a0, a1, a2, g0, g1, g2, g3, g4, g5, sp.eps_h,
                                                                sp.eps_h64, sp.largenum, 0.f, d, own);
  }
  const float nw = fminf(own, r);
  // the target's slab index: component k of the copy's connectivity
  const int tk = reinterpret_cast<const unsigned short*>(sC)[4 * cc + k];
  if (tk < nvp) atomicMin(reinterpret_cast<int*>(&sT[tk]), __float_as_int(nw));
  else reinterpret_cast<float*>(sR)[4 * cc + k] = nw;
}

// Per-copy geometry of the two-copies-per-thread sweep, computed once per
// mesh: the copy's metric terms (copy_metric) as three float4 -- ACAC ACBC
// ACCD BCBC | BCCD CDCD ADAD ADBD | ADCD BDBD CDBD CDCD, so that floats 0-5
// hold the six terms solves 0, 1 and 3 permute and floats 6-11 the six of
// solve 2 -- and the heights of its four vertices over their opposite faces,
// the same expressions the one-copy kernels evaluate per visit.
__global__ void k_geometry(DevMesh m, float4* gm, float4* gh) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < m.full; c += stride) {
    float Mt[11];
    copy_metric<4>(m, c, Mt);
    gm[3 * c] = make_float4(Mt[0], Mt[1], Mt[2], Mt[3]);
    gm[3 * c + 1] = make_float4(Mt[4], Mt[5], Mt[6], Mt[7]);
    gm[3 * c + 2] = make_float4(Mt[8], Mt[9], Mt[10], Mt[5]);
    const float ACAC = Mt[0], ACBC = Mt[1], ACCD = Mt[2], BCBC = Mt[3], BCCD = Mt[4], CDCD = Mt[5];
    const float ADAD = Mt[6], ADBD = Mt[7], BDBD = Mt[9];
    const float det3 = ACAC * (BCBC * CDCD - BCCD * BCCD) - ACBC * (ACBC * CDCD - BCCD * ACCD) +
                       ACCD * (ACBC * BCCD - BCBC * ACCD);
    gh[c] = make_float4(sqrtf(fmaxf(det3 / (BCBC * CDCD - BCCD * BCCD), 0.f)),   // A over BCD
                        sqrtf(fmaxf(det3 / (ACAC * CDCD - ACCD * ACCD), 0.f)),   // B over ACD
                        sqrtf(fmaxf(det3 / (ADAD * BDBD - ADBD * ADBD), 0.f)),   // C over ABD
                        sqrtf(fmaxf(det3 / (ACAC * BCBC - ACBC * ACBC), 0.f)));  // D over ABC
  }
}

// Bulk asynchronous copies of a patch's geometry slabs into shared memory,
// completed on a CTA mbarrier (one phase per patch, one arrival: the issuing
// thread's, which also sets the expected bytes).  Sources are this GPU's
// global memory, destinations this CTA's shared memory; both slabs start on
// 16-byte boundaries and are multiples of 16 bytes long (float4 records).
constexpr long long kSlabWaitCycles = 1ll << 31;  // about one second at the SM clock

__device__ __forceinline__ unsigned smem_u32addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void slab_bar_init(unsigned bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void slab_bar_inval(unsigned bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
}

// The geometry records stream through L2 (about 1.6 GB at 128^3, each read
// once or twice per step): the copies carry an evict-first L2 policy so that
// the small arrays on a patch visit's dependent-load chain (list entries,
// patch offsets, ghost ids, DT) stay in L2.
__device__ __forceinline__ void geo_issue(const DevMesh& m, int es, int nep, float4* sM, float4* sH, unsigned bar) {
  const unsigned bm = 48u * (unsigned)nep, bh = 16u * (unsigned)nep;
  asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(bar),
               "r"(bm + bh)
               : "memory");
  if (nep > 0) {
    unsigned long long pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
            smem_u32addr(sM)),
        "l"(__cvta_generic_to_global(m.geo_m + 3ll * es)), "r"(bm), "r"(bar), "l"(pol)
        : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
            smem_u32addr(sH)),
        "l"(__cvta_generic_to_global(m.geo_h + es)), "r"(bh), "r"(bar), "l"(pol)
        : "memory");
  }
}

// Bounded wait for the phase of the given parity: true once it completed,
// false after kSlabWaitCycles (at once when give_up is set: the test setting
// of the timeout path).
__device__ __forceinline__ bool slab_wait(unsigned bar, unsigned parity, bool give_up) {
  if (give_up) return false;
  const long long t0 = clock64();
  while (true) {
    unsigned ok;
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    if (ok) return true;
    if (clock64() - t0 > kSlabWaitCycles) return false;
  }
}

// Fast-build FIM patch visit for tetrahedra, two element copies per thread.
// The same sweep as k_fim_compact (listing with the lower bound, the
// unchanged-input and unread-ghost skips; dense predicated solves; per-vertex
// minimum; private ghost values) with each copy's carried state in shared
// memory instead of registers, so that a patch of up to 384 copies runs on
// at most 192 threads and five patches are resident per SM (the one-copy
// kernel fits three): the CTA barriers between the listing, solve and
// refresh phases then leave fewer issue slots idle.  Shared memory per CTA
// (ncap = the largest patch's copies, at most 2 x blockDim): copy values
// float4 [ncap] (carried across sweeps), metric float4 [3][ncap] (11 terms
// and a second CDCD, copy-major), heights float4 [ncap], ghost results float4 [ncap],
// connectivity ushort4 [ncap], listed solves ushort [4 ncap] (copy << 2 | k);
// each thread keeps its two copies' flags (changed and ghost vertices) and
// connectivity in registers as well (its own refresh reads them there; the
// solves of other threads read the shared copy).
// The metric and height slabs come from the per-mesh geometry records
// (k_geometry) by two bulk asynchronous copies that thread 0 issues at the
// start of each patch; they land while the threads gather the values and
// load the connectivity, and thread 0 waits for them (bounded) before the
// setup barrier.  A wait that runs out sets ctl[3] = 2, waits once more for
// the copies in flight and ends the CTA's pass; the host then reports
// LS_DEVICE_TIMEOUT.
// Patches: the list entry of the CTA's index first, later ones from
// draw_patch.  On a check launch of at least two patches per CTA, a check
// that finds its patch unconverged goes on to run that patch's visit (the
// next iteration's visit would read the same DT) and marks the patch's entry
// in the next list with kPrevisited; the next sweep skips marked entries.
template <int SOLVER>
__device__ __forceinline__ void fim_pair_pass(const DevMesh& m, const DevState& s, const StepParams& sp, int cur,
                                              int check, int vb) {
  const bool CHECK = check != 0;
  extern __shared__ float4 smem4[];
  float* sT = reinterpret_cast<float*>(smem4);  // owned + ghost values
  float* sOld = sT + sp.lvp + sp.lgp;          // owned values at the start of the last sweep
  const int ncap = sp.lep;
  float4* sTc = smem4 + (((2 * sp.lvp + sp.lgp + 3) & ~3) >> 2);
  float4* sM = sTc + ncap;
  float4* sH = sM + 3 * ncap;
  float4* sR = sH + ncap;
  ushort4* sC = reinterpret_cast<ushort4*>(sR + ncap);
  unsigned short* sItem = reinterpret_cast<unsigned short*>(sC + ncap);
  __shared__ unsigned s_min;
  __shared__ int s_n[2];  // listed solves, by sweep parity (reset one sweep ahead)
  __shared__ int s_li;    // list entry of the next patch
  __shared__ int s_ng;    // ghost-target solves listed when a check becomes a visit
  __shared__ unsigned s_seed[kSeedMaskWords];  // seed flags of the owned vertices (bit i = vertex i)
  __shared__ __align__(8) unsigned long long s_bar;  // geometry slab copies of the current patch
  __shared__ int s_err;  // a slab wait ran out: the pass ends
  const int* list = CHECK ? s.newlist : (cur ? s.list1 : s.list0);
  const int count = CHECK ? s.counts[2] : s.counts[cur];
  const int nxt = cur ^ 1;
  int* nlist = nxt ? s.list1 : s.list0;
  if (!CHECK && blockIdx.x == 0 && threadIdx.x == 0) {
    s.counts[nxt] = 0;
    s.counts[2] = 0;
    if (count > 0) {
      s.counts[4] += 1;
      atomicAdd(&s.stats[5], 1ull);
    }
    atomicAdd(&s.stats[0], (unsigned long long)count);
  }
  if (CHECK && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&s.stats[1], (unsigned long long)count);
  const int niter = CHECK ? 1 : sp.niter;
  const int tid = threadIdx.x;
  const unsigned bar = smem_u32addr(&s_bar);
  unsigned phase = 0;      // thread 0: parity of the slab copies' current phase
  bool in_flight = false;  // thread 0: copies whose wait ran out twice
  // first entry by CTA index, later ones drawn from a counter (draw_patch)
  int* next = s.sched + (CHECK ? 1 : 0);
  // visits run by the checks that activate them only pay when the check
  // launch is throughput bound (four checks or more per resident CTA, the
  // best of 1, 2, 4 and 8 measured at 128^3): on fewer patches they add a
  // visit's length to the iteration, while the next sweep launch still waits
  // for the patches that stayed active
  const bool early = CHECK && sp.niter > 1 && count >= 4 * (int)gridDim.x;
  // the owned vertices' seed flags are kept in shared memory when every patch
  // fits the mask (read by the check's verdict and the copy-out)
  const bool seed_mask = sp.lvp <= 32 * kSeedMaskWords;
  if (tid == 0) {
    s_n[0] = s_n[1] = 0;
    s_li = vb;
    s_err = 0;
    slab_bar_init(bar);
  }
  __syncthreads();
  for (int li = s_li; li < count;) {
    const int entry = list[li];
    // an entry marked as visited ahead was visited by the check that activated
    // it, from the inputs this sweep would read: nothing is left to do
    if (!(entry & kPrevisited)) {
      const int p = entry;
      const int vs = m.vert_off[p], nvp = m.vert_off[p + 1] - vs;
      const int gs = m.ghost_off[p], ngp = m.ghost_off[p + 1] - gs;
      const int es = m.ele_off[p], nep = m.ele_off[p + 1] - es;
      // the metric and height slabs: in flight while the values, seed flags
      // and connectivity load (the previous patch's last reads of sM and sH
      // came before its final barrier)
      if (tid == 0) geo_issue(m, es, nep, sM, sH, bar);
      // every load of the patch's own slab is issued before any of them is
      // stored (values, seed flags, connectivity: independent round trips
      // that overlap; a ghost value waits only for its id), then stored.
      // First slab entry, seed flag and copies of each thread:
      const int nslab = nvp + ngp;
      const int gv0 = tid < nvp ? vs + tid : (tid < nslab ? __ldg(m.ghost_ids + gs + tid - nvp) : -1);
      const bool sd0 = seed_mask && tid < nvp && s.seed[vs + tid] != 0;
      ushort4 cvv[2];
  #pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int c = tid + j * blockDim.x;
        if (c < nep) cvv[j] = __ldcs(m.conn + es + c);  // streamed, like the geometry records (evict-first)
      }
      const float dt0 = gv0 >= 0 ? s.DT[gv0] : 0.f;
      if (tid < nslab) sT[tid] = dt0;
      for (int i = tid + blockDim.x; i < nslab; i += blockDim.x)
        sT[i] = s.DT[i < nvp ? vs + i : __ldg(m.ghost_ids + gs + i - nvp)];
      // whole warps run each 32-vertex word (the block is whole warps and the
      // bound a multiple of 32)
      if (seed_mask)
        for (int i = tid; i < ((nvp + 31) & ~31); i += blockDim.x) {
          const bool sd = i == tid ? sd0 : (i < nvp && s.seed[vs + i] != 0);
          const unsigned b = __ballot_sync(0xffffffffu, sd);
          if ((i & 31) == 0) s_seed[i >> 5] = b;
        }
      // the copies' connectivity (the previous patch's last reads of sC came
      // before its final barrier) and flags, which only this thread reads:
      // bits 8j .. 8j+3 the vertices of copy j that changed in the previous
      // sweep (all on the first), bits 8j+4 .. 8j+7 its ghost vertices
      unsigned flags = 0u;
  #pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int c = tid + j * blockDim.x;
        if (c < nep) {
          const ushort4 cv = cvv[j];
          sC[c] = cv;
          const unsigned ghost = (cv.x >= nvp ? 1u : 0u) | (cv.y >= nvp ? 2u : 0u) | (cv.z >= nvp ? 4u : 0u) |
                                 (cv.w >= nvp ? 8u : 0u);
          flags |= (0xFu | (ghost << 4)) << (8 * j);
        }
      }
      if (tid == 0) {
        s_min = 0x7f800000u;
        s_ng = 0;
        if (!slab_wait(bar, phase, sp.spin_limit < 0)) {
          // abandoned: the host reports a timeout; the copies are waited for
          // once more so that none is in flight when the CTA leaves
          atomicExch(s.ctl + 3, 2);
          in_flight = !slab_wait(bar, phase, false);
          s_err = 1;
        }
        phase ^= 1u;
      }
      __syncthreads();
      if (s_err) break;
      auto is_seed = [&](int i) -> bool {
        return seed_mask ? ((s_seed[i >> 5] >> (i & 31)) & 1u) != 0u : s.seed[vs + i] != 0;
      };
      // each thread's copies' values at the first sweep (read by the listing of
      // the same thread, and by all solves after the listing's barrier)
  #pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int c = tid + j * blockDim.x;
        if (c < nep) {
          const ushort4 cv = cvv[j];
          sTc[c] = make_float4(sT[cv.x], sT[cv.y], sT[cv.z], sT[cv.w]);
        }
      }
      // a check that finds its patch unconverged turns into that patch's visit
      int niter_p = niter;
      bool visit = !CHECK;
      int check_con = 1;  // the verdict of a check that stays a check
      unsigned need[2] = {0u, 0u};
  #pragma unroll 1
      for (int it = 0; it < niter_p; ++it) {
        // the owned values at the start of the last sweep (read back by the
        // same thread only; this sweep's solves change sT only after the
        // listing barrier below, so no barrier of its own)
        if (it == niter_p - 1)
          for (int i = tid; i < nvp; i += blockDim.x) sOld[i] = sT[i];
        // list this thread's solves that can lower their target (the tests of
        // k_fim_compact)
        const unsigned allow_ghost = (it == niter_p - 1) ? 0u : 0xFu;
  #pragma unroll
        for (int j = 0; j < 2; ++j) {
          const int c = tid + j * blockDim.x;
          need[j] = 0u;
          // a copy none of whose values changed in the previous sweep lists
          // nothing: its flags are read first
          const unsigned fl = (flags >> (8 * j)) & 0xFFu;  // zero past nep
          if (fl & 0xFu) {
            const float4 tv = sTc[c];
            const float4 hv = sH[c];
            const unsigned chg = fl & 0xFu, ghost = fl >> 4;
            const float LN = sp.largenum;
            const float m012 = fminf(fminf(tv.x, tv.y), tv.z), m013 = fminf(fminf(tv.x, tv.y), tv.w);
            const float m023 = fminf(fminf(tv.x, tv.z), tv.w), m123 = fminf(fminf(tv.y, tv.z), tv.w);
            unsigned cand = 0u;
            if (chg & 0xEu) cand |= 1u;
            if (chg & 0xDu) cand |= 2u;
            if (chg & 0xBu) cand |= 4u;
            if (chg & 0x7u) cand |= 8u;
            cand &= (~ghost | allow_ghost) & 0xFu;
            unsigned nd = 0u;
            if (pair_may_lower<SOLVER>(cand & 1u, m123, hv.x, tv.x, LN)) nd |= 1u;
            if (pair_may_lower<SOLVER>(cand & 2u, m023, hv.y, tv.y, LN)) nd |= 2u;
            if (pair_may_lower<SOLVER>(cand & 4u, m013, hv.z, tv.z, LN)) nd |= 4u;
            if (pair_may_lower<SOLVER>(cand & 8u, m012, hv.w, tv.w, LN)) nd |= 8u;
            need[j] = nd;
          }
        }
        {
          // list positions: one shared atomic per thread for both copies
          const int nt = __popc(need[0]) + __popc(need[1]);
          if (nt) {
            int pos = atomicAdd(&s_n[it & 1], nt);
  #pragma unroll
            for (int j = 0; j < 2; ++j) {
              const int c = tid + j * blockDim.x;
  #pragma unroll
              for (int k = 0; k < 4; ++k)
                if (need[j] & (1u << k)) sItem[pos++] = (unsigned short)((c << 2) | k);
            }
          }
        }
        __syncthreads();
        const int nitems = s_n[it & 1];
        // the other parity's counter is idle until the next sweep's listing,
        // which starts after the barrier below
        if (tid == 0) s_n[(it & 1) ^ 1] = 0;
        // nothing listed in a visit's sweep before its last: no later sweep
        // lists anything either (unchanged inputs), so the visit ends here
        // with the bits the remaining empty sweeps would leave
        if (nitems == 0 && visit && it < niter_p - 1) {
          for (int i = tid; i < nvp; i += blockDim.x) sOld[i] = sT[i];
          break;
        }
        for (int i = tid; i < nitems; i += blockDim.x) pair_solve<SOLVER>(sItem[i], sTc, sM, sH, sC, sT, sR, nvp, sp);
        __syncthreads();
        if (CHECK && !visit) {
          // the check's verdict (as at the end of a check): does an owned
          // vertex drop by tol or more?
          int c0 = 1;
          for (int i = tid; i < nvp; i += blockDim.x)
            if (!is_seed(i)) c0 &= (sOld[i] - sT[i] < sp.tol) ? 1 : 0;
          check_con = __syncthreads_and(c0);
          if (!check_con && early) {
            // activated: the patch's visit in the next FIM iteration would read
            // the same DT (DT changes only in the copy-back after the sweeps), so
            // it runs here and the next sweep skips the patch.  This sweep was
            // its first sweep minus the ghost targets (the check's last-sweep
            // rule): list and run those from the same sweep-start values.
            visit = true;
            niter_p = sp.niter;
  #pragma unroll
            for (int j = 0; j < 2; ++j) {
              const int c = tid + j * blockDim.x;
              if (c < nep) {
                const float4 tv = sTc[c];
                const float4 hv = sH[c];
                const unsigned ghost = (flags >> (8 * j + 4)) & 0xFu;  // all four inputs count as changed
                const float LN = sp.largenum;
                const float m012 = fminf(fminf(tv.x, tv.y), tv.z), m013 = fminf(fminf(tv.x, tv.y), tv.w);
                const float m023 = fminf(fminf(tv.x, tv.z), tv.w), m123 = fminf(fminf(tv.y, tv.z), tv.w);
                unsigned nd = 0u;
                if (pair_may_lower<SOLVER>(ghost & 1u, m123, hv.x, tv.x, LN)) nd |= 1u;
                if (pair_may_lower<SOLVER>(ghost & 2u, m023, hv.y, tv.y, LN)) nd |= 2u;
                if (pair_may_lower<SOLVER>(ghost & 4u, m013, hv.z, tv.z, LN)) nd |= 4u;
                if (pair_may_lower<SOLVER>(ghost & 8u, m012, hv.w, tv.w, LN)) nd |= 8u;
                need[j] |= nd;
                const int n = __popc(nd);
                if (n) {
                  int pos = nitems + atomicAdd(&s_ng, n);
  #pragma unroll
                  for (int k = 0; k < 4; ++k)
                    if (nd & (1u << k)) sItem[pos++] = (unsigned short)((c << 2) | k);
                }
              }
            }
            __syncthreads();
            const int ng = s_ng;
            for (int i = tid; i < ng; i += blockDim.x) pair_solve<SOLVER>(sItem[nitems + i], sTc, sM, sH, sC, sT, sR, nvp, sp);
            __syncthreads();
          }
        }
        // refresh this thread's copies: owned vertices from the per-vertex
        // minimum, ghost vertices from this sweep's own result where solved
        // (not after the last sweep: only the owned values are read then)
        if (it == niter_p - 1) break;
  #pragma unroll
        for (int j = 0; j < 2; ++j) {
          const int c = tid + j * blockDim.x;
          if (c < nep) {
            const float4 tv = sTc[c];
            const float4 rv = sR[c];
            const ushort4 cv = cvv[j];
            const unsigned nd = need[j];
            float4 nv;
            nv.x = cv.x < nvp ? sT[cv.x] : ((nd & 1u) ? rv.x : tv.x);
            nv.y = cv.y < nvp ? sT[cv.y] : ((nd & 2u) ? rv.y : tv.y);
            nv.z = cv.z < nvp ? sT[cv.z] : ((nd & 4u) ? rv.z : tv.z);
            nv.w = cv.w < nvp ? sT[cv.w] : ((nd & 8u) ? rv.w : tv.w);
            const unsigned chg = (nv.x != tv.x ? 1u : 0u) | (nv.y != tv.y ? 2u : 0u) | (nv.z != tv.z ? 4u : 0u) |
                                 (nv.w != tv.w ? 8u : 0u);
            sTc[c] = nv;
            flags = (flags & ~(0xFu << (8 * j))) | (chg << (8 * j));
          }
        }
        // no barrier here: every thread refreshes only its own copies, and the
        // next sweep's solves read them after the barrier that follows its
        // listing
      }
      __syncthreads();
      // the next list entry is drawn here (draw_patch in two parts), its
      // atomic in flight during the copy-out below; s_li was read by every
      // thread before the barrier above, and is read again after the one
      // below
      int drawn = 0;
      if (tid == 0) {
        s_n[0] = s_n[1] = 0;  // read by every thread before the barrier above
        drawn = atomicAdd(next, 1);
      }
      // a check that stayed a check keeps its verdict: it writes no values
      int con = visit ? 1 : check_con;
      if (visit)
        for (int i = tid; i < nvp; i += blockDim.x) {
          const int v = vs + i;
          const float nt = sT[i];
          float outv;
          if (!is_seed(i)) {
            s.DT_out[v] = nt;
            con &= (sOld[i] - nt < sp.tol) ? 1 : 0;
            outv = nt;
          } else {
            outv = s.DT[v];
          }
          atomicMin(&s_min, __float_as_uint(outv));
        }
      if (tid == 0) {
        if (drawn == count - 1) atomicExch(next, 0);
        s_li = (int)gridDim.x + drawn;
      }
      con = __syncthreads_and(con);
      li = s_li;
      if (tid == 0) {
        if (visit) {
          atomicAdd(&s.stats[7], (unsigned long long)__ldg(m.patch_bytes + p));
          s.bcon[p] = con;
          s.bmin[p] = __uint_as_float(s_min);
          s.blabel[p] = con ? LS_FAR : LS_ACTIVE;
        }
        if (CHECK) {
          // a check that stayed a check read the visit's slab but wrote no DT_out
          if (!visit) atomicAdd(&s.stats[7], (unsigned long long)(__ldg(m.patch_bytes + p) - 4 * nvp));
          if (visit) atomicAdd(&s.stats[8], 1ull);
          if (visit || !con) {
            // activated: joins the next iteration's list (marked when visited
            // here already)
            const int pos = atomicAdd(&s.counts[nxt], 1);
            nlist[pos] = visit ? (p | kPrevisited) : p;
          } else {
            s.blabel[p] = LS_FAR;
          }
        }
      }
    } else {
      __syncthreads();
      if (tid == 0) s_li = draw_patch(next, count);
      __syncthreads();
      li = s_li;
    }
  }
  // every phase was waited for (unless a copy stayed in flight after a
  // timeout): the mbarrier can go
  if (tid == 0 && !in_flight) slab_bar_inval(bar);
}

// FIM settings of the two-copies-per-thread sweep: 5 and 6 run blocks of up
// to 192 threads (two copies each) at five or six CTAs per SM; 7 runs blocks
// of up to 384 threads, one copy each (the same kernel: copy c of a patch is
// thread c mod blockDim), at three CTAs per SM -- shorter visits for lists
// of few patches per SM.
__host__ __device__ constexpr int pair_maxt(int setting) { return setting == 7 ? 384 : 192; }
__host__ __device__ constexpr int pair_minb(int setting) { return setting == 7 ? 3 : setting; }

template <int SETTING, int SOLVER>
__global__ void __launch_bounds__(pair_maxt(SETTING), pair_minb(SETTING))
    k_fim_pair(DevMesh m, DevState s, StepParams sp, int cur, int check) {
  fim_pair_pass<SOLVER>(m, s, sp, cur, check, blockIdx.x);
}

// Schedule of one FIM iteration: one warp per patch of the current list.
__device__ __forceinline__ void schedule_pass(const DevMesh& m, const DevState& s, const StepParams& sp, int cur,
                                              int vb) {
  const int count = s.counts[cur];
  const int* list = cur ? s.list1 : s.list0;
  int* nlist = cur ? s.list0 : s.list1;
  const int nxt = cur ^ 1;
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int w = (vb * blockDim.x + threadIdx.x) >> 5; w < count; w += nwarps) {
    const int p = list[w] & ~kPrevisited;
    // the patch's records, loaded together (none depends on the copy-back)
    const int vs = m.vert_off[p], ve = m.vert_off[p + 1];
    const int con = s.bcon[p];
    const float bmin = s.bmin[p];
    const int a = m.padj_off[p], b = m.padj_off[p + 1];
    for (int v = vs + lane; v < ve; v += 32)
      if (!s.seed[v]) s.DT[v] = s.DT_out[v];
    if (!con) {
      if (lane == 0) {
        const int pos = atomicAdd(&s.counts[nxt], 1);
        nlist[pos] = p;
      }
    } else if (bmin < patch_par(m, sp, p).bw) {
      for (int j0 = a; j0 < b; j0 += 32) {
        const int j = j0 + lane;
        int q = -1;
        bool take = false;
        if (j < b) {
          q = m.padj[j];
          take = atomicCAS(&s.blabel[q], LS_FAR, LS_ACTIVE) == LS_FAR;
        }
        const unsigned mask = __ballot_sync(0xffffffffu, take);
        if (mask) {
          const int leader = __ffs(mask) - 1;
          int base = 0;
          if (lane == leader) base = atomicAdd(&s.counts[2], __popc(mask));
          base = __shfl_sync(0xffffffffu, base, leader);
          if (take) s.newlist[base + __popc(mask & ((1u << lane) - 1u))] = q;
        }
      }
    }
  }
}

__global__ void k_schedule(DevMesh m, DevState s, StepParams sp, int cur) {
  schedule_pass(m, s, sp, cur, blockIdx.x);
}

// ---------------------------------------------------------------------------
// Persistent FIM loop: every iteration of a step's redistance in one
// cooperative launch (all CTAs resident), the sweep, schedule and check
// passes separated by grid-wide barriers instead of kernel boundaries.  The
// passes are the launch-per-pass kernels' bodies, so a step gives the same
// bits either way (the reference's host loop this replaces:
// redistance3d.cu:85-224).
//
// Grid barrier: one counter that grows by gridDim.x per barrier (reset
// before each launch).  Thread 0 of each CTA counts the barriers it has
// reached (epoch), adds its arrival with a release reduction and polls the
// counter with acquire loads until it reaches epoch x gridDim.x, so the last
// arrival releases every CTA without a reset or a second word on the
// critical path.  Every wait is bounded: after sp.spin_limit polls (one if
// it is negative) the CTA
// raises the abort word (ctl[3]) and leaves; a CTA that finds the word
// raised, while waiting or after a barrier, leaves too, so an abort ends the
// whole launch, and the host reports LS_DEVICE_TIMEOUT.  The acq_rel fences
// on both sides make the passes' global writes (plain stores of every
// thread, ordered before thread 0 by the CTA barrier) visible to the next
// pass, which reads them with plain loads: DT, DT_out, lists, counters,
// labels.
__device__ __forceinline__ bool grid_sync(const DevState& s, const StepParams& sp, unsigned& epoch) {
  __shared__ int s_go;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile int* abort_word = s.ctl + 3;
    int go = 1;
    epoch += 1;
    const unsigned target = epoch * gridDim.x;
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(s.gbar) : "memory");
    unsigned polls = 0;
    while (true) {
      unsigned v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(s.gbar) : "memory");
      if ((int)(v - target) >= 0) break;
      if (*abort_word) {
        go = 0;
        break;
      }
      if (++polls > (sp.spin_limit < 0 ? 0u : (unsigned)sp.spin_limit)) {
        atomicExch(s.ctl + 3, 1);
        go = 0;
        break;
      }
      __nanosleep(32);
    }
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
    if (*abort_word) go = 0;
    s_go = go;
  }
  __syncthreads();
  return s_go != 0;
}

// The loop: iteration i sweeps list (i & 1) while it is not empty, at most
// sp.max_fim_iters iterations (the cap sets ctl[1]).
//
// A cooperative launch places consecutive CTAs on the same SM (CTAs 0-19 of
// a 760-CTA grid on four SMs, measured), while an ordinary launch spreads
// them over the SMs; the passes give list entry b to CTA b first, so a short
// list would run on a few SMs.  Each CTA therefore takes a spread index:
// slot on its SM x number of SMs + rank of its SM (every SM holds the same
// number of CTAs of a full cooperative grid; otherwise the index stays
// blockIdx.x).  gbar[2 + smid] counts the CTAs of each SM (reset per launch).
__device__ __forceinline__ int spread_index(const DevState& s, const StepParams& sp, unsigned& epoch, bool* ok) {
  __shared__ int s_vb;
  __shared__ unsigned s_slot, s_smid;
  if (threadIdx.x == 0) {
    unsigned smid, nsmid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    asm volatile("mov.u32 %0, %%nsmid;" : "=r"(nsmid));
    s_smid = smid;
    s_slot = smid < (unsigned)(kGridBarrierWords - 2) && nsmid <= (unsigned)(kGridBarrierWords - 2)
                 ? atomicAdd(s.gbar + 2 + smid, 1u)
                 : 0xffffffffu;
  }
  *ok = grid_sync(s, sp, epoch);
  if (!*ok) return blockIdx.x;
  if (threadIdx.x < 32) {
    // warp 0: SMs holding CTAs, this SM's rank among them, equal counts?
    unsigned nsmid;
    asm volatile("mov.u32 %0, %%nsmid;" : "=r"(nsmid));
    const unsigned smid = s_smid;
    unsigned active = 0, rank = 0, per = 0;
    bool uniform = s_slot != 0xffffffffu && nsmid <= (unsigned)(kGridBarrierWords - 2);
    for (unsigned i0 = 0; uniform && i0 < nsmid; i0 += 32) {
      const unsigned i = i0 + threadIdx.x;
      const unsigned c = i < nsmid ? *reinterpret_cast<volatile unsigned*>(s.gbar + 2 + i) : 0u;
      const unsigned has = __ballot_sync(0xffffffffu, c != 0u);
      active += __popc(has);
      if (smid >= i0) rank += __popc(smid - i0 >= 32 ? has : (has & ((1u << (smid - i0)) - 1u)));
      const unsigned cmax = __reduce_max_sync(0xffffffffu, c);
      const unsigned cmin = __reduce_min_sync(0xffffffffu, c != 0u ? c : 0xffffffffu);
      if (has) {
        if (per == 0) per = cmax;
        if (cmax != per || cmin != per) uniform = false;
      }
    }
    if (threadIdx.x == 0)
      s_vb = (uniform && active * per == gridDim.x) ? (int)(s_slot * active + rank) : (int)blockIdx.x;
  }
  __syncthreads();
  return s_vb;
}

template <class Pass>
__device__ __forceinline__ void fim_loop_persistent(const DevMesh& m, const DevState& s, const StepParams& sp,
                                                    Pass&& pass) {
  int cur = 0;
  unsigned epoch = 0;  // barriers passed (thread 0)
  bool ok = true;
  const int vb = spread_index(s, sp, epoch, &ok);
  if (!ok) return;
  for (int it = 0;; ++it) {
    const int count = *reinterpret_cast<volatile int*>(s.counts + cur);
    if (count == 0) break;
    if (it >= sp.max_fim_iters) {
      if (blockIdx.x == 0 && threadIdx.x == 0) s.ctl[1] = 1;
      break;
    }
    pass(cur, 0, vb);
    if (!grid_sync(s, sp, epoch)) return;
    schedule_pass(m, s, sp, cur, vb);
    if (!grid_sync(s, sp, epoch)) return;
    pass(cur, 1, vb);
    if (!grid_sync(s, sp, epoch)) return;
    cur ^= 1;
  }
}

template <int SETTING, int SOLVER>
__global__ void __launch_bounds__(pair_maxt(SETTING), pair_minb(SETTING))
    k_fim_pair_persist(DevMesh m, DevState s, StepParams sp) {
  fim_loop_persistent(m, s, sp,
                      [&](int cur, int check, int vb) { fim_pair_pass<SOLVER>(m, s, sp, cur, check, vb); });
}

template <int D1, int MAXT, bool XDIV, int MINB, bool PREC>
__global__ void __launch_bounds__(MAXT, MINB) k_fim_persist(DevMesh m, DevState s, StepParams sp) {
  fim_loop_persistent(m, s, sp,
                      [&](int cur, int check, int vb) { fim_copy_pass<D1, XDIV, PREC>(m, s, sp, cur, check, vb); });
}

// Narrowband (K14) fused with the sign recovery (K10b) and the vertex-update
// count: one warp per patch over every patch.
__global__ void k_narrowband(DevMesh m, DevState s, StepParams sp) {
  __shared__ unsigned long long s_cnt, s_pv, s_np;
  if (threadIdx.x == 0) { s_cnt = 0; s_pv = 0; s_np = 0; }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  unsigned cnt = 0, pv = 0, npc = 0;
  for (int p = warp_id_global(); p < m.nparts; p += nwarps) {
    const int vs = m.vert_off[p], ve = m.vert_off[p + 1];
    const PatchPar pp = patch_par(m, sp, p);
    unsigned mn = 0x7f800000u;
    for (int v = vs + lane; v < ve; v += 32) {
      const float d = s.DT[v];
      mn = min(mn, __float_as_uint(d));
      cnt += (d <= pp.bw);
      const float mag = (d >= sp.largenum || pp.scale == 1.f) ? d : d * pp.scale;
      s.phi[v] = s.sign[v] ? mag : -mag;
    }
    mn = __reduce_min_sync(0xffffffffu, mn);
    if (lane == 0 && __uint_as_float(mn) <= pp.bw) {
      const int pos = atomicAdd(&s.counts[3], 1);
      s.nblist[pos] = p;
      pv += ve - vs;
      npc += 1;
    }
  }
  atomicAdd(&s_cnt, (unsigned long long)cnt);
  if (lane == 0) { atomicAdd(&s_pv, (unsigned long long)pv); atomicAdd(&s_np, (unsigned long long)npc); }
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(&s.stats[2], s_cnt);
    atomicAdd(&s.stats[3], s_pv);
    atomicAdd(&s.stats[4], s_np);
  }
}

// ---------------------------------------------------------------------------
// Update on narrowband patches: advection (meshFIM_kernels.h:36-408,
// meshFIM2d_kernels.h:37-362) or mean curvature (meshFIM3d.cu:103-267 in the
// reference form, or the lumped-mass form).  One CTA per patch; per-copy
// contributions go to shared memory, each owned vertex sums its slots in the
// reference order.
struct Contrib {
  float aH[4], aV[4], curv[4], vol, g0, g1, g2;
};

template <int D1>
__device__ __forceinline__ void update_copy(const DevMesh& m, const StepParams& sp, long long c,
                                            long long c_first, const float* sPhi, const float* sX,
                                            int nslab, const int idx[4], Contrib& o) {
#pragma unroll
  for (int k = 0; k < 4; ++k) { o.aH[k] = 0.f; o.aV[k] = 0.f; o.curv[k] = 0.f; }
  o.vol = 0.f; o.g0 = 0.f; o.g1 = 0.f; o.g2 = 0.f;
  const bool curvature = sp.update_kind == 1;
  float e[4];
#pragma unroll
  for (int k = 0; k < D1; ++k) e[k] = sPhi[idx[k]];
  if (D1 == 4) {
    float x[4][3];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      x[k][0] = sX[idx[k]];
      x[k][1] = sX[nslab + idx[k]];
      x[k][2] = sX[2 * nslab + idx[k]];
    }
    if (!sp.ref_compat) {
      // shape-function gradients from coordinates relative to the fourth
      // vertex (translation invariant, well conditioned in FP32); the
      // reference's absolute-coordinate cofactors cancel to O(h^3)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        x[k][0] = x[k][0] - x[3][0];
        x[k][1] = x[k][1] - x[3][1];
        x[k][2] = x[k][2] - x[3][2];
      }
      x[3][0] = 0.f; x[3][1] = 0.f; x[3][2] = 0.f;
    }
    const float v31[3] = {x[1][0] - x[3][0], x[1][1] - x[3][1], x[1][2] - x[3][2]};
    const float v32[3] = {x[2][0] - x[3][0], x[2][1] - x[3][1], x[2][2] - x[3][2]};
    const float v30[3] = {x[0][0] - x[3][0], x[0][1] - x[3][1], x[0][2] - x[3][2]};
    const float cr0 = v31[1] * v32[2] - v31[2] * v32[1];
    const float cr1 = v31[2] * v32[0] - v31[0] * v32[2];
    const float cr2 = v31[0] * v32[1] - v31[1] * v32[0];
    const float volume = fabsf(cr0 * v30[0] + cr1 * v30[1] + cr2 * v30[2]) / 6.0f;
    // gradients of the linear shape functions: rows of the inverse of
    // [[x0 y0 z0 1]; ...; [x3 y3 z3 1]] by cofactors (meshFIM_kernels.h:173-215)
    const float a11 = x[0][0], a12 = x[0][1], a13 = x[0][2];
    const float a21 = x[1][0], a22 = x[1][1], a23 = x[1][2];
    const float a31 = x[2][0], a32 = x[2][1], a33 = x[2][2];
    const float a41 = x[3][0], a42 = x[3][1], a43 = x[3][2];
    float det, b11, b12, b13, b21, b22, b23, b31, b32, b33;
    if (kLbSkip && !sp.ref_compat) {
      // fast build: the fourth vertex is the origin (a41 = a42 = a43 = 0), so
      // the same sums with their zero terms left out and the others in their
      // order (equal values; only the sign of an exactly zero cofactor can
      // differ, so the bit-exact build keeps the reference's full sums)
      det = a11 * a22 * a33 + a12 * a23 * a31 + a13 * a21 * a32 - a11 * a23 * a32 - a12 * a21 * a33 -
            a13 * a22 * a31;
      b11 = a22 * a33 - a23 * a32;
      b12 = a13 * a32 - a12 * a33;
      b13 = a12 * a23 - a13 * a22;
      b21 = a23 * a31 - a21 * a33;
      b22 = a11 * a33 - a13 * a31;
      b23 = a13 * a21 - a11 * a23;
      b31 = a21 * a32 - a22 * a31;
      b32 = a12 * a31 - a11 * a32;
      b33 = a11 * a22 - a12 * a21;
    } else {
      det = a11 * a22 * a33 + a11 * a23 * a42 + a11 * a32 * a43 + a12 * a21 * a43 + a12 * a23 * a31 +
            a12 * a33 * a41 + a13 * a21 * a32 + a13 * a22 * a41 + a13 * a31 * a42 + a21 * a33 * a42 +
            a22 * a31 * a43 + a23 * a32 * a41 - a11 * a22 * a43 - a11 * a23 * a32 - a11 * a33 * a42 -
            a12 * a21 * a33 - a12 * a23 * a41 - a12 * a31 * a43 - a13 * a21 * a42 - a13 * a22 * a31 -
            a13 * a32 * a41 - a21 * a32 * a43 - a22 * a33 * a41 - a23 * a31 * a42;
      b11 = a22 * a33 + a23 * a42 + a32 * a43 - a22 * a43 - a23 * a32 - a33 * a42;
      b12 = a12 * a43 + a13 * a32 + a33 * a42 - a12 * a33 - a13 * a42 - a32 * a43;
      b13 = a12 * a23 + a13 * a42 + a22 * a43 - a12 * a43 - a13 * a22 - a23 * a42;
      b21 = a21 * a43 + a23 * a31 + a33 * a41 - a21 * a33 - a23 * a41 - a31 * a43;
      b22 = a11 * a33 + a13 * a41 + a31 * a43 - a11 * a43 - a13 * a31 - a33 * a41;
      b23 = a11 * a43 + a13 * a21 + a23 * a41 - a11 * a23 - a13 * a41 - a21 * a43;
      b31 = a21 * a32 + a22 * a41 + a31 * a42 - a21 * a42 - a22 * a31 - a32 * a41;
      b32 = a11 * a42 + a12 * a31 + a32 * a41 - a11 * a32 - a12 * a41 - a31 * a42;
      b33 = a11 * a22 + a12 * a41 + a21 * a42 - a11 * a42 - a12 * a21 - a22 * a41;
    }
    const float b14 = a12 * a33 + a13 * a22 + a23 * a32 - a12 * a23 - a13 * a32 - a22 * a33;
    const float b24 = a11 * a23 + a13 * a31 + a21 * a33 - a11 * a33 - a13 * a21 - a23 * a31;
    const float b34 = a11 * a32 + a12 * a21 + a22 * a31 - a11 * a22 - a12 * a31 - a21 * a32;
    float nN[4][3] = {{b11 / det, b21 / det, b31 / det},
                      {b12 / det, b22 / det, b32 / det},
                      {b13 / det, b23 / det, b33 / det},
                      {b14 / det, b24 / det, b34 / det}};
    float gp0 = 0.f, gp1 = 0.f, gp2 = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      gp0 += nN[i][0] * e[i];
      gp1 += nN[i][1] * e[i];
      gp2 += nN[i][2] * e[i];
    }
    const float absg = sqrtf(gp0 * gp0 + gp1 * gp1 + gp2 * gp2);
    float sg0, sg1, sg2;
    if (curvature) {
      sg0 = 1.f; sg1 = 0.f; sg2 = 1.f;
    } else {
      const long long cs = sp.ref_compat ? c_first : c;
      sg0 = __ldg(m.sig + cs); sg1 = __ldg(m.sig + m.full + cs); sg2 = __ldg(m.sig + 2 * m.full + cs);
    }
    float K[4], Kp[4], Km[4], H = 0.f, beta = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      K[i] = volume * (sg0 * nN[i][0] + sg1 * nN[i][1] + sg2 * nN[i][2]);
      H += K[i] * e[i];
      Kp[i] = fmaxf(K[i], 0.f);
      Km[i] = fminf(K[i], 0.f);
      beta += Km[i];
    }
    beta = 1.0f / beta;
    const bool hpass = (double)fabsf(H) > (curvature ? 1e-16 : 1e-8);
    float at[4] = {0.f, 0.f, 0.f, 0.f};
    if (hpass) {
      float alpha[4], theta = 0.f;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float d = Kp[i] * beta *
                        (Km[0] * (e[i] - e[0]) + Km[1] * (e[i] - e[1]) + Km[2] * (e[i] - e[2]) + Km[3] * (e[i] - e[3]));
        alpha[i] = d / H;
        theta += fmaxf(0.f, alpha[i]);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) at[i] = fmaxf(alpha[i], 0.f) / theta;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) { o.aH[i] = at[i] * H; o.aV[i] = at[i] * volume; }
    if (curvature) {
      const bool gate = sp.ref_compat ? hpass : (absg > 0.f);
      if (gate) {
        o.vol = volume;
        o.g0 = volume * gp0; o.g1 = volume * gp1; o.g2 = volume * gp2;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          float acc = 0.f;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int jj = (i + j) & 3;
            acc += (nN[i][0] * nN[jj][0] + nN[i][1] * nN[jj][1] + nN[i][2] * nN[jj][2]) / absg * e[jj];
          }
          o.curv[i] = volume * acc;
        }
      }
    }
  } else {
    const float lc0 = __ldg(m.lc + c), lc1 = __ldg(m.lc + m.full + c), lc2 = __ldg(m.lc + 2 * m.full + c);
    const float z = lc0 * lc2;  // (AB x AC).z in the local frame
    const float volume = sqrtf(z * z) / 2.0f;
    const float det = lc0 * lc2;
    const float nN[3][2] = {{-lc2 / det, (lc1 - lc0) / det}, {lc2 / det, -lc1 / det}, {0.f / det, lc0 / det}};
    float gp0 = 0.f, gp1 = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i) { gp0 += nN[i][0] * e[i]; gp1 += nN[i][1] * e[i]; }
    const float absg = sqrtf(gp0 * gp0 + gp1 * gp1);
    if (!curvature) {
      float sg0, sg1;
      if (sp.ref_compat) {  // meshFIM2d_kernels.h:178-181
        sg0 = e[0] / absg;
        sg1 = e[1] / absg;
      } else {
        sg0 = __ldg(m.sig + c);
        sg1 = __ldg(m.sig + m.full + c);
      }
      float K[3], Kp[3], Km[3], H = 0.f, beta = 0.f;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        K[i] = volume * (sg0 * nN[i][0] + sg1 * nN[i][1]);
        H += K[i] * e[i];
        Kp[i] = fmaxf(K[i], 0.f);
        Km[i] = fminf(K[i], 0.f);
        beta += Km[i];
      }
      beta = 1.0f / beta;
      // the weights stay 0 for an element the gate drops, and the products
      // below are formed in every case, as in the reference
      // (meshFIM2d_kernels.h:198-236): a non-finite H then reaches the sums
      float at[3] = {0.f, 0.f, 0.f};
      if ((double)fabsf(H) > 1e-8) {
        float alpha[3], theta = 0.f;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const float d = Kp[i] * beta * (Km[0] * (e[i] - e[0]) + Km[1] * (e[i] - e[1]) + Km[2] * (e[i] - e[2]));
          alpha[i] = d / H;
          theta += fmaxf(0.f, alpha[i]);
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) at[i] = fmaxf(alpha[i], 0.f) / theta;
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        o.aH[i] = at[i] * H;
        o.aV[i] = at[i] * volume;
      }
    } else if (absg > 0.f) {
      o.vol = volume;
      o.g0 = volume * gp0; o.g1 = volume * gp1;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        float acc = 0.f;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const int jj = (i + j) % 3;
          acc += (nN[i][0] * nN[jj][0] + nN[i][1] * nN[jj][1]) / absg * e[jj];
        }
        o.curv[i] = volume * acc;
      }
    }
  }
}

template <int D1>
__device__ __forceinline__ void update_patches(const DevMesh& m, const DevState& s, const StepParams& sp) {
  extern __shared__ float smem[];
  const int slab = sp.lvp + sp.lgp;
  float* sPhi = smem;                // slab
  float* sX = smem + slab;           // 3 * slab (3D only)
  float* sC = sX + (D1 == 4 ? 3 * slab : 0);  // per copy: aH[4] aV[4] curv[4] vol g0 g1 g2
  const bool curvature = sp.update_kind == 1;
  const int stride = 15;
  const int count = s.counts[3];
  for (int li = blockIdx.x; li < count; li += gridDim.x) {
    const int p = s.nblist[li];
    const PatchPar pp = patch_par(m, sp, p);
    const int vs = m.vert_off[p], nvp = m.vert_off[p + 1] - vs;
    const int gs = m.ghost_off[p], ngp = m.ghost_off[p + 1] - gs;
    const int es = m.ele_off[p], nep = m.ele_off[p + 1] - es;
    const int nslab = nvp + ngp;
    for (int i = threadIdx.x; i < nslab; i += blockDim.x) {
      const int v = i < nvp ? vs + i : __ldg(m.ghost_ids + gs + i - nvp);
      sPhi[i] = s.phi[v];
      if (D1 == 4) {
        sX[i] = __ldg(m.xyz + v);
        sX[nslab + i] = __ldg(m.xyz + m.nv + v);
        sX[2 * nslab + i] = __ldg(m.xyz + 2 * (long long)m.nv + v);
      }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < nep; c += blockDim.x) {
      const ushort4 cv = m.conn[es + c];
      const int idx[4] = {cv.x, cv.y, cv.z, D1 == 4 ? cv.w : 0};
      Contrib o;
      update_copy<D1>(m, sp, (long long)es + c, es, sPhi, sX, nslab, idx, o);
      float* dst = sC + (size_t)c * stride;
#pragma unroll
      for (int k = 0; k < 4; ++k) { dst[k] = o.aH[k]; dst[4 + k] = o.aV[k]; dst[8 + k] = o.curv[k]; }
      dst[12] = o.vol; dst[13] = o.g0; dst[14] = o.g1;
      // g2 packed separately below the copies
      sC[(size_t)nep * stride + c] = o.g2;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nvp; i += blockDim.x) {
      const int v = vs + i;
      const int a = m.vslot_off[v];
      // with the reference's slot limit (m.capped set) the advection sums
      // run over the first slot_cap slots only, as the reference's update
      const int b = (m.capped && !curvature) ? min(m.vslot_off[v + 1], a + m.slot_cap) : m.vslot_off[v + 1];
      const float oldT = sPhi[i];
      float res = oldT;
      if (!curvature) {
        float up = 0.f, down = 0.f;
        for (int q = a; q < b; ++q) {
          const int sl = m.vslot[q];
          up += sC[(sl >> 2) * stride + (sl & 3)];
        }
        for (int q = a; q < b; ++q) {
          const int sl = m.vslot[q];
          down += sC[(sl >> 2) * stride + 4 + (sl & 3)];
        }
        if ((double)fabsf(down) > 1e-8) res = oldT - pp.dt * (up / down);
      } else {
        float down = 0.f, gd = 0.f, g0 = 0.f, g1 = 0.f, g2 = 0.f, cu = 0.f;
        for (int q = a; q < b; ++q) {
          const int sl = m.vslot[q];
          const float* src = sC + (sl >> 2) * stride;
          down += src[4 + (sl & 3)];
          g0 += src[13];
          g1 += src[14];
          g2 += sC[(size_t)nep * stride + (sl >> 2)];
          gd += src[12];
          cu += src[8 + (sl & 3)];
        }
        const float node_eik = sqrtf(g0 * g0 + g1 * g1 + g2 * g2) / gd;
        if (sp.ref_compat && D1 == 4) {
          if ((double)fabsf(down) > 1e-16) res = oldT - pp.cc * node_eik * (cu / gd) * pp.dt;
        } else if (gd > 0.f) {
          // the reference's normalisation (curv_up / sum of element volumes)
          res = oldT - pp.cc * node_eik * (cu / gd) * pp.dt;
        }
      }
      s.phi_out[v] = res;
    }
    __syncthreads();
  }
}

template <int D1>
__global__ void __launch_bounds__(512) k_update(DevMesh m, DevState s, StepParams sp) {
  update_patches<D1>(m, s, sp);
}

// tetrahedra with patches of up to 384 element copies: three CTAs per SM
// (which caps the registers at 56 without spills; the 512-thread form keeps
// two)
__global__ void __launch_bounds__(384, 3) k_update_384(DevMesh m, DevState s, StepParams sp) {
  update_patches<4>(m, s, sp);
}

// phi := phi_out on narrowband patches (CopyOutBack_levelset3d)
__global__ void k_copy_phi(DevMesh m, DevState s) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int count = s.counts[3];
  for (int w = warp_id_global(); w < count; w += nwarps) {
    const int p = s.nblist[w];
    for (int v = m.vert_off[p] + lane; v < m.vert_off[p + 1]; v += 32) s.phi[v] = s.phi_out[v];
  }
}

// out[old] = phi[new] (kernel_compute_vertT_before_permute3d), as a gather
__global__ void k_unpermute(DevMesh m, const float* phi, float* out) {
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < m.nv; o += gridDim.x * blockDim.x)
    out[o] = phi[__ldg(m.ipermute + o)];
}

// out[new] = in[old]
__global__ void k_permute(DevMesh m, const float* in, float* out) {
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < m.nv; o += gridDim.x * blockDim.x)
    out[__ldg(m.ipermute + o)] = in[o];
}

// ---------------------------------------------------------------------------
// Launchers (host side).
// ---------------------------------------------------------------------------
// Learned warm start.

// Raw local-solve candidates of one copy (no minimum with the vertex's own
// value): the support of each of its vertices.
template <int D1, bool XDIV>
__device__ __forceinline__ void solve_copy_raw(const float* Mt, const float T[4], float out[4], float eps_h,
                                               double eps_h64, float LN) {
  if (D1 == 4) {
    const float ACAC = Mt[0], ACBC = Mt[1], ACCD = Mt[2], BCBC = Mt[3], BCCD = Mt[4];
    const float CDCD = Mt[5], ADAD = Mt[6], ADBD = Mt[7], ADCD = Mt[8], BDBD = Mt[9], CDBD = Mt[10];
    const float TA = T[0], TB = T[1], TC = T[2], TD = T[3];
    bool ill = false;
    out[3] = tet_solve<float, XDIV, false>(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD, eps_h, eps_h64, LN, 0.f, ill);
    out[0] = tet_solve<float, XDIV, false>(TB, TD, TC, BCBC, -BCCD, -ACBC, CDCD, ACCD, ACAC, eps_h, eps_h64, LN, 0.f, ill);
    out[1] = tet_solve<float, XDIV, false>(TA, TD, TC, ACAC, -ACCD, -ACBC, CDCD, BCCD, BCBC, eps_h, eps_h64, LN, 0.f, ill);
    out[2] = tet_solve<float, XDIV, false>(TA, TB, TD, ADAD, ADBD, -ADCD, BDBD, -CDBD, CDCD, eps_h, eps_h64, LN, 0.f, ill);
  } else {
    const float LenAB = Mt[0], LenBC = Mt[1], LenCA = Mt[2];
    const float TA = T[0], TB = T[1], TC = T[2];
    out[2] = tri_solve<float>(TA, TB, LenAB, LenBC, LenCA, LN);
    out[0] = tri_solve<float>(TB, TC, LenBC, LenCA, LenAB, LN);
    out[1] = tri_solve<float>(TC, TA, LenCA, LenAB, LenBC, LN);
    out[3] = LN;
  }
}

// Owned vertices of the patches nblist[0, nb) -> lr.vlist (warp per patch).
__global__ void k_nb_vertices(DevMesh m, DevState s, DevLearn lr, int nb) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int w = warp_id_global(); w < nb; w += nwarps) {
    const int p = s.nblist[w];
    const int vs = m.vert_off[p], nvp = m.vert_off[p + 1] - vs;
    int base = 0;
    if (lane == 0) base = atomicAdd(&lr.cnt[0], nvp);
    base = __shfl_sync(0xffffffffu, base, 0);
    for (int i = lane; i < nvp; i += 32) lr.vlist[base + i] = vs + i;
  }
}

// DT := |prediction| + margin on the warm set (FIM frame, unit h); the seed
// search that follows overwrites the seeds.
__global__ void k_warm_apply(DevState s, DevLearn lr, float LN, float margin) {
  const int n = lr.cnt[0];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int v = lr.vlist[i];
    const float w = fminf(fabsf(lr.pred[i]) + margin, LN);
    s.DT[v] = w;
    lr.warm[v] = w;
  }
}

// Support check after the FIM from a warm start: an owned non-seed vertex
// whose value lies more than tol below every local solve of its elements
// (its support) was set by the warm start, not by the wavefront; it is
// reset to LARGENUM and its patch joins list0 for another FIM loop.  One
// CTA per patch over all patches; patches without a reached vertex skip.
template <int D1, bool XDIV>
__global__ void __launch_bounds__(384) k_support(DevMesh m, DevState s, StepParams sp, DevLearn lr, float tol,
                                                 int whole_patch) {
  extern __shared__ float smem[];
  float* sT = smem;
  float* sC = smem + sp.lvp + sp.lgp;  // owned candidates
  const int tid = threadIdx.x;
  for (int p = blockIdx.x; p < m.nparts; p += gridDim.x) {
    const int vs = m.vert_off[p], nvp = m.vert_off[p + 1] - vs;
    const int gs = m.ghost_off[p], ngp = m.ghost_off[p + 1] - gs;
    const int es = m.ele_off[p], nep = m.ele_off[p + 1] - es;
    int reached = 0;
    for (int i = tid; i < nvp + ngp; i += blockDim.x) {
      const float d = s.DT[i < nvp ? vs + i : __ldg(m.ghost_ids + gs + i - nvp)];
      sT[i] = d;
      if (i < nvp) {
        sC[i] = __int_as_float(0x7f800000);
        reached |= (d < sp.largenum) ? 1 : 0;
      }
    }
    reached = __syncthreads_or(reached);
    if (!reached) continue;
    for (int c = tid; c < nep; c += blockDim.x) {
      const ushort4 cv = m.conn[es + c];
      const int idx[4] = {cv.x, cv.y, cv.z, cv.w};
      float T[4] = {0.f, 0.f, 0.f, sp.largenum}, Mt[11], r[4];
#pragma unroll
      for (int k = 0; k < D1; ++k) T[k] = sT[idx[k]];
      copy_metric<D1>(m, (long long)es + c, Mt);
      solve_copy_raw<D1, XDIV>(Mt, T, r, sp.eps_h, sp.eps_h64, sp.largenum);
#pragma unroll
      for (int k = 0; k < D1; ++k)
        if (idx[k] < nvp) atomicMin(reinterpret_cast<int*>(&sC[idx[k]]), __float_as_int(fmaxf(r[k], 0.f)));
    }
    __syncthreads();
    int bad = 0;
    for (int i = tid; i < nvp; i += blockDim.x) {
      const int v = vs + i;
      if (!s.seed[v] && sT[i] < sp.largenum && sT[i] < sC[i] - tol) {
        s.DT[v] = sp.largenum;
        bad++;
      }
    }
    bad = __syncthreads_count(bad);
    if (bad && whole_patch) {
      // reset every non-seed vertex of the patch: values that leaned on the
      // unsupported ones are recomputed in the same FIM loop
      for (int i = tid; i < nvp; i += blockDim.x)
        if (!s.seed[vs + i]) s.DT[vs + i] = sp.largenum;
    }
    if (tid == 0 && bad) {
      atomicAdd(&lr.cnt[1], bad);
      if (atomicCAS(&s.blabel[p], LS_FAR, LS_ACTIVE) == LS_FAR) {
        const int pos = atomicAdd(&s.counts[0], 1);
        s.list0[pos] = p;
        atomicAdd(&lr.cnt[3], 1);
      }
    }
    __syncthreads();
  }
}

// Warm-set vertices whose final value differs from the warm start by more
// than tol (FIM frame).
__global__ void k_moved(DevState s, DevLearn lr, float tol) {
  const int n = lr.cnt[0];
  int moved = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int v = lr.vlist[i];
    moved += (fabsf(s.DT[v] - lr.warm[v]) > tol) ? 1 : 0;
  }
  moved = __reduce_add_sync(0xffffffffu, moved);
  if ((threadIdx.x & 31) == 0 && moved) atomicAdd(&lr.cnt[2], moved);
}

// Collection: signed phi after the redistance, in units of h, per warm-set
// vertex (NaN where the wavefront did not reach).
__global__ void k_targets(DevState s, DevLearn lr, float inv_h, float LN) {
  const int n = lr.cnt[0];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int v = lr.vlist[i];
    const float ph = s.phi[v];
    lr.target[i] = fabsf(ph) >= LN ? __int_as_float(0x7fc00000) : ph * (lr.vinv_h ? lr.vinv_h[v] : inv_h);
  }
}

cudaError_t launch_learn(int op, const DevMesh& m, const DevState& s, const StepParams& sp, const DevLearn& lr,
                         int arg, float fa, const Launch& L, cudaStream_t st) {
  switch (op) {
    case LEARN_NB_VERTICES:
      k_nb_vertices<<<L.warp_grid, 256, 0, st>>>(m, s, lr, arg);
      break;
    case LEARN_WARM:
      k_warm_apply<<<L.flat_grid, 256, 0, st>>>(s, lr, sp.largenum, fa);
      break;
    case LEARN_SEED_WARM:
      if (m.dim == 3) k_seed<4><<<L.seed_grid, L.fim_block, 0, st>>>(m, s, 0, sp.scale, 1);
      else k_seed<3><<<L.seed_grid, L.fim_block, 0, st>>>(m, s, 0, sp.scale, 1);
      break;
    case LEARN_SUPPORT: {
      const int smem = (int)sizeof(float) * (2 * sp.lvp + sp.lgp);
      const int grid = L.sms * 4;
      if (m.dim == 3) {
        if (sp.xdiv) k_support<4, true><<<grid, 384, smem, st>>>(m, s, sp, lr, fa, arg);
        else k_support<4, false><<<grid, 384, smem, st>>>(m, s, sp, lr, fa, arg);
      } else {
        k_support<3, false><<<grid, 384, smem, st>>>(m, s, sp, lr, fa, arg);
      }
      break;
    }
    case LEARN_MOVED:
      k_moved<<<L.flat_grid, 256, 0, st>>>(s, lr, fa);
      break;
    case LEARN_TARGETS:
      k_targets<<<L.flat_grid, 256, 0, st>>>(s, lr, fa, sp.largenum);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_reset(const DevMesh& m, const DevState& s, const StepParams& sp, const Launch& L, cudaStream_t st) {
  k_reset<<<L.flat_grid, 256, 0, st>>>(s, m.nv, sp.largenum);
  return cudaGetLastError();
}

cudaError_t launch_seed(const DevMesh& m, const DevState& s, int use_all, float scale, const Launch& L, cudaStream_t st) {
  if (m.dim == 3) k_seed<4><<<L.seed_grid, L.fim_block, 0, st>>>(m, s, use_all, scale, 0);
  else k_seed<3><<<L.seed_grid, L.fim_block, 0, st>>>(m, s, use_all, scale, 0);
  return cudaGetLastError();
}

// Block size classes: patches of up to 384 element copies run 2, 3 or 4
// CTAs per SM (registers capped at 85 / 56 / 42; StepParams::ctas), larger
// ones one CTA of 512 or 1024 threads.
// dynamic shared memory of k_fim_compact<MAXT>: slab values and owned
// snapshot (rounded up to 16 bytes), then 23 floats, one ushort4 and 8 ints
// (listed solves, FP64 repeats) per thread
inline int compact_smem(const StepParams& sp, int maxt) {
  return (int)sizeof(float) * (((2 * sp.lvp + sp.lgp + 3) & ~3) + 23 * maxt) + 8 * maxt + 32 * maxt;
}

// dynamic shared memory of k_fim_pair for `ncap` copies: slab values, then
// per copy 4 float4 records + metric (48 B) + connectivity (8 B) + listed
// solves (8 B)
inline int pair_smem(const StepParams& sp, int ncap) {
  return (int)sizeof(float) * ((2 * sp.lvp + sp.lgp + 3) & ~3) + ncap * (16 * 3 + 48 + 8 + 8);
}

// The two-copies-per-thread kernels of this build: the planar-wave solver
// (fast build) or the reference's solver (bit-exact build; its interior
// division in double with the reference's semantics).
// Setting 5: five CTAs per SM (64 registers); setting 6: six (56 registers).
#ifdef LS_KERNELS_EXACT
#define LS_PAIR_SOLVERS(K, n, sp) ((sp).xdiv ? (const void*)K<n, kPairRefXdiv> : (const void*)K<n, kPairRef>)
#else
#define LS_PAIR_SOLVERS(K, n, sp) ((const void*)K<n, kPairWave>)
#endif
#define LS_PAIR_PICK(K, sp)                                            \
  ((sp).ctas == 7   ? LS_PAIR_SOLVERS(K, 7, sp)                      \
   : (sp).ctas == 6 ? LS_PAIR_SOLVERS(K, 6, sp)                      \
                    : LS_PAIR_SOLVERS(K, 5, sp))
#define LS_PAIR_KERNEL(sp) LS_PAIR_PICK(k_fim_pair, sp)
#define LS_PAIR_PERSIST(sp) LS_PAIR_PICK(k_fim_pair_persist, sp)

// Tetrahedra without capped corners, no precision form, patches of up to
// 384 copies, FIM setting 5: the two-copies-per-thread sweep (L.pair_block).
__host__ __device__ inline bool use_pair(const DevMesh& m, const StepParams& sp, const Launch& L) {
  return m.dim == 3 && !m.capped && !(sp.tau > 0.f) && L.pair_block > 0;
}

cudaError_t launch_pair(const DevMesh& m, const DevState& s, const StepParams& sp, int cur, int c, const Launch& L,
                        cudaStream_t st) {
  void* args[] = {(void*)&m, (void*)&s, (void*)&sp, (void*)&cur, (void*)&c};
  return cudaLaunchKernel(LS_PAIR_KERNEL(sp), dim3((unsigned)L.fim_grid), dim3((unsigned)L.pair_block), args,
                          (size_t)pair_smem(sp, sp.lep), st);
}

cudaError_t launch_sweep(const DevMesh& m, const DevState& s, const StepParams& sp, int cur, bool check,
                         const Launch& L, cudaStream_t st) {
  const bool xd = sp.xdiv != 0;
  const bool pr = sp.tau > 0.f;
  const int c = check ? 1 : 0;
  // precision-form kernels: one 384-class register budget (2 CTAs/SM) and
  // the deferred-solve queue in shared memory
  const int psmem = L.fim_smem + (int)sizeof(DeferredSolve) * kDeferCap;
#define LS_FIM(D, T, X, B, P) \
  k_fim<D, T, X, B, P><<<L.fim_grid, L.fim_block, P ? psmem : L.fim_smem, st>>>(m, s, sp, cur, c)
#define LS_FIM3(T, B) \
  do { \
    if (xd) { if (pr) LS_FIM(4, T, true, (T == 384 ? 2 : 1), true); else LS_FIM(4, T, true, B, false); } \
    else { if (pr) LS_FIM(4, T, false, (T == 384 ? 2 : 1), true); else LS_FIM(4, T, false, B, false); } \
  } while (0)
  // meshes with corners beyond the reference's slot limit (reference
  // semantics only) take the one-copy-per-thread kernel, which keeps those
  // corners private
  const bool compact = kLbSkip && m.dim == 3 && !m.capped;
  if (use_pair(m, sp, L)) {
    // tetrahedra: compacted solves, two copies per thread
    return launch_pair(m, s, sp, cur, c, L, st);
  } else if (compact && pr) {
    // fast build, tetrahedra, precision form: compacted solves, FP64 repeats
    // run densely after each sweep's FP32 pass
    const int cs = compact_smem(sp, L.fim_block <= 384 ? 384 : L.fim_block <= 512 ? 512 : 1024);
    if (L.fim_block <= 384) k_fim_compact<384, 2, true><<<L.fim_grid, L.fim_block, cs, st>>>(m, s, sp, cur, c);
    else if (L.fim_block <= 512) k_fim_compact<512, 1, true><<<L.fim_grid, L.fim_block, cs, st>>>(m, s, sp, cur, c);
    else k_fim_compact<1024, 1, true><<<L.fim_grid, L.fim_block, cs, st>>>(m, s, sp, cur, c);
  } else if (compact) {
    // fast build, tetrahedra: compacted solves
    const int cs = compact_smem(sp, L.fim_block <= 384 ? 384 : L.fim_block <= 512 ? 512 : 1024);
    if (L.fim_block <= 384) {
      if (sp.ctas == 2) k_fim_compact<384, 2, false><<<L.fim_grid, L.fim_block, cs, st>>>(m, s, sp, cur, c);
      else if (sp.ctas == 4) k_fim_compact<384, 4, false><<<L.fim_grid, L.fim_block, cs, st>>>(m, s, sp, cur, c);
      else k_fim_compact<384, 3, false><<<L.fim_grid, L.fim_block, cs, st>>>(m, s, sp, cur, c);
    } else if (L.fim_block <= 512) {
      k_fim_compact<512, 1, false><<<L.fim_grid, L.fim_block, cs, st>>>(m, s, sp, cur, c);
    } else {
      k_fim_compact<1024, 1, false><<<L.fim_grid, L.fim_block, cs, st>>>(m, s, sp, cur, c);
    }
  } else if (m.dim == 3) {
    if (L.fim_block <= 384) {
      if (sp.ctas == 2) LS_FIM3(384, 2);
      else if (sp.ctas == 4) LS_FIM3(384, 4);
      else LS_FIM3(384, 3);
    } else if (L.fim_block <= 512) {
      LS_FIM3(512, 1);
    } else {
      LS_FIM3(1024, 1);
    }
  } else {
    if (L.fim_block <= 384) LS_FIM(3, 384, false, 3, false);
    else if (L.fim_block <= 512) LS_FIM(3, 512, false, 1, false);
    else LS_FIM(3, 1024, false, 1, false);
  }
#undef LS_FIM3
#undef LS_FIM
  return cudaGetLastError();
}

// The persistent form of the sweep kernel launch_sweep would pick, where it
// has one: the two-copies-per-thread kernel, or the one-copy kernel with
// 384-thread blocks (bit-exact build, triangles, meshes with capped slots).
// Cooperative launch: the runtime refuses a grid that cannot be resident.
cudaError_t launch_fim_persistent(const DevMesh& m, const DevState& s, const StepParams& sp, const Launch& L,
                                  cudaStream_t st) {
  if (L.persist_grid <= 0) return cudaErrorNotSupported;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.gridDim = dim3((unsigned)L.persist_grid);
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const bool xd = sp.xdiv != 0;
  const bool pr = sp.tau > 0.f;
  const bool compact = kLbSkip && m.dim == 3 && !m.capped;
  if (use_pair(m, sp, L)) {
    cfg.blockDim = dim3((unsigned)L.pair_block);
    cfg.dynamicSmemBytes = (size_t)pair_smem(sp, sp.lep);
    void* args[] = {(void*)&m, (void*)&s, (void*)&sp};
    return cudaLaunchKernelExC(&cfg, LS_PAIR_PERSIST(sp), args);
  }
  if (compact || L.fim_block > 384) return cudaErrorNotSupported;
  cfg.blockDim = dim3((unsigned)L.fim_block);
  const int psmem = L.fim_smem + (int)sizeof(DeferredSolve) * kDeferCap;
  cfg.dynamicSmemBytes = (size_t)(pr ? psmem : L.fim_smem);
  if (m.dim == 3) {
    if (pr) {
      if (xd) return cudaLaunchKernelEx(&cfg, k_fim_persist<4, 384, true, 2, true>, m, s, sp);
      return cudaLaunchKernelEx(&cfg, k_fim_persist<4, 384, false, 2, true>, m, s, sp);
    }
    if (xd) return cudaLaunchKernelEx(&cfg, k_fim_persist<4, 384, true, 2, false>, m, s, sp);
    return cudaLaunchKernelEx(&cfg, k_fim_persist<4, 384, false, 2, false>, m, s, sp);
  }
  return cudaLaunchKernelEx(&cfg, k_fim_persist<3, 384, false, 2, false>, m, s, sp);
}

// Resident CTAs of the persistent kernel launch_fim_persistent picks (0
// where there is no persistent form).
cudaError_t configure_persistent(const DevMesh& m, const StepParams& sp, Launch& L) {
  L.persist_grid = 0;
  const bool xd = sp.xdiv != 0;
  const bool pr = sp.tau > 0.f;
  const bool compact = kLbSkip && m.dim == 3 && !m.capped;
  int occ = 0;
  cudaError_t e = cudaSuccess;
  auto query = [&](const void* fn, int block, int smem) {
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, block, smem);
  };
  if (use_pair(m, sp, L)) {
    query(LS_PAIR_PERSIST(sp), L.pair_block, pair_smem(sp, sp.lep));
  } else if (!compact && L.fim_block <= 384) {
    const int psmem = L.fim_smem + (int)sizeof(DeferredSolve) * kDeferCap;
    const int sm = pr ? psmem : L.fim_smem;
    const void* fn = m.dim == 3 ? (pr ? (xd ? (const void*)k_fim_persist<4, 384, true, 2, true>
                                           : (const void*)k_fim_persist<4, 384, false, 2, true>)
                                      : (xd ? (const void*)k_fim_persist<4, 384, true, 2, false>
                                            : (const void*)k_fim_persist<4, 384, false, 2, false>))
                                : (const void*)k_fim_persist<3, 384, false, 2, false>;
    query(fn, L.fim_block, sm);
  } else {
    return cudaSuccess;
  }
  if (e != cudaSuccess) return e;
  L.persist_grid = occ > 0 ? L.sms * occ : 0;
  return cudaSuccess;
}

cudaError_t launch_schedule(const DevMesh& m, const DevState& s, const StepParams& sp, int cur, const Launch& L,
                            cudaStream_t st) {
  k_schedule<<<L.warp_grid, 256, 0, st>>>(m, s, sp, cur);
  return cudaGetLastError();
}

cudaError_t launch_narrowband(const DevMesh& m, const DevState& s, const StepParams& sp, const Launch& L,
                              cudaStream_t st) {
  k_narrowband<<<L.warp_grid, 256, 0, st>>>(m, s, sp);
  return cudaGetLastError();
}

cudaError_t launch_update(const DevMesh& m, const DevState& s, const StepParams& sp, const Launch& L,
                          cudaStream_t st) {
  if (m.dim == 3 && L.upd_block <= 384) k_update_384<<<L.upd_grid, L.upd_block, L.upd_smem, st>>>(m, s, sp);
  else if (m.dim == 3) k_update<4><<<L.upd_grid, L.upd_block, L.upd_smem, st>>>(m, s, sp);
  else k_update<3><<<L.upd_grid, L.upd_block, L.upd_smem, st>>>(m, s, sp);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_copy_phi<<<L.warp_grid, 256, 0, st>>>(m, s);
  return cudaGetLastError();
}

cudaError_t launch_unpermute(const DevMesh& m, const float* phi, float* out, const Launch& L, cudaStream_t st) {
  k_unpermute<<<L.flat_grid, 256, 0, st>>>(m, phi, out);
  return cudaGetLastError();
}

cudaError_t launch_permute(const DevMesh& m, const float* in, float* out, const Launch& L, cudaStream_t st) {
  k_permute<<<L.flat_grid, 256, 0, st>>>(m, in, out);
  return cudaGetLastError();
}

// Geometry records of the two-copies-per-thread sweep (L.pair_block > 0).
cudaError_t launch_geometry(const DevMesh& m, float4* gm, float4* gh, const Launch& L, cudaStream_t st) {
  if (L.pair_block <= 0 || m.full == 0) return cudaSuccess;
  k_geometry<<<L.flat_grid, 256, 0, st>>>(m, gm, gh);
  return cudaGetLastError();
}

cudaError_t configure_launch(const DevMesh& m, const StepParams& sp, Launch& L) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, dev);
  if (e != cudaSuccess) return e;
  L.sms = prop.multiProcessorCount;
  L.fim_block = ((sp.lep + 31) / 32) * 32;
  if (L.fim_block < 64) L.fim_block = 64;
  L.fim_smem = (int)sizeof(float) * (2 * sp.lvp + sp.lgp);
  int occ = 0;
  L.pair_block = 0;
  if (kLbSkip && m.dim == 3 && !m.capped) {
    // compacted kernel (fast build): opt in to its shared memory, size the
    // grid by its occupancy
    const int maxt = L.fim_block <= 384 ? 384 : L.fim_block <= 512 ? 512 : 1024;
    const int cs = compact_smem(sp, maxt);
    if (L.fim_block <= 384 && sp.ctas >= 5 && sp.ctas <= 7) {
      // two copies per thread: ceil(lep / 2) threads, whole warps (setting
      // 7: one copy per thread, lep threads)
      L.pair_block = sp.ctas == 7 ? L.fim_block : ((sp.lep + 1) / 2 + 31) / 32 * 32;
      const int ps = pair_smem(sp, sp.lep);
      e = cudaFuncSetAttribute(LS_PAIR_KERNEL(sp), cudaFuncAttributeMaxDynamicSharedMemorySize, ps);
      if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, LS_PAIR_KERNEL(sp), L.pair_block, ps);
    } else if (L.fim_block <= 384 && sp.ctas == 2) {
      e = cudaFuncSetAttribute(k_fim_compact<384, 2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
      if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fim_compact<384, 2, false>, L.fim_block, cs);
    } else if (L.fim_block <= 384 && sp.ctas == 4) {
      e = cudaFuncSetAttribute(k_fim_compact<384, 4, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
      if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fim_compact<384, 4, false>, L.fim_block, cs);
    } else if (L.fim_block <= 384) {
      e = cudaFuncSetAttribute(k_fim_compact<384, 3, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
      if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fim_compact<384, 3, false>, L.fim_block, cs);
    } else if (L.fim_block <= 512) {
      e = cudaFuncSetAttribute(k_fim_compact<512, 1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
      if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fim_compact<512, 1, false>, L.fim_block, cs);
    } else {
      e = cudaFuncSetAttribute(k_fim_compact<1024, 1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
      if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fim_compact<1024, 1, false>, L.fim_block, cs);
    }
    // precision-form variants (selected at launch when tau > 0)
    if (e == cudaSuccess) {
      if (L.fim_block <= 384)
        e = cudaFuncSetAttribute(k_fim_compact<384, 2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
      else if (L.fim_block <= 512)
        e = cudaFuncSetAttribute(k_fim_compact<512, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
      else
        e = cudaFuncSetAttribute(k_fim_compact<1024, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
    }
  } else if (m.dim == 3) {
    if (!m.capped && L.fim_block <= 384 && sp.ctas >= 5 && sp.ctas <= 7) {
      // bit-exact build: two copies per thread with the reference's solver
      // (the precision form keeps the one-copy kernel)
      L.pair_block = sp.ctas == 7 ? L.fim_block : ((sp.lep + 1) / 2 + 31) / 32 * 32;
      const int ps = pair_smem(sp, sp.lep);
      e = cudaFuncSetAttribute(LS_PAIR_KERNEL(sp), cudaFuncAttributeMaxDynamicSharedMemorySize, ps);
      if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, LS_PAIR_KERNEL(sp), L.pair_block, ps);
    } else if (L.fim_block <= 384 && sp.ctas == 2)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fim<4, 384, false, 2, false>, L.fim_block, L.fim_smem);
    else if (L.fim_block <= 384 && sp.ctas == 4)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fim<4, 384, false, 4, false>, L.fim_block, L.fim_smem);
    else if (L.fim_block <= 384)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fim<4, 384, false, 3, false>, L.fim_block, L.fim_smem);
    else if (L.fim_block <= 512)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fim<4, 512, false, 1, false>, L.fim_block, L.fim_smem);
    else
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fim<4, 1024, false, 1, false>, L.fim_block, L.fim_smem);
  } else {
    if (L.fim_block <= 384)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fim<3, 384, false, 3, false>, L.fim_block, L.fim_smem);
    else if (L.fim_block <= 512)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fim<3, 512, false, 1, false>, L.fim_block, L.fim_smem);
    else
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fim<3, 1024, false, 1, false>, L.fim_block, L.fim_smem);
  }
  if (e != cudaSuccess) return e;
  if (occ < 1) occ = 1;
  L.fim_grid = L.sms * occ;
  L.seed_grid = L.sms * 8;
  L.upd_block = L.fim_block > 512 ? 512 : L.fim_block;
  const int slab = sp.lvp + sp.lgp;
  L.upd_smem = (int)sizeof(float) * (slab * (m.dim == 3 ? 4 : 1) + sp.lep * 16);
  {
    const void* fn = m.dim == 3 ? (L.upd_block <= 384 ? (const void*)k_update_384 : (const void*)k_update<4>)
                                : (const void*)k_update<3>;
    if (L.upd_smem > 48 * 1024) {
      e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, L.upd_smem);
      if (e != cudaSuccess) return e;
    }
    occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, L.upd_block, L.upd_smem);
  }
  if (e != cudaSuccess) return e;
  if (occ < 1) occ = 1;
  L.upd_grid = L.sms * occ;
  L.warp_grid = L.sms * 8;
  L.flat_grid = L.sms * 8;
  return configure_persistent(m, sp, L);
}


const KernelSet& kernel_table() {
  static const KernelSet t = {configure_launch,  launch_reset,  launch_seed,      launch_sweep,
                              launch_schedule,   launch_fim_persistent, launch_narrowband, launch_update,
                              launch_unpermute,  launch_permute, launch_learn,     launch_geometry};
  return t;
}
