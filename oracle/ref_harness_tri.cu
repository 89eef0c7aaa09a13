/*
 * Exposes the reference's FP64 local solvers of the 2D stack
 * (src/core2d/include/redistance_kernels.h:124-285 localSolverTet1 and
 * :287-334 localSolverTri) as host functions, compiled from the reference
 * header itself.  Built into oracle/_ref/ by oracle/build_ref.py.
 */
#include <redistance.h>
#include <cuda_fp16.h>
#undef __device__
#define __device__ __location__(host) __location__(device)
#include <redistance_kernels.h>

extern "C" double lsref_tri_solve_f64(double TA, double TB, double LenAB, double LenBC,
                                      double LenAC) {
  return localSolverTri(TA, TB, LenAB, LenBC, LenAC);
}
extern "C" double lsref_tet_solve_f64(double TA, double TB, double TC, double ACAC,
                                      double ACBC, double ACCD, double BCBC, double BCCD,
                                      double CDCD) {
  return localSolverTet1(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD);
}
