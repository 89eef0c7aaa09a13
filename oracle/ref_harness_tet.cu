/*
 * Exposes the reference's FP32 tet local solver
 * (src/core3d/include/redistance_kernels3d.h:124-285, localSolverTet1Levelset)
 * as a host function, compiled from the reference header itself.  Built into
 * oracle/_ref/ by oracle/build_ref.py; used only to pin the oracle.
 */
#include <redistance3d.h>
#include <cuda_fp16.h>
#undef __device__
#define __device__ __location__(host) __location__(device)
#include <redistance_kernels3d.h>

extern "C" float lsref_tet_solve_f32(float TA, float TB, float TC, float ACAC, float ACBC,
                                     float ACCD, float BCBC, float BCCD, float CDCD) {
  return localSolverTet1Levelset(TA, TB, TC, ACAC, ACBC, ACCD, BCBC, BCCD, CDCD);
}
extern "C" double lsref_smallnum(void) { return (double)SMALLNUM; }
extern "C" double lsref_largenum(void) { return (double)LARGENUM; }
