// One instantiation of the column kernel, selected at compile time:
//   -DCRM_INST_T=double -DCRM_INST_SHAPE=s   FP64 plain form, compiled with
//       -fmad=false so every multiply and add is separately rounded, the same
//       contract as the CPU restatement of crm(): the two produce identical bits;
//   -DCRM_INST_T=float  -DCRM_INST_SHAPE=s   FP32-mixed form: fields and bulk
//       arithmetic in FP32; the pressure tridiagonal solve, the conservation
//       sums and the saturation-adjustment Newton iteration in FP64;
// -DCRM_INST_NX=n: the compile-time horizontal size (0: generic);
// -DCRM_INST_NY=m: 1 (default) the 2D CRM, 0 the generic 3D CRM;
// -DCRM_INST_VAR=v: 0 the plain forms, 1 the 3D FP32-mixed form with the
// tensor-core transforms, 2 the FP64 form with multiply-add contraction
// (compiled without -fmad=false).
// The build compiles this file once per (precision, nx, launch shape), in
// parallel.
#include "crm_kernel.cuh"

#if !defined(CRM_INST_T) || !defined(CRM_INST_SHAPE) || !defined(CRM_INST_NX)
#error "define CRM_INST_T, CRM_INST_NX and CRM_INST_SHAPE"
#endif

#ifndef CRM_INST_NY
#define CRM_INST_NY 1
#endif
#ifndef CRM_INST_VAR
#define CRM_INST_VAR 0
#endif

namespace crm {
template void launch_crm_columns<CRM_INST_T, CRM_INST_NX, CRM_INST_NY, CRM_INST_SHAPE, CRM_INST_VAR>(const KParams &, int,
                                                                                                  cudaStream_t, bool);
template int occupancy_crm_columns<CRM_INST_T, CRM_INST_NX, CRM_INST_NY, CRM_INST_SHAPE, CRM_INST_VAR>(int, int, int, int);
}  // namespace crm
