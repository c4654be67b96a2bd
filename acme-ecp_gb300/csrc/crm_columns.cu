// One instantiation of the column kernel, selected at compile time:
//   -DCRM_INST_T=double -DCRM_INST_SHAPE=s   FP64 plain form, compiled with
//       -fmad=false so every multiply and add is separately rounded, the same
//       contract as the CPU restatement of crm(): the two produce identical bits;
//   -DCRM_INST_T=float  -DCRM_INST_SHAPE=s   FP32-mixed form: fields and bulk
//       arithmetic in FP32; the pressure tridiagonal solve, every domain-mean /
//       column sum and the saturation-adjustment Newton iteration in FP64.
// The build compiles this file once per (precision, launch shape), in parallel.
#include "crm_kernel.cuh"

#if !defined(CRM_INST_T) || !defined(CRM_INST_SHAPE)
#error "define CRM_INST_T and CRM_INST_SHAPE"
#endif

namespace crm {
template void launch_crm_columns<CRM_INST_T, CRM_INST_SHAPE>(const KParams &, int, cudaStream_t);
template int occupancy_crm_columns<CRM_INST_T, CRM_INST_SHAPE>(int, int);
}  // namespace crm
