// FP32-mixed form of the column kernel: fields and bulk arithmetic in FP32;
// the pressure tridiagonal solve, every domain-mean / column sum and the
// saturation-adjustment Newton iteration stay in FP64 (see crm_kernel.cuh).
#include "crm_kernel.cuh"

namespace crm {
template void launch_crm_columns<float>(const KParams &, int, int, cudaStream_t);
template int occupancy_crm_columns<float>(int, int, int);
}
