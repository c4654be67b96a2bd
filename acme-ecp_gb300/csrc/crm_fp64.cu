// FP64 plain form of the column kernel.  Compiled with -fmad=false so every
// multiply and add is separately rounded, the same contract as the CPU
// restatement of crm(): the two produce identical bits.
#include "crm_kernel.cuh"

namespace crm {
template void launch_crm_columns<double>(const KParams &, int, int, cudaStream_t);
template int occupancy_crm_columns<double>(int, int, int);
}
