// crm_tc_probe.cu -- crm_debug_tc_transform: the tensor-core transforms of
// the 3D pressure solve (crm_tc.cuh) on their own, one CTA over host data,
// so that they can be checked against the discrete Fourier transform.
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/crm_gb300.h"
#include "crm_tc.cuh"

namespace {

constexpr int kProbeThreads = 512;

__global__ void __launch_bounds__(kProbeThreads, 1)
    crm_tc_probe_kernel(float *ff, int n, int nlev, int dir, const float *mats, int *status) {
  __shared__ unsigned long long mbar;
  __shared__ unsigned tmem, phase;
  __shared__ int fail;
  extern __shared__ __align__(16) unsigned char dsm[];
  float *sm = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(dsm) + 127) & ~(uintptr_t)127);
  using namespace crm::tc;
  if (threadIdx.x < 32) {
    tmem_alloc(smem_u32(&tmem), kTmemCols);
    fence_before();
  }
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&mbar));
    phase = 0;
    fail = 0;
  }
  Engine(n, sm, 0u, 0u, nullptr, nullptr, threadIdx.x, blockDim.x).load_mats(mats);
  __syncthreads();
  fence_after();
  Engine E(n, sm, tmem, smem_u32(&mbar), &phase, &fail, threadIdx.x, blockDim.x);
  const int n2 = n + 2;
  auto FF = [&](int i, int j, int k) -> float & { return ff[((size_t)(k - 1) * n2 + (j - 1)) * n2 + (i - 1)]; };
  for (int k0 = 1; k0 <= nlev; k0 += E.d.L) {
    if (dir < 0) E.forward_tile(FF, k0, nlev);
    else E.inverse_tile(FF, k0, nlev);
  }
  if (threadIdx.x == 0 && fail) mbar_wait(smem_u32(&mbar), phase ^ 1u, kWaitLimit);
  __syncthreads();
  if (threadIdx.x < 32) {
    fence_after();
    tmem_free(tmem, kTmemCols);
  }
  if (threadIdx.x == 0) *status = fail ? CRM_ERR_TIMEOUT : CRM_OK;
}

// the transform matrices (crm_host.cu)
}  // namespace

namespace crm_tc_host {
void dft_matrices(float *out, int n);
size_t dft_elems(int n);
}  // namespace crm_tc_host

extern "C" int crm_debug_tc_transform(int n, int nlev, int dir, const float *in, float *out) {
  if ((n != 16 && n != 32) || nlev < 1 || nlev > 4096 || (dir != -1 && dir != 1) || !in || !out)
    return CRM_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return CRM_ERR_NO_DEVICE;
  const size_t nf = (size_t)nlev * (n + 2) * (n + 2), nm = crm_tc_host::dft_elems(n);
  std::vector<float> m(nm);
  crm_tc_host::dft_matrices(m.data(), n);
  float *d_ff = nullptr, *d_m = nullptr;
  int *d_st = nullptr, st = CRM_ERR_CUDA;
  const size_t smem = crm::tc::smem_bytes(n);
  bool ok = cudaMalloc(&d_ff, sizeof(float) * nf) == cudaSuccess && cudaMalloc(&d_m, sizeof(float) * nm) == cudaSuccess &&
            cudaMalloc(&d_st, sizeof(int)) == cudaSuccess &&
            cudaMemcpy(d_ff, in, sizeof(float) * nf, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(d_m, m.data(), sizeof(float) * nm, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaFuncSetAttribute(crm_tc_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ==
                cudaSuccess;
  if (ok) {
    crm_tc_probe_kernel<<<1, kProbeThreads, smem>>>(d_ff, n, nlev, dir, d_m, d_st);
    ok = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess &&
         cudaMemcpy(out, d_ff, sizeof(float) * nf, cudaMemcpyDeviceToHost) == cudaSuccess &&
         cudaMemcpy(&st, d_st, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
  }
  cudaFree(d_ff);
  cudaFree(d_m);
  cudaFree(d_st);
  return ok ? st : CRM_ERR_CUDA;
}
