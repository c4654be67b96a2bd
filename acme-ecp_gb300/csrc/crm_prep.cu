// crm_prep.cu -- per-column set-up that precedes the column kernel:
// the roughness length z0 (crm_module.F90:583-594, crmsurface.F90:104-133)
// and the setperturb random draws (setperturb.F90:33-80 with the
// Mersenne-Twister variant of cam/RNG_MT.F90:52-142, seed gcol*1000).
// One thread per column.  Compiled with -fmad=false: z0 uses the
// deterministic exp/log/atan, so it matches a CPU evaluation bit for bit.
#include <cstring>
#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/crm_detmath.h"

namespace crm {

using namespace crm_detmath;
#define R4P(x) ((double)(x##f))

struct PrepParams {
  int ncrms, ld, plev, nx, igstep;
  const double *zmid, *zint, *pdel, *tau00, *bflxls, *wndls;
  const int *gcol;
  const int *col_map;   // optional (ncrms) slots
  double *z0;     // (ld), by slot
  double *rnd;    // (ld, 5, nx) by slot: 1 - 2 r
};

__global__ void crm_prep_kernel(const __grid_constant__ PrepParams p) {
  int pos = blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= p.ncrms) return;
  const int c = p.col_map ? p.col_map[pos] : pos;   // slot
  if (c < 0 || c >= p.ld) return;                   // reported by the column kernel
  auto IN = [&](const double *a, int l) { return a[(size_t)c + (size_t)p.ld * (l - 1)]; };
  const int plev = p.plev;
  // grid values of the lowest level (crm_module.F90:341-370)
  double z1 = IN(p.zmid, plev) - IN(p.zint, plev + 1);
  double z2 = IN(p.zmid, plev - 1) - IN(p.zint, plev + 1);
  double dz = 0.5 * (z1 + z2);
  double zi1 = IN(p.zint, plev + 1) - IN(p.zint, plev + 1);
  double zi2 = IN(p.zint, plev) - IN(p.zint, plev + 1);
  double adz1 = (zi2 - zi1) / dz;
  double rho1 = IN(p.pdel, plev) / 9.80616 / (adz1 * dz);
  double ustar = sqrt(p.tau00[c] / rho1);
  {
    const double vonk = R4P(0.4), am = R4P(4.8), bm = R4P(19.3), eps = R4P(1.e-10);
    const double c1 = (double)(3.14159f / 2.f - 3.f * 0.693147182f);
    double bflx = p.bflxls[c], wnd = p.wndls[c];
    double rlmo = -bflx * vonk / (ustar * ustar * ustar + eps);
    double zeta = z1 * rlmo;
    zeta = (zeta < 1.) ? zeta : 1.;
    double psi1;
    if (zeta >= 0.) psi1 = -am * zeta;
    else {
      double x = sqrt(sqrt(1.0 - bm * zeta));
      psi1 = 2. * det_log(1.0 + x) + det_log(1.0 + x * x) - 2. * det_atan(x) + c1;
    }
    double lnz = vonk * wnd / (ustar + eps) + psi1;
    lnz = (lnz > 0.) ? lnz : 0.;
    double z0 = z1 * det_exp(-lnz);
    z0 = (z0 < 1.) ? z0 : 1.;
    p.z0[c] = (z0 > R4P(0.00001)) ? z0 : R4P(0.00001);
  }
  if (p.igstep > 1) return;
  // RNG_MT_set_seed / RNG_MT_gen_rand
  int32_t mt[624];
  mt[0] = (int32_t)(p.gcol[pos] * 1000);
  for (int i = 1; i < 624; ++i) mt[i] = (int32_t)((uint32_t)69069 * (uint32_t)mt[i - 1]);
  int mti = 624;
  const int32_t UMASK = -1147483648, LMASK = 2147483647, MATA = -1727483681;
  const int32_t TMASKB = -1658038656, TMASKC = -272236544;
  double *r = p.rnd + (size_t)c * 5 * p.nx;
  for (int e = 0; e < 5 * p.nx; ++e) {
    int32_t y;
    if (mti >= 624) {
      int kk;
      for (kk = 0; kk < 624 - 397; ++kk) {
        y = (mt[kk] & UMASK) | (mt[kk + 1] & LMASK);
        mt[kk] = mt[kk + 397] ^ (int32_t)((uint32_t)y >> 1) ^ ((y & 1) ? MATA : 0);
      }
      for (; kk < 623; ++kk) {
        y = (mt[kk] & UMASK) | (mt[kk + 1] & LMASK);
        mt[kk] = mt[kk + (397 - 624)] ^ (int32_t)((uint32_t)y >> 1) ^ ((y & 1) ? MATA : 0);
      }
      y = (mt[623] & UMASK) | (mt[0] & LMASK);
      mt[623] = mt[396] ^ (int32_t)((uint32_t)y >> 1) ^ ((y & 1) ? MATA : 0);
      mti = 0;
    }
    y = mt[mti++];
    y ^= (int32_t)((uint32_t)y >> 11);
    y ^= (int32_t)(((uint32_t)y << 7) & (uint32_t)TMASKB);
    y ^= (int32_t)(((uint32_t)y << 15) & (uint32_t)TMASKC);
    y ^= (int32_t)((uint32_t)y >> 18);
    double g = (y < 0) ? ((double)y + 4294967296.0) / 4294967296.0 : ((double)y + 0.5) / 4294967296.0;
    r[e] = 1. - 2. * g;
  }
}

void launch_crm_prep(const PrepParams &p, cudaStream_t s) {
  int block = 128, grid = (p.ncrms + block - 1) / block;
  crm_prep_kernel<<<grid, block, 0, s>>>(p);
}

// Host bytes carried to the device as kernel parameters: a launch recorded
// into a CUDA graph keeps its parameters by value, where a copy from host
// memory would keep only the host address.
struct ConstChunk {
  unsigned long long w[480];
  int nwords;
};

__global__ void crm_consts_kernel(unsigned long long *dst, const __grid_constant__ ConstChunk c) {
  for (int i = threadIdx.x; i < c.nwords; i += blockDim.x) dst[i] = c.w[i];
}

int launch_crm_consts(void *dst, const void *src, size_t bytes, cudaStream_t s) {
  ConstChunk c;
  int launches = 0;
  const unsigned char *from = static_cast<const unsigned char *>(src);
  unsigned char *to = static_cast<unsigned char *>(dst);
  for (size_t off = 0; off < bytes; off += sizeof c.w) {
    const size_t n = bytes - off < sizeof c.w ? bytes - off : sizeof c.w;
    memset(c.w, 0, sizeof c.w);
    memcpy(c.w, from + off, n);
    c.nwords = (int)((n + 7) / 8);
    crm_consts_kernel<<<1, 128, 0, s>>>(reinterpret_cast<unsigned long long *>(to + off), c);
    ++launches;
  }
  return launches;
}

}  // namespace crm
