// crm_host.cu -- the C ABI of include/crm_gb300.h: the drop-in for the
// reference's subroutine crm() (crm/crm_module.F90:45-1718).
//
// Host work per call, as in the reference (whose grid setup and setperturb
// also run on the host, crm_module.F90:320-375,677-681): the per-call
// constants (FFT factors and REAL*4 trig tables, fft.F90:156-300; Laplacian
// eigenvalues, pressure.F90:172-198; gamma functions, gammafff.c; fall-speed
// coefficients, microphysics.F90:500-507), the roughness length z0
// (crmsurface.F90:104-133) and the random draws of setperturb
// (setperturb.F90:33-80, cam/RNG_MT.F90:52-142).  Everything else runs in
// one launch of the persistent column kernel.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/crm_gb300.h"
#include "../../include/crm_detmath.h"
#include "crm_kernel.h"

using namespace crm_detmath;

#define R4H(x) ((double)(x##f))

struct crm_ctx {
  crm_config cfg;
  crm::Layout L;
  int device = 0, nsm = 0, block = 256, grid_max = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // device buffers
  void *slabs = nullptr;
  size_t slab_bytes = 0;
  double *d_in = nullptr;        // crm_input arrays, packed
  size_t in_elems = 0;
  double *d_state = nullptr;     // 7 state fields
  double *d_rad = nullptr;       // qrad + 5 outputs
  double *d_out = nullptr;       // all outputs
  double *d_consts = nullptr;    // trigs, eign
  double *d_colconst = nullptr;  // z0 (ncrms), rnd (ncrms * 5 * nx)
  int *d_status = nullptr;
  int ld_cap = 0;
  // host-side constants
  std::vector<double> trigs, eign;
  int ifax[20];
  double gam[10];
  double vrain, vsnow, vgrau, crain, csnow, cgrau, a_bg, a_pr, a_gr;
  int last_launches = 0;
  double last_kernel_ms = 0.;
};

namespace {

const double kPi4 = R4H(3.141592653589793);

// fax_crm (fft.F90:181-246), mode 3
void fft_factors(int *ifax, int n) {
  int nn = n / 2, k = 0;
  if (nn + nn != n) { ifax[0] = -99; return; }
  while (nn % 4 == 0) { ifax[++k] = 4; nn /= 4; if (nn == 1) goto done; }
  if (nn % 2 == 0) { ifax[++k] = 2; nn /= 2; if (nn == 1) goto done; }
  while (nn % 3 == 0) { ifax[++k] = 3; nn /= 3; if (nn == 1) goto done; }
  {
    int l = 5, inc = 2;
    for (;;) {
      while (nn % l == 0) { ifax[++k] = l; nn /= l; if (nn == 1) goto done; }
      l += inc; inc = 6 - inc;
    }
  }
done:
  ifax[0] = k;
  for (int ii = 2; ii <= k; ++ii)
    for (int i = 1; i <= k + 1 - ii; ++i)
      if (ifax[i + 1] < ifax[i]) { int t = ifax[i]; ifax[i] = ifax[i + 1]; ifax[i + 1] = t; }
}

// fftrig_crm (fft.F90:247-300), mode 3: REAL*4 pi, del, angle, cos, sin
void fft_trigs(std::vector<double> &trigs, int n) {
  trigs.assign(3 * n / 2 + 2 + n, 0.0);
  float pi_f = (float)(2.0f * asinf(1.0f));
  int nn = n / 2;
  float del = (float)((double)(pi_f + pi_f) / (double)nn);
  for (int i = 1; i <= nn + nn; i += 2) {
    float angle = (float)(0.5 * (double)(i - 1) * (double)del);
    trigs[i - 1] = (double)cosf(angle);
    trigs[i] = (double)sinf(angle);
  }
  del = 0.5f * del;
  int nh = (nn + 1) / 2, l = nh + nh, la = nn + nn;
  for (int i = 1; i <= l; i += 2) {
    float angle = (float)(0.5 * (double)(i - 1) * (double)del);
    trigs[la + i - 1] = (double)cosf(angle);
    trigs[la + i] = (double)sinf(angle);
  }
}

float gammafff(float x) { return (float)exp(lgamma((double)x)); }

// MT19937 variant of cam/RNG_MT.F90:52-142 (its UMASK is 0xBB9ACA00)
struct RngMT {
  int32_t mt[624];
  int mti;
  explicit RngMT(int32_t seed) {
    mt[0] = seed;
    for (mti = 1; mti < 624; ++mti) mt[mti] = (int32_t)((uint32_t)69069 * (uint32_t)mt[mti - 1]);
  }
  double next() {
    const int32_t UMASK = -1147483648, LMASK = 2147483647, MATA = -1727483681;
    const int32_t TMASKB = -1658038656, TMASKC = -272236544;
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
    if (y < 0) return ((double)y + 4294967296.0) / 4294967296.0;
    return ((double)y + 0.5) / 4294967296.0;
  }
};

double dmax2(double a, double b) { return (b > a) ? b : a; }
double dmin2(double a, double b) { return (b < a) ? b : a; }

// z0_est (crmsurface.F90:104-133) with the roughness-length clamp of
// crm_module.F90:590
double z0_of(double z, double bflx, double wnd, double ustar) {
  const double vonk = R4H(0.4), am = R4H(4.8), bm = R4H(19.3), eps = R4H(1.e-10);
  double c1 = (double)(3.14159f / 2.f - 3.f * logf(2.f));
  double rlmo = -bflx * vonk / (ustar * ustar * ustar + eps);
  double zeta = dmin2(1., z * rlmo);
  double psi1;
  if (zeta >= 0.) psi1 = -am * zeta;
  else {
    double x = sqrt(sqrt(1.0 - bm * zeta));
    psi1 = 2. * det_log(1.0 + x) + det_log(1.0 + x * x) - 2. * atan(x) + c1;
  }
  double lnz = dmax2(0., vonk * wnd / (ustar + eps) + psi1);
  double z0 = z * det_exp(-lnz);
  return dmax2(R4H(0.00001), dmin2(1., z0));
}

enum InField { I_ZMID, I_ZINT, I_TL, I_QL, I_QCCL, I_QIIL, I_PMID, I_PINT, I_PDEL, I_UL, I_VL, I_NIN };

size_t out_elems(const crm_config &c, int f, int ld) {
  if (f < CRM_OUT_FIRST_3D) return (size_t)ld * c.crm_nx * c.crm_ny * c.crm_nz;
  if (f < CRM_OUT_FIRST_1D) return (size_t)ld * c.crm_nx * c.crm_ny;
  if (f < CRM_OUT_FIRST_2D) return (size_t)ld;
  return (size_t)ld * c.plev;
}

#define CK(x)                                     \
  do {                                            \
    cudaError_t e_ = (x);                         \
    if (e_ != cudaSuccess) return CRM_ERR_CUDA;   \
  } while (0)

int validate(const crm_config *c) {
  if (!c) return CRM_ERR_ARG;
  if (c->crm_ny != 1) return CRM_ERR_UNSUPPORTED;          // 3D not built
  if (c->microphysics != CRM_MICRO_SAM1MOM) return CRM_ERR_UNSUPPORTED;
  if (c->batch_mode != CRM_PER_COLUMN) return CRM_ERR_UNSUPPORTED;
  if (c->precision != CRM_FP64 && c->precision != CRM_FP32_MIXED) return CRM_ERR_ARG;
  if (c->crm_nx < 8 || c->crm_nx % 2 || c->crm_nz < 4 || c->plev < c->crm_nz + 2) return CRM_ERR_ARG;
  if (c->crm_nx_rad < 1 || c->crm_nx % c->crm_nx_rad || c->crm_ny_rad != 1) return CRM_ERR_ARG;
  if (!(c->crm_dx > 0) || !(c->crm_dt > 0) || 60. < 2 * c->crm_dt) return CRM_ERR_ARG;
  if (c->max_ncrms < 1) return CRM_ERR_ARG;
  int f[20];
  fft_factors(f, c->crm_nx);
  if (f[0] < 1) return CRM_ERR_ARG;
  for (int k = 1; k <= f[0]; ++k)
    if (f[k] != 2 && f[k] != 4) return CRM_ERR_UNSUPPORTED;  // device FFT: radix 2, 4
  if (f[0] > 7) return CRM_ERR_ARG;
  return CRM_OK;
}

int alloc_ctx(crm_ctx *c) {
  const crm_config &g = c->cfg;
  CK(cudaGetDevice(&c->device));
  CK(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->device));
  c->L = crm::make_layout(g.crm_nx, g.crm_nz, g.plev, g.crm_nx_rad);
  const size_t esz = g.precision == CRM_FP64 ? sizeof(double) : sizeof(float);
  int per_sm = g.precision == CRM_FP64 ? crm::occupancy_crm_columns<double>(c->block)
                                       : crm::occupancy_crm_columns<float>(c->block);
  if (per_sm < 1) per_sm = 1;
  c->grid_max = c->nsm * per_sm;
  if (c->grid_max > g.max_ncrms) c->grid_max = g.max_ncrms;
  c->slab_bytes = c->L.slab * esz;
  CK(cudaMalloc(&c->slabs, c->slab_bytes * (size_t)c->grid_max));
  c->ld_cap = g.max_ncrms;
  const int ld = c->ld_cap, plev = g.plev, nx = g.crm_nx, nz = g.crm_nz;
  c->in_elems = (size_t)ld * (plev + 1);
  CK(cudaMalloc(&c->d_in, sizeof(double) * c->in_elems * I_NIN + sizeof(double) * 4 * ld));
  CK(cudaMalloc(&c->d_state, sizeof(double) * (size_t)ld * nx * nz * 7));
  CK(cudaMalloc(&c->d_rad, sizeof(double) * (size_t)ld * g.crm_nx_rad * nz * 6));
  size_t no = 0;
  for (int f = 0; f < CRM_NOUT; ++f) no += out_elems(g, f, ld);
  CK(cudaMalloc(&c->d_out, sizeof(double) * no));
  fft_factors(c->ifax, nx);
  fft_trigs(c->trigs, nx);
  // eigenvalues (pressure.F90:172-198), 2D: jd = 0
  c->eign.assign(nx + 1, 0.0);
  {
    double dx = g.crm_dx, dy = g.crm_dx;
    double ddx2 = 1.0 / (dx * dx), ddy2 = 1.0 / (dy * dy);
    double pii = 3.14159265358979323846;
    double xnx = pii / nx, xny = pii / 1;
    int jd = (int)(((float)1 - 0.1f) / 2.f);
    double xj = jd, facty = 2.0;
    for (int i = 1; i <= nx + 1; ++i) {
      int id = (int)(((float)i - 0.1f) / 2.f);
      double xi = id, factx = 2.0;
      c->eign[i - 1] = (2.0 * cos(factx * xnx * xi) - 2.0) * ddx2 + (2.0 * cos(facty * xny * xj) - 2.0) * ddy2;
    }
  }
  CK(cudaMalloc(&c->d_consts, sizeof(double) * (c->trigs.size() + c->eign.size())));
  CK(cudaMemcpy(c->d_consts, c->trigs.data(), sizeof(double) * c->trigs.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_consts + c->trigs.size(), c->eign.data(), sizeof(double) * c->eign.size(), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&c->d_colconst, sizeof(double) * (size_t)ld * (1 + 5 * nx)));
  CK(cudaMalloc(&c->d_status, sizeof(int) * (size_t)ld));
  // gamma functions and fall speeds (precip_init.F90:25-49, microphysics.F90:500-507)
  const double b_rain = R4H(0.8), b_snow = 0.25, b_grau = 0.5;
  c->gam[0] = gammafff(3.f);
  c->gam[1] = gammafff((float)(3. + b_rain));
  c->gam[2] = gammafff((float)((5. + b_rain) / 2.));
  c->gam[3] = gammafff((float)(4. + b_rain));
  c->gam[4] = gammafff((float)(3. + b_snow));
  c->gam[5] = gammafff((float)((5. + b_snow) / 2.));
  c->gam[6] = gammafff((float)(4. + b_snow));
  c->gam[7] = gammafff((float)(3. + b_grau));
  c->gam[8] = gammafff((float)((5. + b_grau) / 2.));
  c->gam[9] = gammafff((float)(4. + b_grau));
  c->crain = b_rain / 4.; c->csnow = b_snow / 4.; c->cgrau = b_grau / 4.;
  c->vrain = 842. * c->gam[3] / 6. / det_pow(kPi4 * 1000. * 8.e6, c->crain);
  c->vsnow = R4H(4.84) * c->gam[6] / 6. / det_pow(kPi4 * 100. * 3.e6, c->csnow);
  c->vgrau = 94.5 * c->gam[9] / 6. / det_pow(kPi4 * 400. * 4.e6, c->cgrau);
  c->a_bg = 1. / (R4H(273.16) - R4H(253.16));
  c->a_pr = 1. / (R4H(283.16) - R4H(268.16));
  c->a_gr = 1. / (R4H(283.16) - R4H(223.16));
  CK(cudaEventCreate(&c->ev0));
  CK(cudaEventCreate(&c->ev1));
  return CRM_OK;
}

void free_ctx(crm_ctx *c) {
  if (!c) return;
  cudaFree(c->slabs); cudaFree(c->d_in); cudaFree(c->d_state); cudaFree(c->d_rad);
  cudaFree(c->d_out); cudaFree(c->d_consts); cudaFree(c->d_colconst); cudaFree(c->d_status);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
}

}  // namespace

extern "C" {

crm_ctx *crm_create(const crm_config *cfg, int *status) {
  int rc = validate(cfg);
  int ndev = 0;
  if (rc == CRM_OK && (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)) rc = CRM_ERR_NO_DEVICE;
  if (rc != CRM_OK) {
    if (status) *status = rc;
    return nullptr;
  }
  crm_ctx *c = new (std::nothrow) crm_ctx();
  if (!c) { if (status) *status = CRM_ERR_ARG; return nullptr; }
  c->cfg = *cfg;
  rc = alloc_ctx(c);
  if (rc != CRM_OK) {
    free_ctx(c);
    delete c;
    if (status) *status = rc;
    return nullptr;
  }
  if (status) *status = CRM_OK;
  return c;
}

void crm_destroy(crm_ctx *ctx) {
  if (!ctx) return;
  free_ctx(ctx);
  delete ctx;
}

int crm_set_stream(crm_ctx *ctx, void *stream) {
  if (!ctx) return CRM_ERR_ARG;
  ctx->stream = (cudaStream_t)stream;
  return CRM_OK;
}

int crm_last_launch_count(const crm_ctx *ctx) { return ctx ? ctx->last_launches : 0; }
double crm_last_kernel_ms(const crm_ctx *ctx) { return ctx ? ctx->last_kernel_ms : 0.; }

const char *crm_status_string(int s) {
  switch (s) {
    case CRM_OK: return "ok";
    case CRM_ERR_ARG: return "invalid argument or configuration";
    case CRM_ERR_CFL: return "CFL limit: more than 16 subcycles needed (kurant)";
    case CRM_ERR_NONFINITE: return "non-finite state";
    case CRM_ERR_CUDA: return "CUDA runtime error";
    case CRM_ERR_UNSUPPORTED: return "configuration not built";
    case CRM_ERR_TIMEOUT: return "bounded device wait timed out";
    case CRM_ERR_BUDGET: return "HBM admission budget exhausted";
    case CRM_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

const char *crm_version(void) { return "crm-gb300 0.1 (sm_103a; 2D sam1mom; fp64 plain + fp32 mixed)"; }

int crm_run(crm_ctx *c, const crm_call_desc *d, const crm_input_c *in, crm_state_c *st, crm_rad_c *rad,
            crm_output_c *out, int *col_status) {
  if (!c || !d || !in || !st || !rad || !out) return CRM_ERR_ARG;
  const crm_config &g = c->cfg;
  const int ncrms = d->ncrms, ld = d->ld, plev = g.plev, nx = g.crm_nx, nz = g.crm_nz;
  if (ncrms < 1 || ld < ncrms || ld > c->ld_cap || !(d->dt_gl > 0)) return CRM_ERR_ARG;
  if (!d->gcol && d->igstep <= 1) return CRM_ERR_ARG;
  int nstop = (int)(d->dt_gl / g.crm_dt);
  if (nstop < 1) return CRM_ERR_ARG;
  double dt = d->dt_gl / nstop;
  if (60. < 2 * dt) return CRM_ERR_ARG;
  cudaStream_t s = c->stream;
  // inputs: GCM profiles (ld, plev[+1])
  const double *src[I_NIN] = {in->zmid, in->zint, in->tl, in->ql, in->qccl, in->qiil, in->pmid, in->pint, in->pdel, in->ul, in->vl};
  for (int f = 0; f < I_NIN; ++f) {
    if (!src[f]) return CRM_ERR_ARG;
    size_t n = (size_t)ld * ((f == I_ZINT || f == I_PINT) ? plev + 1 : plev);
    CK(cudaMemcpyAsync(c->d_in + (size_t)f * c->in_elems, src[f], sizeof(double) * n, cudaMemcpyHostToDevice, s));
  }
  // state and qrad
  double *sp[7] = {st->u_wind, st->v_wind, st->w_wind, st->temperature, st->qt, st->qp, st->qn};
  const size_t n4 = (size_t)ld * nx * nz;
  for (int f = 0; f < 7; ++f) {
    if (!sp[f]) return CRM_ERR_ARG;
    CK(cudaMemcpyAsync(c->d_state + f * n4, sp[f], sizeof(double) * n4, cudaMemcpyHostToDevice, s));
  }
  const size_t nr = (size_t)ld * g.crm_nx_rad * nz;
  if (!rad->qrad) return CRM_ERR_ARG;
  CK(cudaMemcpyAsync(c->d_rad, rad->qrad, sizeof(double) * nr, cudaMemcpyHostToDevice, s));
  // per-column host constants: z0 and the setperturb draws
  std::vector<double> colc((size_t)ncrms * (1 + 5 * nx));
  for (int i = 0; i < ncrms; ++i) {
    auto IN = [&](const double *a, int l) { return a[(size_t)i + (size_t)ld * (l - 1)]; };
    double z1 = IN(in->zmid, plev) - IN(in->zint, plev + 1);
    double z2 = IN(in->zmid, plev - 1) - IN(in->zint, plev + 1);
    double dz = 0.5 * (z1 + z2);
    double zi1 = IN(in->zint, plev + 1) - IN(in->zint, plev + 1);
    double zi2 = IN(in->zint, plev) - IN(in->zint, plev + 1);
    double adz1 = (zi2 - zi1) / dz;
    double rho1 = IN(in->pdel, plev) / 9.80616 / (adz1 * dz);
    double ustar = sqrt(in->tau00[i] / rho1);
    colc[i] = z0_of(z1, in->bflxls[i], in->wndls[i], ustar);
    if (d->igstep <= 1) {
      RngMT rng((int32_t)(d->gcol[i] * 1000));
      double *r = &colc[(size_t)ncrms + (size_t)i * 5 * nx];
      for (int k = 0; k < 5; ++k)
        for (int ii = 0; ii < nx; ++ii) r[(size_t)k * nx + ii] = 1. - 2. * rng.next();
    }
  }
  CK(cudaMemcpyAsync(c->d_colconst, colc.data(), sizeof(double) * colc.size(), cudaMemcpyHostToDevice, s));
  // kernel parameters
  crm::KParams p;
  memset(&p, 0, sizeof p);
  p.L = c->L;
  p.ncrms = ncrms; p.ld = ld; p.nstop = nstop; p.igstep = d->igstep;
  p.batch_mode = g.batch_mode; p.clamp_batch = 0;
  p.dx = g.crm_dx; p.dy = g.crm_dx; p.dt = dt; p.dt_gl = d->dt_gl;
  p.gams1 = c->gam[4]; p.gams2 = c->gam[5]; p.gamg1 = c->gam[7]; p.gamg2 = c->gam[8];
  p.gamr1 = c->gam[1]; p.gamr2 = c->gam[2];
  p.vrain = c->vrain; p.vsnow = c->vsnow; p.vgrau = c->vgrau;
  p.crain = c->crain; p.csnow = c->csnow; p.cgrau = c->cgrau;
  p.a_bg = c->a_bg; p.a_pr = c->a_pr; p.a_gr = c->a_gr;
  p.nfax = c->ifax[0];
  for (int k = 0; k <= c->ifax[0] && k < 8; ++k) p.ifax[k] = c->ifax[k];
  p.trigs = c->d_consts;
  p.eign = c->d_consts + c->trigs.size();
  p.z0 = c->d_colconst;
  p.rnd = c->d_colconst + ncrms;
  double *const *inp = nullptr;
  (void)inp;
  p.zmid = c->d_in + (size_t)I_ZMID * c->in_elems;
  p.zint = c->d_in + (size_t)I_ZINT * c->in_elems;
  p.tl = c->d_in + (size_t)I_TL * c->in_elems;
  p.ql = c->d_in + (size_t)I_QL * c->in_elems;
  p.qccl = c->d_in + (size_t)I_QCCL * c->in_elems;
  p.qiil = c->d_in + (size_t)I_QIIL * c->in_elems;
  p.pmid = c->d_in + (size_t)I_PMID * c->in_elems;
  p.pint = c->d_in + (size_t)I_PINT * c->in_elems;
  p.pdel = c->d_in + (size_t)I_PDEL * c->in_elems;
  p.ul = c->d_in + (size_t)I_UL * c->in_elems;
  p.vl = c->d_in + (size_t)I_VL * c->in_elems;
  for (int f = 0; f < 7; ++f) p.st[f] = c->d_state + f * n4;
  p.qrad = c->d_rad;
  for (int f = 0; f < 5; ++f) p.radout[f] = c->d_rad + (f + 1) * nr;
  {
    size_t o = 0;
    for (int f = 0; f < CRM_NOUT; ++f) {
      p.out[f] = c->d_out + o;
      o += out_elems(g, f, ld);
    }
    CK(cudaMemsetAsync(c->d_out, 0, sizeof(double) * o, s));
  }
  p.slabs = c->slabs;
  p.col_status = c->d_status;
  int grid = ncrms < c->grid_max ? ncrms : c->grid_max;
  CK(cudaEventRecord(c->ev0, s));
  if (g.precision == CRM_FP64) crm::launch_crm_columns<double>(p, grid, c->block, s);
  else crm::launch_crm_columns<float>(p, grid, c->block, s);
  CK(cudaGetLastError());
  CK(cudaEventRecord(c->ev1, s));
  c->last_launches = 1;
  // results back
  for (int f = 0; f < 7; ++f)
    CK(cudaMemcpyAsync(sp[f], c->d_state + f * n4, sizeof(double) * n4, cudaMemcpyDeviceToHost, s));
  double *rp[5] = {rad->temperature, rad->qv, rad->qc, rad->qi, rad->cld};
  for (int f = 0; f < 5; ++f)
    if (rp[f]) CK(cudaMemcpyAsync(rp[f], c->d_rad + (f + 1) * nr, sizeof(double) * nr, cudaMemcpyDeviceToHost, s));
  for (int f = 0; f < CRM_NOUT; ++f)
    if (out->field[f])
      CK(cudaMemcpyAsync(out->field[f], p.out[f], sizeof(double) * out_elems(g, f, ld), cudaMemcpyDeviceToHost, s));
  std::vector<int> stat(ncrms, 0);
  CK(cudaMemcpyAsync(stat.data(), c->d_status, sizeof(int) * ncrms, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  c->last_kernel_ms = ms;
  int worst = CRM_OK;
  for (int i = 0; i < ncrms; ++i) {
    if (col_status) col_status[i] = stat[i];
    if (stat[i] != CRM_OK) worst = stat[i];
  }
  return worst;
}

}  // extern "C"
