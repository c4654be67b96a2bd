// crm_host.cu -- the C ABI of include/crm_gb300.h: the drop-in for the
// reference's subroutine crm() (crm/crm_module.F90:45-1718).
//
// Host work, once per handle: the per-configuration constants (FFT factors
// and REAL*4 trig tables, fft.F90:156-300; Laplacian eigenvalues,
// pressure.F90:172-198; gamma functions, gammafff.c; fall-speed
// coefficients, microphysics.F90:500-507).  Per call two kernels run: the
// per-column set-up (z0 and the setperturb draws, crm_prep.cu) and the
// persistent column kernel (crm_kernel.cuh).  crm_run stages host arrays
// through the handle's device buffers; crm_run_device takes device arrays;
// crm_run_device_noalloc takes device arrays and no handle, and keeps its
// scratch in a fixed static device array.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/crm_gb300.h"
#include "../../include/crm_detmath.h"
#include "crm_kernel.h"
#include "crm_tc.cuh"

using namespace crm_detmath;

#define R4H(x) ((double)(x##f))

struct crm_ctx {
  crm_config cfg;
  crm::Layout L;
  int device = 0, nsm = 0, shape = 0, grid_max = 0;
  int shape_grid[crm::kNumShapes] = {};   // co-resident CTAs per launch shape
  int slab_cap = 0;                         // slabs allocated (max over shapes)
  int tc_n = 0;                             // 3D transforms on the tensor cores (n) or 0
  float *d_dft = nullptr;                   // their matrices (inside d_consts)
  bool shape_auto = true;                   // choose the shape per call
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
  double *d_consts = nullptr;    // trigs, eign, trigs (float), 3D: trigs_y, trigs_y (float)
  double *d_colconst = nullptr;  // z0 (ncrms), rnd (ncrms * 5 * nx * ny)
  int *d_status = nullptr;
  unsigned long long *d_phase = nullptr;   // per-CTA phase cycle counters
  unsigned long long *d_gsync = nullptr;   // batch-mode grid barrier + maxima
  int ld_cap = 0;
  // host-side constants
  std::vector<double> trigs, eign, trigs_y;
  int ifax[20], ifax_y[20];
  crm::KParams mc;                // gamma functions and fall speeds (micro_consts)
  size_t device_bytes = 0;        // device memory the handle holds
  long long barrier_spins = 1ll << 24;      // grid-barrier wait limit (spins)
  int barrier_withhold = -1;                 // test hook, see crm_debug_barrier_test
  int last_launches = 0;
  double last_kernel_ms = 0.;
  bool pending_timing = false;
};

namespace crm {
struct PrepParams {
  int ncrms, ld, plev, nx, igstep;
  const double *zmid, *zint, *pdel, *tau00, *bflxls, *wndls;
  const int *gcol;
  const int *col_map;
  double *z0;
  double *rnd;
};
void launch_crm_prep(const PrepParams &p, cudaStream_t s);
int launch_crm_consts(void *dst, const void *src, size_t bytes, cudaStream_t s);

// 3D builds no shapes with shared-memory scratch planes (its planes do not
// fit): shapes 2 and 5 are never chosen there (occupancy 0).  The tensor-core
// and contracted-FP64 instances have one launch shape each.
template <typename T, int NX, int NY, int VAR>
static void launch_tn(int shape, const KParams &p, int grid, cudaStream_t s, bool coop) {
  if constexpr (VAR == kVarFma) {
    launch_crm_columns<T, NX, NY, (NY != 1 ? kFmaShape3d : kFmaShape2d), kVarFma>(p, grid, s, coop);
    return;
  }
  if constexpr (NY != 1) {
    if constexpr (sizeof(T) == 4) {
      if (p.tc_n) {
        launch_crm_columns<T, NX, NY, kTcShape, kVarTc>(p, grid, s, coop);
        return;
      }
    }
    switch (shape) {
      case 0: launch_crm_columns<T, NX, NY, 0>(p, grid, s, coop); break;
      case 1: launch_crm_columns<T, NX, NY, 1>(p, grid, s, coop); break;
      case 4: launch_crm_columns<T, NX, NY, 4>(p, grid, s, coop); break;
      default: launch_crm_columns<T, NX, NY, 3>(p, grid, s, coop); break;
    }
    return;
  }
  switch (shape) {
    case 0: launch_crm_columns<T, NX, NY, 0>(p, grid, s, coop); break;
    case 1: launch_crm_columns<T, NX, NY, 1>(p, grid, s, coop); break;
    case 2: launch_crm_columns<T, NX, NY, 2>(p, grid, s, coop); break;
    case 3: launch_crm_columns<T, NX, NY, 3>(p, grid, s, coop); break;
    case 4: launch_crm_columns<T, NX, NY, 4>(p, grid, s, coop); break;
    default: launch_crm_columns<T, NX, NY, 5>(p, grid, s, coop); break;
  }
}

template <typename T, int NX, int NY, int VAR>
static int occupancy_tn(int shape, int nx, int ny, int nzm, int tc_n) {
  if constexpr (VAR == kVarFma) {
    constexpr int fs = NY != 1 ? kFmaShape3d : kFmaShape2d;
    return shape == fs ? occupancy_crm_columns<T, NX, NY, fs, kVarFma>(nx, ny, nzm, 0) : 0;
  }
  if constexpr (NY != 1) {
    if (tc_n) {
      if constexpr (sizeof(T) == 4) {
        if (shape == kTcShape) return occupancy_crm_columns<T, NX, NY, kTcShape, kVarTc>(nx, ny, nzm, tc_n);
      }
      return 0;
    }
    switch (shape) {
      case 0: return occupancy_crm_columns<T, NX, NY, 0>(nx, ny, nzm, tc_n);
      case 1: return occupancy_crm_columns<T, NX, NY, 1>(nx, ny, nzm, tc_n);
      case 3: return occupancy_crm_columns<T, NX, NY, 3>(nx, ny, nzm, tc_n);
      case 4: return occupancy_crm_columns<T, NX, NY, 4>(nx, ny, nzm, tc_n);
      default: return 0;
    }
  }
  switch (shape) {
    case 0: return occupancy_crm_columns<T, NX, NY, 0>(nx, ny, nzm, tc_n);
    case 1: return occupancy_crm_columns<T, NX, NY, 1>(nx, ny, nzm, tc_n);
    case 2: return occupancy_crm_columns<T, NX, NY, 2>(nx, ny, nzm, tc_n);
    case 3: return occupancy_crm_columns<T, NX, NY, 3>(nx, ny, nzm, tc_n);
    case 4: return occupancy_crm_columns<T, NX, NY, 4>(nx, ny, nzm, tc_n);
    default: return occupancy_crm_columns<T, NX, NY, 5>(nx, ny, nzm, tc_n);
  }
}

// 2D: a kernel specialised on nx where one is built; 3D: the generic kernel
template <typename T, int VAR>
static void launch_t(int shape, const KParams &p, int grid, cudaStream_t s, bool coop) {
  if (p.L.ny > 1) {
    launch_tn<T, 0, 0, VAR>(shape, p, grid, s, coop);
    return;
  }
  switch (p.L.nx) {
    case 32: launch_tn<T, 32, 1, VAR>(shape, p, grid, s, coop); break;
    case 64: launch_tn<T, 64, 1, VAR>(shape, p, grid, s, coop); break;
    case 128: launch_tn<T, 128, 1, VAR>(shape, p, grid, s, coop); break;
    default: launch_tn<T, 0, 1, VAR>(shape, p, grid, s, coop); break;
  }
}

template <typename T, int VAR>
static int occupancy_t(int shape, int nx, int nzm, int ny, int tc_n) {
  if (ny > 1) return occupancy_tn<T, 0, 0, VAR>(shape, nx, ny, nzm, tc_n);
  switch (nx) {
    case 32: return occupancy_tn<T, 32, 1, VAR>(shape, nx, 1, nzm, 0);
    case 64: return occupancy_tn<T, 64, 1, VAR>(shape, nx, 1, nzm, 0);
    case 128: return occupancy_tn<T, 128, 1, VAR>(shape, nx, 1, nzm, 0);
    default: return occupancy_tn<T, 0, 1, VAR>(shape, nx, 1, nzm, 0);
  }
}

void launch_columns(int precision, int shape, const KParams &p, int grid, cudaStream_t s, bool coop) {
  if (precision == CRM_FP64) launch_t<double, kVarPlain>(shape, p, grid, s, coop);
  else if (precision == CRM_FP64_FMA) launch_t<double, kVarFma>(shape, p, grid, s, coop);
  else launch_t<float, kVarPlain>(shape, p, grid, s, coop);
}

int occupancy_columns(int precision, int shape, int nx, int nzm, int ny, int tc_n) {
  if (precision == CRM_FP64) return occupancy_t<double, kVarPlain>(shape, nx, nzm, ny, tc_n);
  if (precision == CRM_FP64_FMA) return occupancy_t<double, kVarFma>(shape, nx, nzm, ny, tc_n);
  return occupancy_t<float, kVarPlain>(shape, nx, nzm, ny, tc_n);
}
}  // namespace crm

namespace crm_tc_host {
// floats of the transform matrices of length n: forward (n+2 rounded up to
// 16 rows, n columns), inverse (n rows, n+2 rounded up to 8 columns)
size_t dft_elems(int n) {
  if (!n) return 0;
  const crm::tc::Dims d(n);
  return (size_t)d.nf * n + (size_t)n * d.ki;
}
// The real transform of length n as matrices (fft991's output order and
// scaling, crm/fft.F90): forward Bf[2k][i] = cos(2 pi i k / n) / n,
// Bf[2k+1][i] = -sin(2 pi i k / n) / n; inverse Bi[i][2k] = w_k cos,
// Bi[i][2k+1] = -w_k sin, w_0 = w_n/2 = 1, else 2; Im X_0 and Im X_n/2 rows
// and columns exactly zero; the padding zero.  Angles reduced exactly
// (i k mod n) before the trigonometry, in FP64.
void dft_matrices(float *out, int n) {
  const crm::tc::Dims d(n);
  const double pi = 3.14159265358979323846;
  auto cs = [&](int m, double &c, double &sn) {
    m %= n;
    if (m == 0) { c = 1.; sn = 0.; return; }
    if (2 * m == n) { c = -1.; sn = 0.; return; }
    if (4 * m == n) { c = 0.; sn = 1.; return; }
    if (4 * m == 3 * n) { c = 0.; sn = -1.; return; }
    c = cos(2. * pi * m / n);
    sn = sin(2. * pi * m / n);
  };
  float *bf = out, *bi = out + (size_t)d.nf * n;
  for (int r = 0; r < d.nf; ++r)
    for (int i = 0; i < n; ++i) {
      double v = 0.;
      if (r < n + 2) {
        const int k = r / 2;
        double c, sn;
        cs(i * k, c, sn);
        v = (r % 2 == 0) ? c / n : -sn / n;
      }
      bf[(size_t)r * n + i] = (float)v;
    }
  for (int i = 0; i < n; ++i)
    for (int col = 0; col < d.ki; ++col) {
      double v = 0.;
      if (col < n + 2) {
        const int k = col / 2;
        const double w = (k == 0 || 2 * k == n) ? 1. : 2.;
        double c, sn;
        cs(i * k, c, sn);
        v = (col % 2 == 0) ? w * c : -w * sn;
      }
      bi[(size_t)i * d.ki + col] = (float)v;
    }
}

}  // namespace crm_tc_host

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
void fft_trigs_into(double *trigs, int n) {
  for (int i = 0; i < 3 * n / 2 + 2 + n; ++i) trigs[i] = 0.0;
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
void fft_trigs(std::vector<double> &trigs, int n) {
  trigs.assign(3 * n / 2 + 2 + n, 0.0);
  fft_trigs_into(trigs.data(), n);
}

float gammafff(float x) { return (float)exp(lgamma((double)x)); }

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

// Launch shape of the column kernel per precision (crm_kernel.h kShapes),
// chosen by measurement on GB300; CRM_GB300_SHAPE=<index> overrides it.
int default_shape(int precision, int nx, int ny = 1) {
  const char *e = getenv("CRM_GB300_SHAPE");
  if (e && *e) {
    int v = atoi(e);
    if (v >= 0 && v < crm::kNumShapes) return v;
  }
  // 3D (nx x ny cells per level): 512 threads at 2 CTAs/SM
  if (ny > 1) return precision == CRM_FP64_FMA ? crm::kFmaShape3d : 3;
  // measured on 1024 columns of nx x 58, 30 steps (column-steps/s):
  //   FP64: 256 threads at 3 CTAs/SM (105K at nx 64; the other shapes are
  //     4-15 % slower);
  //   FP32-mixed: 256 threads at 4 CTAs/SM with scratch planes A/B in
  //     shared memory for nx <= 64 (1.06M at nx 32, 586K at nx 64; 4-17 %
  //     over the other shapes), 512 threads at 2 CTAs/SM with the planes in
  //     shared memory for nx >= 128 (291K against 282K without them and
  //     192K at 256 threads).
  if (precision == CRM_FP64) return 0;
  if (precision == CRM_FP64_FMA) return crm::kFmaShape2d;
  return nx >= 128 ? 5 : 2;
}

// crm_accel_nstop (accelerate_crm.F90:84-106): nstop / (1 + crm_accel_factor),
// which must divide it; -1 when it does not.
int accel_nstop(const crm_config &g, int nstop) {
  if (!g.use_crm_accel) return nstop;
  if (!(g.crm_accel_factor >= 0.) || nstop % (int)(1 + g.crm_accel_factor) != 0) return -1;
  return (int)((double)nstop / (1 + g.crm_accel_factor));
}

// A transform length the device FFT takes: fax_crm factors 2, 3, 4 and 5
// (vpass_warp), at most 7 of them; pow2 = true: 2 and 4 only (the 3D CRM
// decodes a cell index with a shift, so its nx and ny are powers of two).
int check_fft_size(int n, bool pow2 = false) {
  int f[20];
  fft_factors(f, n);
  if (f[0] < 1) return CRM_ERR_ARG;
  for (int k = 1; k <= f[0]; ++k) {
    if (f[k] != 2 && f[k] != 3 && f[k] != 4 && f[k] != 5) return CRM_ERR_UNSUPPORTED;
    if (pow2 && f[k] != 2 && f[k] != 4) return CRM_ERR_UNSUPPORTED;
  }
  if (f[0] > 7) return CRM_ERR_ARG;
  return CRM_OK;
}

// The y spacing: crm_dy where a 3D configuration gives one, else crm_dx (the
// reference's grid takes dy = dx)
double crm_dy_of(const crm_config &g) { return g.crm_ny > 1 && g.crm_dy > 0 ? g.crm_dy : g.crm_dx; }

int validate(const crm_config *c) {
  if (!c) return CRM_ERR_ARG;
  if (c->crm_ny < 1) return CRM_ERR_ARG;
  if (c->microphysics != CRM_MICRO_SAM1MOM) return CRM_ERR_UNSUPPORTED;
  if (c->batch_mode != CRM_PER_COLUMN && c->batch_mode != CRM_REFERENCE_BATCH) return CRM_ERR_ARG;
  if (c->precision != CRM_FP64 && c->precision != CRM_FP32_MIXED && c->precision != CRM_FP64_FMA)
    return CRM_ERR_ARG;
  if (c->crm_nx < 8 || c->crm_nx % 2 || c->crm_nz < 4 || c->plev < c->crm_nz + 2) return CRM_ERR_ARG;
  if (c->crm_nx_rad < 1 || c->crm_nx % c->crm_nx_rad) return CRM_ERR_ARG;
  if (!(c->crm_dx > 0) || !(c->crm_dt > 0) || 60. < 2 * c->crm_dt) return CRM_ERR_ARG;
  if (c->max_ncrms < 1) return CRM_ERR_ARG;
  int rc = check_fft_size(c->crm_nx, c->crm_ny > 1);
  if (rc != CRM_OK) return rc;
  if (c->crm_ny == 1) {
    if (c->crm_ny_rad != 1) return CRM_ERR_ARG;
  } else {
    // 3D: ny a transform length of its own; radiation on every CRM column
    if (c->crm_ny < 8) return CRM_ERR_ARG;
    rc = check_fft_size(c->crm_ny, true);
    if (rc != CRM_OK) return rc;
    if (c->crm_dy < 0) return CRM_ERR_ARG;
    if (c->crm_ny_rad < 1 || c->crm_ny % c->crm_ny_rad) return CRM_ERR_ARG;
    if (c->crm_nx_rad != c->crm_nx || c->crm_ny_rad != c->crm_ny) return CRM_ERR_UNSUPPORTED;
  }
  return CRM_OK;
}

// Per-configuration constants, written into caller-provided storage so that
// the handle (alloc_ctx) and the no-allocation entry build the same values:
//   trigs: 3 n / 2 + 2 + n REAL*4 trig values of a transform of length n
//          (fft.F90:247-300)
//   eign:  Laplacian eigenvalues (pressure.F90:172-198), (nx + 1) x (ny + 2)
//          with i fastest in 3D, nx + 1 in 2D (jd = 0)
size_t n_trigs(int n) { return 3 * (size_t)n / 2 + 2 + n; }
size_t n_eigen(const crm_config &g) { return (size_t)(g.crm_nx + 1) * (g.crm_ny > 1 ? g.crm_ny + 2 : 1); }
void laplace_eigen(double *eign, const crm_config &g) {
  const int nx = g.crm_nx, ny = g.crm_ny;
  double dx = g.crm_dx, dy = crm_dy_of(g);
  double ddx2 = 1.0 / (dx * dx), ddy2 = 1.0 / (dy * dy);
  double pii = 3.14159265358979323846;
  double xnx = pii / nx, xny = pii / ny;
  const int nj = ny > 1 ? ny + 2 : 1;
  for (int j = 1; j <= nj; ++j) {
    int jd = (int)(((float)j - 0.1f) / 2.f);
    double xj = jd, facty = 2.0;
    for (int i = 1; i <= nx + 1; ++i) {
      int id = (int)(((float)i - 0.1f) / 2.f);
      double xi = id, factx = 2.0;
      eign[(size_t)(j - 1) * (nx + 1) + (i - 1)] =
          (2.0 * cos(factx * xnx * xi) - 2.0) * ddx2 + (2.0 * cos(facty * xny * xj) - 2.0) * ddy2;
    }
  }
}

// Gamma functions and fall-speed coefficients of sam1mom
// (precip_init.F90:25-49, microphysics.F90:500-507) into the kernel
// parameters.
void micro_consts(crm::KParams &p) {
  const double b_rain = R4H(0.8), b_snow = 0.25, b_grau = 0.5;
  double gam[10];
  gam[0] = gammafff(3.f);
  gam[1] = gammafff((float)(3. + b_rain));
  gam[2] = gammafff((float)((5. + b_rain) / 2.));
  gam[3] = gammafff((float)(4. + b_rain));
  gam[4] = gammafff((float)(3. + b_snow));
  gam[5] = gammafff((float)((5. + b_snow) / 2.));
  gam[6] = gammafff((float)(4. + b_snow));
  gam[7] = gammafff((float)(3. + b_grau));
  gam[8] = gammafff((float)((5. + b_grau) / 2.));
  gam[9] = gammafff((float)(4. + b_grau));
  p.gams1 = gam[4]; p.gams2 = gam[5]; p.gamg1 = gam[7]; p.gamg2 = gam[8];
  p.gamr1 = gam[1]; p.gamr2 = gam[2];
  p.crain = b_rain / 4.; p.csnow = b_snow / 4.; p.cgrau = b_grau / 4.;
  p.vrain = 842. * gam[3] / 6. / det_pow(kPi4 * 1000. * 8.e6, p.crain);
  p.vsnow = R4H(4.84) * gam[6] / 6. / det_pow(kPi4 * 100. * 3.e6, p.csnow);
  p.vgrau = 94.5 * gam[9] / 6. / det_pow(kPi4 * 400. * 4.e6, p.cgrau);
  p.a_bg = 1. / (R4H(273.16) - R4H(253.16));
  p.a_pr = 1. / (R4H(283.16) - R4H(268.16));
  p.a_gr = 1. / (R4H(283.16) - R4H(223.16));
}

// The 3D FP32-mixed form with nx = ny in {16, 32} can run the transforms of
// the pressure solve on the tensor cores (CRM_GB300_TRANSFORM=tc).  Not the
// default: they are 2.5x faster than the warp FFT, but a kernel with tcgen05
// code runs one CTA per SM, and the warp-FFT kernel at two CTAs per SM is
// 9 % faster overall on 256 columns of 32 x 32 x 58.
int tc_n_of(const crm_config &g) {
  if (g.precision != CRM_FP32_MIXED || g.crm_ny <= 1 || g.crm_nx != g.crm_ny) return 0;
  if (g.crm_nx != 16 && g.crm_nx != 32) return 0;
  const char *e = getenv("CRM_GB300_TRANSFORM");
  if (!e || strcmp(e, "tc") != 0) return 0;
  return g.crm_nx;
}
using crm_tc_host::dft_elems;
using crm_tc_host::dft_matrices;

// Sizes of a handle's device buffers, decided without allocating: the slab
// count is the largest co-resident CTA count over the launch shapes (so the
// shape can change per call), capped at max_ncrms.
int plan_ctx(crm_ctx *c) {
  const crm_config &g = c->cfg;
  CK(cudaGetDevice(&c->device));
  CK(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->device));
  const size_t esz = g.precision == CRM_FP32_MIXED ? sizeof(float) : sizeof(double);
  c->L = crm::make_layout(g.crm_nx, g.crm_nz, g.plev, g.crm_nx_rad, (int)esz, g.crm_ny, g.crm_ny_rad);
  c->tc_n = tc_n_of(g);
  c->slab_cap = 0;
  for (int s = 0; s < crm::kNumShapes; ++s) {
    int per = crm::occupancy_columns(g.precision, s, g.crm_nx, g.crm_nz, g.crm_ny, c->tc_n);
    int grid = per > 0 ? c->nsm * per : 0;
    if (grid > g.max_ncrms) grid = g.max_ncrms;
    c->shape_grid[s] = grid;
    if (grid > c->slab_cap) c->slab_cap = grid;
  }
  c->slab_bytes = c->L.slab * esz;
  c->ld_cap = g.max_ncrms;
  return CRM_OK;
}

// The handle's default launch shape: the measured default of its precision
// and size if that shape can run this handle's kernel, else the launchable
// shape with the most co-resident CTAs (the tensor-core and contracted-FP64
// instances have one shape each).
int handle_default_shape(const crm_ctx *c) {
  const crm_config &g = c->cfg;
  int s = default_shape(g.precision, g.crm_nx, g.crm_ny);
  if (c->shape_grid[s] > 0) return s;
  int best = -1;
  for (int s2 = 0; s2 < crm::kNumShapes; ++s2)
    if (c->shape_grid[s2] > 0 && (best < 0 || c->shape_grid[s2] > c->shape_grid[best])) best = s2;
  return best < 0 ? s : best;
}

// Device bytes alloc_ctx allocates for a planned handle (the staging
// buffers of crm_run come later, on its first call).
size_t handle_bytes(const crm_ctx *c) {
  const crm_config &g = c->cfg;
  const size_t ld = (size_t)c->ld_cap, nt = n_trigs(g.crm_nx), nty = g.crm_ny > 1 ? n_trigs(g.crm_ny) : 0;
  size_t b = c->slab_bytes * (size_t)c->slab_cap;
  b += sizeof(double) * (nt + n_eigen(g) + (nt + 1) / 2 + nty + (nty + 1) / 2 + (dft_elems(c->tc_n) + 1) / 2);
  b += sizeof(double) * ld * (1 + 5 * (size_t)g.crm_nx * g.crm_ny);
  b += sizeof(int) * ld + 8 * sizeof(unsigned long long);
  return b;
}

int alloc_ctx(crm_ctx *c) {
  const crm_config &g = c->cfg;
  int rc = plan_ctx(c);
  if (rc != CRM_OK) return rc;
  c->shape = handle_default_shape(c);
  {
    const char *e = getenv("CRM_GB300_SHAPE");
    if (e && *e) c->shape_auto = false;
  }
  if (c->shape_grid[c->shape] < 1) {
    for (int s = 0; s < crm::kNumShapes; ++s)
      if (c->shape_grid[s] > 0) { c->shape = s; break; }
  }
  if (c->shape_grid[c->shape] < 1) return CRM_ERR_UNSUPPORTED;
  c->grid_max = c->shape_grid[c->shape];
  CK(cudaMalloc(&c->slabs, c->slab_bytes * (size_t)c->slab_cap));
  const int ld = c->ld_cap, nx = g.crm_nx, ny = g.crm_ny;
  fft_factors(c->ifax, nx);
  fft_trigs(c->trigs, nx);
  c->eign.assign(n_eigen(g), 0.0);
  laplace_eigen(c->eign.data(), g);
  c->ifax_y[0] = 0;
  c->trigs_y.clear();
  if (ny > 1) {
    fft_factors(c->ifax_y, ny);
    fft_trigs(c->trigs_y, ny);
  }
  // trigs, eign (FP64), trigs again as float (exact: REAL*4 values), then
  // in 3D the y table as FP64 and as float
  const size_t nt = c->trigs.size(), ne = c->eign.size(), ntf = (nt + 1) / 2;
  const size_t nty = c->trigs_y.size(), ntyf = (nty + 1) / 2;
  const size_t ndft = dft_elems(c->tc_n), ndftd = (ndft + 1) / 2;
  CK(cudaMalloc(&c->d_consts, sizeof(double) * (nt + ne + ntf + nty + ntyf + ndftd)));
  CK(cudaMemcpy(c->d_consts, c->trigs.data(), sizeof(double) * nt, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d_consts + nt, c->eign.data(), sizeof(double) * ne, cudaMemcpyHostToDevice));
  {
    std::vector<float> tf(nt);
    for (size_t i = 0; i < nt; ++i) tf[i] = (float)c->trigs[i];
    CK(cudaMemcpy(c->d_consts + nt + ne, tf.data(), sizeof(float) * nt, cudaMemcpyHostToDevice));
  }
  if (nty) {
    double *dy = c->d_consts + nt + ne + ntf;
    CK(cudaMemcpy(dy, c->trigs_y.data(), sizeof(double) * nty, cudaMemcpyHostToDevice));
    std::vector<float> tf(nty);
    for (size_t i = 0; i < nty; ++i) tf[i] = (float)c->trigs_y[i];
    CK(cudaMemcpy(dy + nty, tf.data(), sizeof(float) * nty, cudaMemcpyHostToDevice));
  }
  if (ndft) {
    std::vector<float> m(ndft);
    dft_matrices(m.data(), c->tc_n);
    c->d_dft = reinterpret_cast<float *>(c->d_consts + nt + ne + ntf + nty + ntyf);
    CK(cudaMemcpy(c->d_dft, m.data(), sizeof(float) * ndft, cudaMemcpyHostToDevice));
  }
  CK(cudaMalloc(&c->d_colconst, sizeof(double) * (size_t)ld * (1 + 5 * (size_t)nx * ny)));
  CK(cudaMalloc(&c->d_status, sizeof(int) * (size_t)ld));
  CK(cudaMalloc(&c->d_gsync, 8 * sizeof(unsigned long long)));
  CK(cudaMemset(c->d_gsync, 0, 8 * sizeof(unsigned long long)));
  c->device_bytes = handle_bytes(c);
#ifdef CRM_PHASE_TIMERS
  CK(cudaMalloc(&c->d_phase, sizeof(unsigned long long) * 64 * (size_t)c->slab_cap));
  CK(cudaMemset(c->d_phase, 0, sizeof(unsigned long long) * 64 * (size_t)c->slab_cap));
#endif
  micro_consts(c->mc);
  CK(cudaEventCreate(&c->ev0));
  CK(cudaEventCreate(&c->ev1));
  return CRM_OK;
}

// crm_run's staging buffers for host arguments, allocated by its first call
// (a handle used only through crm_run_device never holds them).
int ensure_staging(crm_ctx *c) {
  if (c->d_in) return CRM_OK;
  const crm_config &g = c->cfg;
  const int ld = c->ld_cap, plev = g.plev, nx = g.crm_nx, ny = g.crm_ny, nz = g.crm_nz;
  c->in_elems = (size_t)ld * (plev + 1);
  // GCM profiles, then tau00, bflxls, wndls (ld each), gcol and col_map (ld ints each)
  const size_t b_in = sizeof(double) * c->in_elems * I_NIN + sizeof(double) * 4 * ld;
  const size_t b_st = sizeof(double) * (size_t)ld * nx * ny * nz * 7;
  const size_t b_rad = sizeof(double) * (size_t)ld * g.crm_nx_rad * g.crm_ny_rad * nz * 6;
  size_t no = 0;
  for (int f = 0; f < CRM_NOUT; ++f) no += out_elems(g, f, ld);
  CK(cudaMalloc(&c->d_in, b_in));
  CK(cudaMalloc(&c->d_state, b_st));
  CK(cudaMalloc(&c->d_rad, b_rad));
  CK(cudaMalloc(&c->d_out, sizeof(double) * no));
  c->device_bytes += b_in + b_st + b_rad + sizeof(double) * no;
  return CRM_OK;
}

void free_ctx(crm_ctx *c) {
  if (!c) return;
  cudaFree(c->slabs); cudaFree(c->d_in); cudaFree(c->d_state); cudaFree(c->d_rad);
  cudaFree(c->d_out); cudaFree(c->d_consts); cudaFree(c->d_colconst); cudaFree(c->d_status);
  if (c->d_phase) cudaFree(c->d_phase);
  if (c->d_gsync) cudaFree(c->d_gsync);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
}

// Checks one call on device-resident arguments and fills the parameters of
// its set-up and column kernels.
int build_params(crm_ctx *c, const crm_call_desc *d, const crm_input_c *in, crm_state_c *st, crm_rad_c *rad,
                 crm_output_c *out, int *d_status, crm::KParams &p, crm::PrepParams &pp) {
  const crm_config &g = c->cfg;
  const int ncrms = d->ncrms, ld = d->ld;
  if (ncrms < 1 || ld < ncrms || ncrms > g.max_ncrms || !(d->dt_gl > 0)) return CRM_ERR_ARG;
  if (!d->gcol && d->igstep <= 1) return CRM_ERR_ARG;
  const double *need[] = {in->zmid, in->zint, in->tl, in->ql, in->qccl, in->qiil, in->pmid,
                          in->pint, in->pdel, in->ul, in->vl, in->tau00, in->bflxls, in->wndls};
  for (const double *q : need)
    if (!q) return CRM_ERR_ARG;
  double *sp[7] = {st->u_wind, st->v_wind, st->w_wind, st->temperature, st->qt, st->qp, st->qn};
  for (double *q : sp)
    if (!q) return CRM_ERR_ARG;
  double *rp[5] = {rad->temperature, rad->qv, rad->qc, rad->qi, rad->cld};
  if (!rad->qrad) return CRM_ERR_ARG;
  for (double *q : rp)
    if (!q) return CRM_ERR_ARG;
  for (int f = 0; f < CRM_NOUT; ++f)
    if (!out->field[f]) return CRM_ERR_ARG;
  int nstop = (int)(d->dt_gl / g.crm_dt);       // crm_module.F90:712-713
  if (nstop < 1) return CRM_ERR_ARG;
  double dt = d->dt_gl / nstop;
  if (60. < 2 * dt) return CRM_ERR_ARG;         // damping.F90:39-42
  const int nstop_run = accel_nstop(g, nstop);   // crm_module.F90:718-720
  if (nstop_run < 1) return CRM_ERR_ARG;
  pp.ncrms = ncrms; pp.ld = ld; pp.plev = g.plev; pp.nx = g.crm_nx * g.crm_ny; pp.igstep = d->igstep;
  pp.zmid = in->zmid; pp.zint = in->zint; pp.pdel = in->pdel;
  pp.tau00 = in->tau00; pp.bflxls = in->bflxls; pp.wndls = in->wndls;
  pp.gcol = d->gcol;
  pp.col_map = d->col_map;
  pp.z0 = c->d_colconst;
  pp.rnd = c->d_colconst + g.max_ncrms;
  memset(&p, 0, sizeof p);
  p.L = c->L;
  p.ncrms = ncrms; p.ld = ld; p.nstop = nstop; p.igstep = d->igstep;
  p.batch_mode = g.batch_mode; p.clamp_batch = 0;
  p.nstop = nstop_run;
  p.use_accel = g.use_crm_accel != 0; p.accel_uv = g.crm_accel_uv != 0;
  p.accel_factor = g.crm_accel_factor;
  p.dx = g.crm_dx; p.dy = crm_dy_of(g); p.dt = dt; p.dt_gl = d->dt_gl;
  p.gams1 = c->mc.gams1; p.gams2 = c->mc.gams2; p.gamg1 = c->mc.gamg1; p.gamg2 = c->mc.gamg2;
  p.gamr1 = c->mc.gamr1; p.gamr2 = c->mc.gamr2;
  p.vrain = c->mc.vrain; p.vsnow = c->mc.vsnow; p.vgrau = c->mc.vgrau;
  p.crain = c->mc.crain; p.csnow = c->mc.csnow; p.cgrau = c->mc.cgrau;
  p.a_bg = c->mc.a_bg; p.a_pr = c->mc.a_pr; p.a_gr = c->mc.a_gr;
  p.nfax = c->ifax[0];
  for (int k = 0; k <= c->ifax[0] && k < 8; ++k) p.ifax[k] = c->ifax[k];
  p.trigs = c->d_consts;
  p.eign = c->d_consts + c->trigs.size();
  p.trigs_f = reinterpret_cast<const float *>(c->d_consts + c->trigs.size() + c->eign.size());
  if (!c->trigs_y.empty()) {
    p.nfax_y = c->ifax_y[0];
    for (int k = 0; k <= c->ifax_y[0] && k < 8; ++k) p.ifax_y[k] = c->ifax_y[k];
    p.trigs_y = c->d_consts + c->trigs.size() + c->eign.size() + (c->trigs.size() + 1) / 2;
    p.trigs_y_f = reinterpret_cast<const float *>(p.trigs_y + c->trigs_y.size());
  }
  p.tc_n = c->tc_n;
  p.dft_tc = c->d_dft;
  p.z0 = pp.z0;
  p.rnd = pp.rnd;
  p.zmid = in->zmid; p.zint = in->zint; p.tl = in->tl; p.ql = in->ql; p.qccl = in->qccl;
  p.qiil = in->qiil; p.pmid = in->pmid; p.pint = in->pint; p.pdel = in->pdel;
  p.ul = in->ul; p.vl = in->vl;
  for (int f = 0; f < 7; ++f) p.st[f] = sp[f];
  p.qrad = rad->qrad;
  for (int f = 0; f < 5; ++f) p.radout[f] = rp[f];
  for (int f = 0; f < CRM_NOUT; ++f) p.out[f] = out->field[f];
  p.slabs = c->slabs;
  p.col_map = d->col_map;
  p.phase_cycles = c->d_phase;
  p.col_status = d_status ? d_status : c->d_status;
  return CRM_OK;
}

// Enqueue the set-up and column kernels for device-resident arguments.
int enqueue(crm_ctx *c, const crm_call_desc *d, const crm_input_c *in, crm_state_c *st, crm_rad_c *rad,
            crm_output_c *out, int *d_status, cudaStream_t s) {
  crm::KParams p;
  crm::PrepParams pp;
  int rc = build_params(c, d, in, st, rad, out, d_status, p, pp);
  if (rc != CRM_OK) return rc;
  const crm_config &g = c->cfg;
  const int ncrms = d->ncrms;
  if (c->shape_auto) {
    // A call that fits the GPU in one round runs fastest with the most
    // threads per column (1024 threads: 10.2 ms for 16 columns of 64 x 58
    // against 17.9 ms at 256); larger batches take the throughput default.
    int best = -1;
    for (int s2 = 0; s2 < crm::kNumShapes; ++s2)
      if (c->shape_grid[s2] >= ncrms && (best < 0 || crm::kShapes[s2].threads > crm::kShapes[best].threads))
        best = s2;
    const int dflt = handle_default_shape(c);
    if (best < 0 || c->shape_grid[dflt] >= ncrms && crm::kShapes[dflt].threads >= crm::kShapes[best].threads)
      best = dflt;
    c->shape = best;
    c->grid_max = c->shape_grid[best];
  }
  const bool batch = g.batch_mode == CRM_REFERENCE_BATCH;
  // reference-batch mode: one co-resident CTA per column (cooperative
  // launch), so the batch must fit the GPU at once and slots are 0..ncrms-1
  if (batch && (ncrms > c->grid_max || d->col_map)) return CRM_ERR_UNSUPPORTED;
  p.gsync = c->d_gsync;
  p.barrier_spins = c->barrier_spins;
  p.barrier_withhold = c->barrier_withhold;
  int grid = ncrms < c->grid_max ? ncrms : c->grid_max;
  CK(cudaEventRecord(c->ev0, s));
  if (batch) CK(cudaMemsetAsync(c->d_gsync, 0, 8 * sizeof(unsigned long long), s));
  crm::launch_crm_prep(pp, s);
  crm::launch_columns(g.precision, c->shape, p, grid, s, batch);
  CK(cudaGetLastError());
  CK(cudaEventRecord(c->ev1, s));
  c->last_launches = 2;
  c->pending_timing = true;
  return CRM_OK;
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
  if (!c) {
    if (status) *status = CRM_ERR_ARG;
    return nullptr;
  }
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

double crm_last_kernel_ms(const crm_ctx *ctx) {
  if (!ctx) return 0.;
  if (ctx->pending_timing) {
    float ms = 0.f;
    if (cudaEventSynchronize(ctx->ev1) == cudaSuccess && cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) == cudaSuccess)
      return ms;
    return 0.;
  }
  return ctx->last_kernel_ms;
}

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
    case CRM_ERR_TOO_LARGE: return "call exceeds the 32 MiB fixed scratch of crm_run_device_noalloc";
  }
  return "unknown status";
}

// Per-phase cycle counters summed over the CTAs (profiling builds only,
// -DCRM_PHASE_TIMERS); returns the number of phases written or -1.
int crm_debug_phase_cycles(crm_ctx *ctx, unsigned long long *out, int n) {
  if (!ctx || !ctx->d_phase || !out) return -1;
  std::vector<unsigned long long> h((size_t)64 * ctx->slab_cap);
  if (cudaMemcpy(h.data(), ctx->d_phase, sizeof(unsigned long long) * h.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
    return -1;
  int m = n < crm::PH_COUNT ? n : crm::PH_COUNT;
  for (int i = 0; i < m; ++i) {
    unsigned long long s = 0;
    for (int b = 0; b < ctx->slab_cap; ++b) s += h[(size_t)b * 64 + i];
    out[i] = s;
  }
  cudaMemset(ctx->d_phase, 0, sizeof(unsigned long long) * h.size());
  return m;
}

int crm_num_launch_shapes(void) { return crm::kNumShapes; }

int crm_launch_shape_info(int shape, int *threads, int *ctas_per_sm, int *smem_planes) {
  if (shape < 0 || shape >= crm::kNumShapes) return CRM_ERR_ARG;
  if (threads) *threads = crm::kShapes[shape].threads;
  if (ctas_per_sm) *ctas_per_sm = crm::kShapes[shape].min_ctas;
  if (smem_planes) *smem_planes = crm::kShapes[shape].smem_planes;
  return CRM_OK;
}

int crm_set_launch_shape(crm_ctx *ctx, int shape) {
  if (!ctx) return CRM_ERR_ARG;
  if (shape == -1) {                       // back to the per-call choice
    ctx->shape_auto = true;
    ctx->shape = handle_default_shape(ctx);
    ctx->grid_max = ctx->shape_grid[ctx->shape];
    return CRM_OK;
  }
  if (shape < 0 || shape >= crm::kNumShapes || ctx->shape_grid[shape] < 1) return CRM_ERR_ARG;
  ctx->shape_auto = false;
  ctx->shape = shape;
  ctx->grid_max = ctx->shape_grid[shape];
  return CRM_OK;
}

int crm_get_launch_shape(const crm_ctx *ctx) { return ctx ? ctx->shape : -1; }

int crm_debug_barrier_test(crm_ctx *ctx, long long spin_limit, int withhold_column) {
  if (!ctx || spin_limit < 1 || withhold_column < -1) return CRM_ERR_ARG;
  ctx->barrier_spins = spin_limit;
  ctx->barrier_withhold = withhold_column;
  return CRM_OK;
}

unsigned long long crm_device_bytes(const crm_ctx *ctx) { return ctx ? (unsigned long long)ctx->device_bytes : 0ull; }

int crm_plan_device_bytes(const crm_config *cfg, unsigned long long *bytes) {
  if (!bytes) return CRM_ERR_ARG;
  *bytes = 0;
  int rc = validate(cfg);
  int ndev = 0;
  if (rc == CRM_OK && (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)) rc = CRM_ERR_NO_DEVICE;
  if (rc != CRM_OK) return rc;
  crm_ctx c;
  c.cfg = *cfg;
  rc = plan_ctx(&c);
  if (rc != CRM_OK) return rc;
  *bytes = handle_bytes(&c);
  return CRM_OK;
}

const char *crm_version(void) { return "crm-gb300 0.2 (sm_103a; 2D and 3D sam1mom; fp64 plain + fp32 mixed)"; }

int crm_run_device(crm_ctx *c, const crm_call_desc *d, const crm_input_c *in, crm_state_c *st, crm_rad_c *rad,
                   crm_output_c *out, int *col_status, void *stream) {
  if (!c || !d || !in || !st || !rad || !out) return CRM_ERR_ARG;
  cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
  return enqueue(c, d, in, st, rad, out, col_status, s);
}

int crm_run(crm_ctx *c, const crm_call_desc *d, const crm_input_c *in, crm_state_c *st, crm_rad_c *rad,
            crm_output_c *out, int *col_status) {
  if (!c || !d || !in || !st || !rad || !out) return CRM_ERR_ARG;
  const crm_config &g = c->cfg;
  const int ncrms = d->ncrms, ld = d->ld, plev = g.plev, nx = g.crm_nx, ny = g.crm_ny, nz = g.crm_nz;
  if (ncrms < 1 || ld < ncrms || ld > c->ld_cap) return CRM_ERR_ARG;
  if (!d->gcol && d->igstep <= 1) return CRM_ERR_ARG;
  {
    int rs = ensure_staging(c);
    if (rs != CRM_OK) return rs;
  }
  cudaStream_t s = c->stream;
  // stage the host arguments through the handle's device buffers
  crm_input_c din;
  memset(&din, 0, sizeof din);
  const double *src[I_NIN] = {in->zmid, in->zint, in->tl, in->ql, in->qccl, in->qiil,
                              in->pmid, in->pint, in->pdel, in->ul, in->vl};
  const double **dst[I_NIN] = {&din.zmid, &din.zint, &din.tl, &din.ql, &din.qccl, &din.qiil,
                               &din.pmid, &din.pint, &din.pdel, &din.ul, &din.vl};
  for (int f = 0; f < I_NIN; ++f) {
    if (!src[f]) return CRM_ERR_ARG;
    size_t n = (size_t)ld * ((f == I_ZINT || f == I_PINT) ? plev + 1 : plev);
    double *dp = c->d_in + (size_t)f * c->in_elems;
    CK(cudaMemcpyAsync(dp, src[f], sizeof(double) * n, cudaMemcpyHostToDevice, s));
    *dst[f] = dp;
  }
  double *scal = c->d_in + (size_t)I_NIN * c->in_elems;
  const double *s1[3] = {in->tau00, in->bflxls, in->wndls};
  const double **d1[3] = {&din.tau00, &din.bflxls, &din.wndls};
  for (int f = 0; f < 3; ++f) {
    if (!s1[f]) return CRM_ERR_ARG;
    CK(cudaMemcpyAsync(scal + (size_t)f * c->ld_cap, s1[f], sizeof(double) * ld, cudaMemcpyHostToDevice, s));
    *d1[f] = scal + (size_t)f * c->ld_cap;
  }
  int *dgcol = reinterpret_cast<int *>(scal + (size_t)3 * c->ld_cap);
  if (d->gcol) CK(cudaMemcpyAsync(dgcol, d->gcol, sizeof(int) * ncrms, cudaMemcpyHostToDevice, s));
  int *dmap = dgcol + c->ld_cap;
  if (d->col_map) CK(cudaMemcpyAsync(dmap, d->col_map, sizeof(int) * ncrms, cudaMemcpyHostToDevice, s));
  crm_call_desc dd = *d;
  dd.gcol = d->gcol ? dgcol : nullptr;
  dd.col_map = d->col_map ? dmap : nullptr;
  double *sp[7] = {st->u_wind, st->v_wind, st->w_wind, st->temperature, st->qt, st->qp, st->qn};
  const size_t n4 = (size_t)ld * nx * ny * nz;
  crm_state_c dst_state;
  double **ds[7] = {&dst_state.u_wind, &dst_state.v_wind, &dst_state.w_wind, &dst_state.temperature,
                    &dst_state.qt, &dst_state.qp, &dst_state.qn};
  for (int f = 0; f < 7; ++f) {
    if (!sp[f]) return CRM_ERR_ARG;
    CK(cudaMemcpyAsync(c->d_state + f * n4, sp[f], sizeof(double) * n4, cudaMemcpyHostToDevice, s));
    *ds[f] = c->d_state + f * n4;
  }
  const size_t nr = (size_t)ld * g.crm_nx_rad * g.crm_ny_rad * nz;
  if (!rad->qrad) return CRM_ERR_ARG;
  CK(cudaMemcpyAsync(c->d_rad, rad->qrad, sizeof(double) * nr, cudaMemcpyHostToDevice, s));
  crm_rad_c drad;
  drad.qrad = c->d_rad;
  double **dr[5] = {&drad.temperature, &drad.qv, &drad.qc, &drad.qi, &drad.cld};
  for (int f = 0; f < 5; ++f) *dr[f] = c->d_rad + (f + 1) * nr;
  crm_output_c dout;
  size_t o = 0;
  for (int f = 0; f < CRM_NOUT; ++f) {
    dout.field[f] = c->d_out + o;
    o += out_elems(g, f, ld);
  }
  double *rp[5] = {rad->temperature, rad->qv, rad->qc, rad->qi, rad->cld};
  // Results travel back for the columns the call integrated only: columns
  // 0..ncrms-1 as strided rows of every (ld, ...) array, or, under a
  // col_map, whole arrays after staging the host values of the rad means and
  // outputs, so slots outside the map keep their host contents.
  const bool mapped = d->col_map != nullptr;
  if (!mapped) CK(cudaMemsetAsync(c->d_out, 0, sizeof(double) * o, s));
  if (mapped) {
    for (int f = 0; f < 5; ++f)
      if (rp[f]) CK(cudaMemcpyAsync(c->d_rad + (f + 1) * nr, rp[f], sizeof(double) * nr, cudaMemcpyHostToDevice, s));
    for (int f = 0; f < CRM_NOUT; ++f)
      if (out->field[f])
        CK(cudaMemcpyAsync(dout.field[f], out->field[f], sizeof(double) * out_elems(g, f, ld), cudaMemcpyHostToDevice, s));
  }
  int rc = enqueue(c, &dd, &din, &dst_state, &drad, &dout, c->d_status, s);
  if (rc != CRM_OK) return rc;
  const int cols = mapped ? ld : ncrms;
  auto back = [&](double *dst, const double *src, size_t elems) -> cudaError_t {
    const size_t rows = elems / (size_t)ld;
    if (cols == ld) return cudaMemcpyAsync(dst, src, sizeof(double) * elems, cudaMemcpyDeviceToHost, s);
    return cudaMemcpy2DAsync(dst, sizeof(double) * ld, src, sizeof(double) * ld, sizeof(double) * cols, rows,
                             cudaMemcpyDeviceToHost, s);
  };
  for (int f = 0; f < 7; ++f) CK(back(sp[f], c->d_state + f * n4, n4));
  for (int f = 0; f < 5; ++f)
    if (rp[f]) CK(back(rp[f], c->d_rad + (f + 1) * nr, nr));
  for (int f = 0; f < CRM_NOUT; ++f)
    if (out->field[f]) CK(back(out->field[f], dout.field[f], out_elems(g, f, ld)));
  std::vector<int> stat(ncrms, 0);
  CK(cudaMemcpyAsync(stat.data(), c->d_status, sizeof(int) * ncrms, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  c->last_kernel_ms = ms;
  c->pending_timing = false;
  int worst = CRM_OK;
  for (int i = 0; i < ncrms; ++i) {
    if (col_status) col_status[i] = stat[i];
    if (stat[i] != CRM_OK) worst = stat[i];
  }
  return worst;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// crm_run_device_noalloc: the same two kernels with their scratch in one
// fixed static device array instead of handle buffers.  Nothing here calls
// cudaMalloc/cudaFree or allocates host memory: the per-configuration
// constants are built in fixed-size host arrays on the stack and written into
// the static array by small kernels that carry them as parameters, so every
// device operation of a call is a kernel launch on the caller's stream and
// the call can be captured into a CUDA graph.

namespace {

// Scratch layout: [trigs | eign] [z0 (ncrms) | rnd (ncrms * 5 * nx)] [slabs].
static __device__ __align__(256) unsigned char crm_noalloc_scratch[CRM_NOALLOC_SCRATCH_BYTES];

constexpr int kNoallocMaxDevices = 64;
constexpr int kNoallocMaxTrigs = 3 * CRM_NOALLOC_MAX_NX / 2 + 2 + CRM_NOALLOC_MAX_NX;

struct NoallocDevice {
  unsigned char *scratch = nullptr;   // device address of crm_noalloc_scratch
  int nsm = 0;
};
NoallocDevice g_noalloc[kNoallocMaxDevices];
std::mutex g_noalloc_mu;

size_t round256(size_t n) { return (n + 255) / 256 * 256; }

struct NoallocPlan {
  crm::Layout L;
  size_t esz, const_bytes, col_bytes, slab_bytes;
  int ntrigs, neign, nslab;
};

// Host arithmetic only: what one call needs and how many slabs fit.
int noalloc_plan(const crm_config &g, int ncrms, NoallocPlan &q) {
  if (g.crm_nx > CRM_NOALLOC_MAX_NX) return CRM_ERR_TOO_LARGE;
  q.esz = g.precision == CRM_FP32_MIXED ? sizeof(float) : sizeof(double);
  q.L = crm::make_layout(g.crm_nx, g.crm_nz, g.plev, g.crm_nx_rad, (int)q.esz);
  q.ntrigs = 3 * g.crm_nx / 2 + 2 + g.crm_nx;
  q.neign = g.crm_nx + 1;
  q.const_bytes = round256(sizeof(double) * (size_t)(q.ntrigs + q.neign) + sizeof(float) * (size_t)q.ntrigs);
  q.col_bytes = round256(sizeof(double) * (size_t)ncrms * (1 + 5 * (size_t)g.crm_nx));
  q.slab_bytes = round256(q.L.slab * q.esz);
  const size_t cap = CRM_NOALLOC_SCRATCH_BYTES;
  if (q.const_bytes > cap || q.col_bytes > cap - q.const_bytes ||
      q.slab_bytes > cap - q.const_bytes - q.col_bytes)
    return CRM_ERR_TOO_LARGE;
  size_t n = (cap - q.const_bytes - q.col_bytes) / q.slab_bytes;
  q.nslab = n > (size_t)ncrms ? ncrms : (int)n;
  return CRM_OK;
}

// Once per device, with that device current: the array's device address.
int noalloc_device(NoallocDevice &out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return CRM_ERR_NO_DEVICE;
  if (dev >= kNoallocMaxDevices) return CRM_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  NoallocDevice &d = g_noalloc[dev];
  if (!d.scratch) {
    void *ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, crm_noalloc_scratch) != cudaSuccess || !ptr) return CRM_ERR_CUDA;
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1)
      return CRM_ERR_CUDA;
    d.nsm = nsm;
    d.scratch = static_cast<unsigned char *>(ptr);
  }
  out = d;
  return CRM_OK;
}

}  // namespace

extern "C" int crm_run_device_noalloc(const crm_config *cfg, const crm_call_desc *d, const crm_input_c *in,
                                      crm_state_c *st, crm_rad_c *rad, crm_output_c *out, int *col_status,
                                      void *stream) {
  if (!cfg) return CRM_ERR_ARG;
  crm_config g = *cfg;
  g.max_ncrms = 1;   // no handle: the column count is bounded by the scratch only
  int rc = validate(&g);
  if (rc != CRM_OK) return rc;
  if (g.crm_ny > 1) return CRM_ERR_UNSUPPORTED;   // 2D only: the fixed tables hold one transform
  if (!d || d->ncrms < 1 || d->ld < d->ncrms || !(d->dt_gl > 0) || d->col_map) return CRM_ERR_ARG;
  if (g.batch_mode != CRM_PER_COLUMN) return CRM_ERR_UNSUPPORTED;
  const int ncrms = d->ncrms, nx = g.crm_nx;
  NoallocPlan q;
  rc = noalloc_plan(g, ncrms, q);
  if (rc != CRM_OK) return rc;
  if (!in || !st || !rad || !out || !col_status) return CRM_ERR_ARG;
  if (!d->gcol && d->igstep <= 1) return CRM_ERR_ARG;
  const double *need[] = {in->zmid, in->zint, in->tl, in->ql, in->qccl, in->qiil, in->pmid,
                          in->pint, in->pdel, in->ul, in->vl, in->tau00, in->bflxls, in->wndls};
  for (const double *x : need)
    if (!x) return CRM_ERR_ARG;
  double *sp[7] = {st->u_wind, st->v_wind, st->w_wind, st->temperature, st->qt, st->qp, st->qn};
  for (double *x : sp)
    if (!x) return CRM_ERR_ARG;
  double *rp[5] = {rad->temperature, rad->qv, rad->qc, rad->qi, rad->cld};
  if (!rad->qrad) return CRM_ERR_ARG;
  for (double *x : rp)
    if (!x) return CRM_ERR_ARG;
  for (int f = 0; f < CRM_NOUT; ++f)
    if (!out->field[f]) return CRM_ERR_ARG;
  const int nstop = (int)(d->dt_gl / g.crm_dt);   // crm_module.F90:712-713
  if (nstop < 1) return CRM_ERR_ARG;
  const double dt = d->dt_gl / nstop;
  if (60. < 2 * dt) return CRM_ERR_ARG;           // damping.F90:39-42
  const int nstop_run = accel_nstop(g, nstop);     // crm_module.F90:718-720
  if (nstop_run < 1) return CRM_ERR_ARG;

  NoallocDevice dv;
  rc = noalloc_device(dv);
  if (rc != CRM_OK) return rc;
  const int shape = default_shape(g.precision, nx);
  int per_sm = crm::occupancy_columns(g.precision, shape, nx, g.crm_nz);
  if (per_sm < 1) return CRM_ERR_UNSUPPORTED;
  int grid = dv.nsm * per_sm;
  if (grid > q.nslab) grid = q.nslab;

  // per-configuration constants (the same tables alloc_ctx builds), on the stack
  double consts[kNoallocMaxTrigs + CRM_NOALLOC_MAX_NX + 1 + (kNoallocMaxTrigs + 1) / 2];
  int ifax[20];
  fft_factors(ifax, nx);
  {
    fft_trigs_into(consts, nx);
    laplace_eigen(consts + q.ntrigs, g);
  }

  cudaStream_t s = (cudaStream_t)stream;
  unsigned char *base = dv.scratch;
  double *d_consts = reinterpret_cast<double *>(base);
  double *d_col = reinterpret_cast<double *>(base + q.const_bytes);
  void *d_slabs = base + q.const_bytes + q.col_bytes;
  {
    float *tf = reinterpret_cast<float *>(consts + q.ntrigs + q.neign);   // float copy of trigs
    for (int i = 0; i < q.ntrigs; ++i) tf[i] = (float)consts[i];
  }
  // uploaded as kernel parameters, so that the call can be captured into a
  // CUDA graph (the stack buffer is gone by the time a graph replays)
  crm::launch_crm_consts(d_consts, consts,
                         sizeof(double) * (size_t)(q.ntrigs + q.neign) + sizeof(float) * (size_t)q.ntrigs, s);

  crm::PrepParams pp;
  pp.ncrms = ncrms; pp.ld = d->ld; pp.plev = g.plev; pp.nx = nx; pp.igstep = d->igstep;
  pp.zmid = in->zmid; pp.zint = in->zint; pp.pdel = in->pdel;
  pp.tau00 = in->tau00; pp.bflxls = in->bflxls; pp.wndls = in->wndls;
  pp.gcol = d->gcol;
  pp.col_map = nullptr;
  pp.z0 = d_col;
  pp.rnd = d_col + ncrms;
  crm::KParams p;
  memset(&p, 0, sizeof p);
  p.L = q.L;
  p.ncrms = ncrms; p.ld = d->ld; p.nstop = nstop; p.igstep = d->igstep;
  p.batch_mode = g.batch_mode; p.clamp_batch = 0;
  p.nstop = nstop_run;
  p.use_accel = g.use_crm_accel != 0; p.accel_uv = g.crm_accel_uv != 0;
  p.accel_factor = g.crm_accel_factor;
  p.dx = g.crm_dx; p.dy = g.crm_dx; p.dt = dt; p.dt_gl = d->dt_gl;
  p.barrier_spins = 1ll << 24;
  p.barrier_withhold = -1;
  micro_consts(p);
  p.nfax = ifax[0];
  for (int k = 0; k <= ifax[0] && k < 8; ++k) p.ifax[k] = ifax[k];
  p.trigs = d_consts;
  p.trigs_f = reinterpret_cast<const float *>(d_consts + q.ntrigs + q.neign);
  p.eign = d_consts + q.ntrigs;
  p.z0 = pp.z0;
  p.rnd = pp.rnd;
  p.zmid = in->zmid; p.zint = in->zint; p.tl = in->tl; p.ql = in->ql; p.qccl = in->qccl;
  p.qiil = in->qiil; p.pmid = in->pmid; p.pint = in->pint; p.pdel = in->pdel;
  p.ul = in->ul; p.vl = in->vl;
  for (int f = 0; f < 7; ++f) p.st[f] = sp[f];
  p.qrad = rad->qrad;
  for (int f = 0; f < 5; ++f) p.radout[f] = rp[f];
  for (int f = 0; f < CRM_NOUT; ++f) p.out[f] = out->field[f];
  p.slabs = d_slabs;
  p.phase_cycles = nullptr;
  p.col_map = nullptr;
  p.col_status = col_status;
  crm::launch_crm_prep(pp, s);
  crm::launch_columns(g.precision, shape, p, grid, s);
  CK(cudaGetLastError());
  return CRM_OK;
}
