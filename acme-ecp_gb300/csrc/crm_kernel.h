// crm_kernel.h -- parameters of the column kernel (host <-> device).
#pragma once
#include "crm_layout.h"
#include "../../include/crm_gb300.h"

namespace crm {

struct KParams {
  Layout L;
  int ncrms, ld, nstop, igstep, batch_mode, clamp_batch;
  // mean-state acceleration (nstop above is already divided by 1 + factor)
  int use_accel, accel_uv;
  double accel_factor;
  double dx, dy, dt, dt_gl;
  // per-call constants computed on the host (gamma functions, fall speeds)
  double gams1, gams2, gamg1, gamg2, gamr1, gamr2;
  double vrain, vsnow, vgrau, crain, csnow, cgrau;
  double a_bg, a_pr, a_gr;
  int nfax;
  int ifax[8];
  const double *trigs;      // fft trig table (3n/2 + 2 + n), REAL*4 values
  const float *trigs_f;     // the same values as float (exact: they are REAL*4)
  const double *eign;       // (nx + 1) x (ny + 2) eigenvalues of the horizontal Laplacian (2D: ny + 2 -> 1)
  // the y transform of the 3D CRM (fft.F90 factors and REAL*4 trig table of ny)
  int nfax_y;
  int ifax_y[8];
  const double *trigs_y;
  const float *trigs_y_f;
  // 3D FP32-mixed form with nx = ny in {16, 32}: the transforms of the
  // pressure solve on the tensor cores (crm_tc.cuh); tc_n = nx, dft_tc the
  // forward ((n+2 rounded up to 16) x n) and inverse (n x (n+2 rounded up to
  // 8)) transform matrices, row-major; tc_n = 0: the warp FFT
  int tc_n;
  const float *dft_tc;
  const double *z0;         // (ncrms) roughness length
  const double *rnd;        // (ncrms, 5, nx) setperturb draws 1 - 2 r
  // crm_input (device, Fortran (ld, *) order)
  const double *zmid, *zint, *tl, *ql, *qccl, *qiil, *pmid, *pint, *pdel, *ul, *vl;
  // crm_state in/out (ld, nx, 1, nz): u, v, w, T, qt, qp, qn
  double *st[7];
  const double *qrad;       // (ld, nx_rad, 1, nz)
  double *radout[5];        // temperature, qv, qc, qi, cld
  double *out[CRM_NOUT];
  void *slabs;              // gridDim.x slabs of L.slab elements of T
  int *col_status;          // (ncrms)
  const int *col_map;       // optional (ncrms) slots: column c uses slot col_map[c]
  // reference-batch mode: grid barrier state [count, generation] (u32 x 2,
  // in gsync[0]) and a ring of four batch maxima gsync[2..5] (zeroed by the
  // host before the launch); all columns are co-resident CTAs
  unsigned long long *gsync;
  // spin iterations of one grid-barrier wait before it gives up (~4 s at the
  // default 2^24), and a test hook: the CTA integrating call position
  // barrier_withhold never arrives at the first barrier (-1: none), so the
  // others' waits run out and report CRM_ERR_TIMEOUT
  long long barrier_spins;
  int barrier_withhold;
  unsigned long long *phase_cycles;  // (gridDim.x, 64) when built with CRM_PHASE_TIMERS
};

// phase ids for the optional per-phase cycle counters
enum PhaseId {
  PH_INIT, PH_KURANT, PH_BUOY, PH_FORCING, PH_DAMPING, PH_ICEFALL, PH_BOUND, PH_TKE,
  PH_ADVMOM, PH_DIFFMOM, PH_PRESS_RHS, PH_FFT_FWD, PH_TRIDIAG, PH_FFT_INV, PH_PRESS_GRAD,
  PH_ADAMS, PH_ADV_T, PH_ADV_QT, PH_ADV_QP, PH_FALL1, PH_FALL2, PH_UVW, PH_DIFF_T,
  PH_DIFF_Q, PH_PINIT, PH_CLOUD, PH_PPROC, PH_MDIAG, PH_DIAG, PH_STATS, PH_FINAL, PH_COUNT
};

// Launch shapes of the column kernel: threads per CTA (one CTA integrates one
// CRM column at a time) and the CTAs per SM the register budget is sized for
// (__launch_bounds__).  More, smaller CTAs per SM hide more latency at the
// cost of register spills; the best shape is chosen per precision by
// measurement (crm_host.cu).
struct KShape {
  int threads, min_ctas;
  int smem_planes;   // scratch planes A and B in shared memory (0 or 2)
};
constexpr int kNumShapes = 6;
constexpr KShape kShapes[kNumShapes] = {{256, 3, 0}, {256, 4, 0}, {256, 4, 2}, {512, 2, 0}, {1024, 1, 0},
                                        {512, 2, 2}};

// Horizontal sizes with a kernel specialised at compile time (the reference
// fixes CRM_NX at build time too); any other power of two runs the generic
// kernel (NX = 0), which reads nx from the layout.
constexpr int kNumNx = 4;
constexpr int kNxBuilt[kNumNx] = {32, 64, 128, 0};

// Kernel variants, each its own instance: the plain forms; the 3D
// FP32-mixed form with the tensor-core transforms; the FP64 form compiled
// with multiply-add contraction (CRM_FP64_FMA).
constexpr int kVarPlain = 0, kVarTc = 1, kVarFma = 2;
// One instantiation per (T, NX, NY, shape, variant) lives in its own object
// (crm_columns.cu); NY = 1 is the 2D CRM, NY = 0 the generic 3D CRM.
template <typename T, int NX, int NY, int SHAPE, int VAR = kVarPlain>
void launch_crm_columns(const KParams &p, int grid, cudaStream_t s, bool cooperative);
template <typename T, int NX, int NY, int SHAPE, int VAR = kVarPlain>
int occupancy_crm_columns(int nx, int ny, int nzm, int tc_n);
// the launch shape of the tensor-core instance (1024 threads, one CTA per SM:
// a kernel with tcgen05 code is not co-resident with another CTA on GB300)
constexpr int kTcShape = 4;
// the launch shapes of the contracted FP64 instances: those of the plain
// FP64 form's defaults (2D: 256 threads x 3 CTAs/SM, 3D: 512 x 2)
constexpr int kFmaShape2d = 0, kFmaShape3d = 3;

// Dispatch on (precision, nx, ny, shape) at run time.
void launch_columns(int precision, int shape, const KParams &p, int grid, cudaStream_t s,
                    bool cooperative = false);
int occupancy_columns(int precision, int shape, int nx, int nzm, int ny = 1, int tc_n = 0);

}  // namespace crm
