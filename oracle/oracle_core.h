// oracle_core.h -- data structures of the CPU FP64 restatement of crm().
//
// TEST INFRASTRUCTURE ONLY.  This restatement is the parity oracle for the
// GB300 library: only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline may load it.  Nothing in the product links or calls it.
//
// Layout: one Column struct holds every module-global array of the reference
// for one CRM instance (crm/vars.F90, grid.F90, microphysics.F90,
// SGS_TKE/sgs.F90), with the reference's index ranges including halos
// (crm/grid.F90:31-46, NADV = NADVS = 0).  The reference stores all columns
// in one array with the column index fastest; every per-column sum in the
// reference runs over (k, j, i) for a fixed column, so evaluating one column
// at a time reproduces the reference's CPU summation order exactly.
#pragma once
#include <vector>
#include <cstddef>
#include <cstdio>
#include <cstdlib>

namespace oracle {

// Fortran default-REAL literal promoted to double: the reference is built
// without -r8, so e.g. `0.61` in crm/setparm.F90:87 is (double)0.61f.
#define R4(x) ((double)(x##f))

struct A3 {
  std::vector<double> v;
  int x1 = 0, y1 = 0, z1 = 0, x2 = -1, y2 = -1, z2 = -1, nxa = 0, nya = 0;
  void init(int x1_, int x2_, int y1_, int y2_, int z1_, int z2_) {
    x1 = x1_; x2 = x2_; y1 = y1_; y2 = y2_; z1 = z1_; z2 = z2_;
    nxa = x2 - x1 + 1; nya = y2 - y1 + 1;
    v.assign((size_t)nxa * nya * (z2 - z1 + 1), 0.0);
  }
  inline double &operator()(int i, int j, int k) {
#ifdef ORACLE_CHECK
    if (i < x1 || i > x2 || j < y1 || j > y2 || k < z1 || k > z2) {
      fprintf(stderr, "oracle A3 index (%d,%d,%d) outside [%d:%d,%d:%d,%d:%d]\n",
              i, j, k, x1, x2, y1, y2, z1, z2);
      abort();
    }
#endif
    return v[((size_t)(k - z1) * nya + (j - y1)) * nxa + (i - x1)];
  }
  void zero() { std::fill(v.begin(), v.end(), 0.0); }
};

// 1-D profile with Fortran bounds lo..hi
struct A1 {
  std::vector<double> v;
  int lo = 0, hi = -1;
  void init(int lo_, int hi_) { lo = lo_; hi = hi_; v.assign(hi - lo + 1, 0.0); }
  inline double &operator()(int k) {
#ifdef ORACLE_CHECK
    if (k < lo || k > hi) {
      fprintf(stderr, "oracle A1 index %d outside [%d:%d]\n", k, lo, hi);
      abort();
    }
#endif
    return v[k - lo];
  }
  void zero() { std::fill(v.begin(), v.end(), 0.0); }
};

struct Grid {           // per-call constants shared by all columns
  int nx, ny, nzm, nz, YES3D, plev, nx_rad, ny_rad;
  double dx, dy, dt;    // dt after nstop = dt_gl/dt; dt = dt_gl/nstop
  int nstop;
  // FFT (crm/fft.F90): factors and float-rounded trig tables
  int ifaxi[20], ifaxj[20];
  std::vector<double> trigxi, trigxj;
  // pressure eigenvalues eign(i,j) (crm/pressure.F90:172-198)
  std::vector<double> eign;   // (nx+1) x (ny2 or 1)
  int eign_ni, eign_nj;
  // microphysics gamma-function constants (real*4) and fall-speed coefs
  double gam3, gamr1, gamr2, gamr3, gams1, gams2, gams3, gamg1, gamg2, gamg3;
  double vrain, vsnow, vgrau, crain, csnow, cgrau;
  double a_bg, a_pr, a_gr;
  int batch_mode;
  // mean-state acceleration (accelerate_crm.F90)
  bool use_accel, accel_uv;
  double accel_factor;
};

struct Column {
  // prognostic / diagnostic 3D fields (crm/vars.F90:180-200)
  A3 u, v, w, t, p, tabs, qv, qcl, qpl, qci, qpi;
  A3 qt, qp, qn;          // micro_field(:,:,:,:,1:2), qn (MICRO_SAM1MOM)
  A3 tke, tk, tkh;        // sgs_field(1), sgs_field_diag(1:2)
  A3 dudt[3], dvdt[3], dwdt[3];
  A3 precsfc, precssfc;   // (nx, ny, 1)
  // profiles
  A1 z, pres, zi, presi, adz, adzw, prespot, rho, rhow, bet, gamaz;
  A1 t0, q0, qv0, tabs0, u0, v0, tke0, qp0, qn0, t00;
  A1 ttend, qtend, utend, vtend, ug0, vg0, tg0, qg0;
  A1 grdf_x, grdf_y, grdf_z;
  A1 accrsc, accrsi, accrrc, coefice, accrgc, accrgi;
  A1 evaps1, evaps2, evapr1, evapr2, evapg1, evapg2;
  // statistics profiles (nz)
  A1 uwle, vwle, uwsb, vwsb, precflux, qpfall, tlat, tlatqi, qifall;
  A1 mkwle[2], mkwsb[2], mkadv[2], mkdiff[2], qpsrc, qpevp;
  double dz;
  double z0, ustar, bflx, wnd;
  // time stepping state (per column in per-column mode)
  int na, nb, nc, ncycle, icycle;
  double dt3[3], at, bt, ct, dtn, dtfactor;
  double cfl;              // last kurant cfl
  bool nonfinite = false;  // last kurant found a NaN/Inf in u, v, w or tkh
  double prec_cfl;
  int nprec;
  int status;
  int nstop;               // per column: grows if acceleration ceases
  int nstep;               // current CRM step
  bool ceaseflag;          // acceleration stopped for the rest of the call
  // per-call accumulators
  double colprec, colprecs;
  // per-step statistics (GCM levels 1..plev, interfaces 1..plev+1)
  A1 o_cld, o_cldtop, o_gicewp, o_gliqwp, o_mcup, o_mcdn, o_mcuup, o_mcudn;
  A1 mui, mdi;
  double cltot, clhgh, clmed, cllow;
  // per-step column scratch of the cloud statistics (nx*ny)
  std::vector<double> st_cwp, st_cwph, st_cwpm, st_cwpl, st_ct, st_ch, st_cm, st_cl;
  // crm_rad accumulators (nx_rad, ny_rad, nzm)
  A3 rad_t, rad_qv, rad_qc, rad_qi, rad_cld;
  A3 qrad;
};

}  // namespace oracle
