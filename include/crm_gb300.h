/*
 * crm_gb300.h -- C ABI of the GB300-native superparameterized CRM step.
 *
 * One call advances ncrms embedded 2D or 3D cloud-resolving models (one per
 * GCM column) over one GCM timestep dt_gl, exactly like the Fortran entry
 *
 *   subroutine crm(lchnk, icol, ncrms, dt_gl, plev, crm_input, crm_state,
 *                  crm_rad, crm_ecpp_output, crm_output)
 *
 * in components/cam/src/physics/crm/crm_module.F90:45-56 (default build:
 * sam1mom microphysics, SGS_TKE closure, MPDATA scalar advection, no CLUBB,
 * no MAML, no ECPP), called from crm_physics_tend in
 * components/cam/src/physics/cam/crm_physics.F90:1145-1156.
 *
 * Array convention: every array argument is a plain pointer to host memory
 * laid out in Fortran (column-major) order with the CRM column index fastest,
 * exactly as the derived types of the reference hold them:
 *   (ld, plev)              crm_input_module.F90:10-47
 *   (ld, nx, ny, nz)        crm_state_module.F90:12-56, crm_output_module.F90
 *   (ld, nx_rad, ny_rad, nz) crm_rad_module.F90:17-34
 * where ld (= pcols in CAM) >= ncrms and only columns 0..ncrms-1 are touched
 * (crm_module.F90:268-281).  nz here is crm_nz (the number of CRM scalar
 * levels, nzm in the reference grid module).
 *
 * Errors are returned, never raised: every entry point returns a crm_status
 * and the per-column status array (optional) receives one code per column.
 * The reference stops the model instead (endrun / task_abort), e.g.
 * kurant.F90:66-75 when ncycle exceeds 16.
 */
#ifndef CRM_GB300_H
#define CRM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
enum crm_status {
  CRM_OK = 0,
  CRM_ERR_ARG = 1,          /* bad argument / unsupported configuration     */
  CRM_ERR_CFL = 2,          /* kurant(): ncycle > 16 (kurant.F90:66-75)     */
  CRM_ERR_NONFINITE = 3,    /* a state field became NaN/Inf                  */
  CRM_ERR_CUDA = 4,         /* CUDA runtime error                            */
  CRM_ERR_UNSUPPORTED = 5,  /* feature not built (e.g. m2005)                */
  CRM_ERR_TIMEOUT = 6,      /* a bounded device wait gave up                 */
  CRM_ERR_BUDGET = 7,       /* serving admission: HBM budget exhausted       */
  CRM_ERR_NO_DEVICE = 8,    /* no CUDA device                                */
  CRM_ERR_TOO_LARGE = 9,    /* exceeds crm_run_device_noalloc's fixed scratch */
  CRM_PENDING = 10          /* crm_poll: the step has not completed yet      */
};

enum crm_microphysics { CRM_MICRO_SAM1MOM = 0, CRM_MICRO_M2005 = 1 };
/* CRM_FP64: every multiply and add separately rounded, bit-identical to the
 * CPU restatement; CRM_FP32_MIXED: FP32 fields and bulk arithmetic, FP64 for
 * the pressure tridiagonal solve, the conservation sums and the saturation
 * Newton iteration, every GCM tendency within 1e-4 relative L2 of CRM_FP64
 * after a GCM step; CRM_FP64_FMA: FP64 with multiply-add contraction (within
 * 1e-11 relative L2 of CRM_FP64 after a GCM step, 12-14 % faster: GB300's FP64
 * pipe is the bound of the FP64 form). */
enum crm_precision { CRM_FP64 = 0, CRM_FP32_MIXED = 1, CRM_FP64_FMA = 2 };
/* Subcycle count ncycle (kurant.F90:54-64) and precipitation sub-steps nprec
 * (MICRO_SAM1MOM/microphysics.F90:602-661) are batch maxima in the
 * reference, the first-step velocity clamp tests only the first column
 * (crm_module.F90:400-417) and the acceleration cease flag is batch-wide
 * (accelerate_crm.F90:236).  CRM_PER_COLUMN makes each column independent of
 * its batch-mates; CRM_REFERENCE_BATCH reproduces the batch coupling: all
 * columns of the call run at once (ncrms at most the GPU's co-resident
 * columns, no col_map; else CRM_ERR_UNSUPPORTED). */
enum crm_batch_mode { CRM_PER_COLUMN = 0, CRM_REFERENCE_BATCH = 1 };

/* Compile-time CPP constants of the reference (bld/configure:1883-1914,
 * crmdims.F90, domain.F90), passed at run time.
 *
 * Built: crm_nx a power of two >= 8 (the device transform takes factors 2
 * and 4); crm_ny = 1 (2D; crm_ny_rad = 1, crm_dy unused: dy = dx) or crm_ny
 * a power of two >= 8 (3D; crm_dy > 0, or 0 for dy = dx), the 3D CRM with
 * radiation on every CRM column (crm_nx_rad = crm_nx, crm_ny_rad = crm_ny).
 * Other transform lengths and coarser 3D radiation groups give
 * CRM_ERR_UNSUPPORTED. */
typedef struct crm_config {
  int crm_nx, crm_ny, crm_nz;   /* CRM_NX, CRM_NY, CRM_NZ (ny == 1: 2D)  */
  int crm_nx_rad, crm_ny_rad;   /* radiation column groups               */
  int plev;                     /* GCM levels (pver)                     */
  double crm_dx, crm_dy;        /* CRM_DX, CRM_DY [m]                    */
  double crm_dt;                /* CRM_DT [s]                            */
  int microphysics;             /* enum crm_microphysics                 */
  int precision;                /* enum crm_precision                    */
  int batch_mode;               /* enum crm_batch_mode                   */
  int max_ncrms;                /* largest ncrms a handle will be given  */
  /* Mean-state acceleration (accelerate_crm.F90; Jones et al. 2015), the
   * use_crm_accel / crm_accel_factor / crm_accel_uv namelist options: the
   * horizontal-mean tendency of t and qt (and u, v) is applied
   * crm_accel_factor extra times after each microphysics call and nstop is
   * divided by 1 + crm_accel_factor, which must divide it. */
  int use_crm_accel;
  double crm_accel_factor;
  int crm_accel_uv;
} crm_config;

/* crm_input_type (crm_input_module.F90:10-47); (ld, plev) unless noted. */
typedef struct crm_input_c {
  const double *zmid, *zint;    /* zint: (ld, plev+1)                    */
  const double *tl, *ql, *qccl, *qiil;
  const double *ps;             /* (ld)                                  */
  const double *pmid, *pint, *pdel;  /* pint: (ld, plev+1)               */
  const double *phis;           /* (ld)                                  */
  const double *ul, *vl;
  const double *ocnfrac, *tau00, *wndls, *bflxls;   /* (ld)              */
  const double *fluxu00, *fluxv00, *fluxt00, *fluxq00; /* (ld)           */
} crm_input_c;

/* crm_state_type (crm_state_module.F90:12-56): (ld, nx, ny, nz), in/out. */
typedef struct crm_state_c {
  double *u_wind, *v_wind, *w_wind, *temperature;
  double *qt, *qp, *qn;          /* sam1mom prognostics                   */
} crm_state_c;

/* crm_rad_type (crm_rad_module.F90:17-34): (ld, nx_rad, ny_rad, nz).
 * qrad is read; the others are written (time means over the call). */
typedef struct crm_rad_c {
  double *qrad, *temperature, *qv, *qc, *qi, *cld;
} crm_rad_c;

/* crm_output_type (crm_output_module.F90:7-133), sam1mom subset.  Shapes:
 * 4D = (ld,nx,ny,nz), 3D = (ld,nx,ny), 2D = (ld,plev), 1D = (ld). */
enum crm_output_field {
  /* 4D */
  CRM_OUT_QCL, CRM_OUT_QCI, CRM_OUT_QPL, CRM_OUT_QPI, CRM_OUT_TK, CRM_OUT_TKH,
  /* 3D */
  CRM_OUT_PREC_CRM,
  /* 1D */
  CRM_OUT_CLTOT, CRM_OUT_CLHGH, CRM_OUT_CLMED, CRM_OUT_CLLOW,
  CRM_OUT_PRECC, CRM_OUT_PRECL, CRM_OUT_PRECSC, CRM_OUT_PRECSL,
  CRM_OUT_JT_CRM, CRM_OUT_MX_CRM, CRM_OUT_PRECTEND, CRM_OUT_PRECSTEND,
  CRM_OUT_TAUX, CRM_OUT_TAUY, CRM_OUT_Z0M, CRM_OUT_TIMING_FACTOR,
  /* 2D */
  CRM_OUT_CLDTOP, CRM_OUT_QC_MEAN, CRM_OUT_QI_MEAN, CRM_OUT_QS_MEAN,
  CRM_OUT_QG_MEAN, CRM_OUT_QR_MEAN,
  CRM_OUT_SLTEND, CRM_OUT_QLTEND, CRM_OUT_QCLTEND, CRM_OUT_QILTEND,
  CRM_OUT_CLD, CRM_OUT_GICEWP, CRM_OUT_GLIQWP, CRM_OUT_MCTOT, CRM_OUT_MCUP,
  CRM_OUT_MCDN, CRM_OUT_MCUUP, CRM_OUT_MCUDN, CRM_OUT_MU_CRM, CRM_OUT_MD_CRM,
  CRM_OUT_DU_CRM, CRM_OUT_EU_CRM, CRM_OUT_ED_CRM,
  CRM_OUT_FLUX_QT, CRM_OUT_FLUXSGS_QT, CRM_OUT_TKEZ, CRM_OUT_TKESGSZ,
  CRM_OUT_TKZ, CRM_OUT_FLUX_U, CRM_OUT_FLUX_V, CRM_OUT_FLUX_QP,
  CRM_OUT_PRECFLUX, CRM_OUT_QT_LS, CRM_OUT_QT_TRANS, CRM_OUT_QP_TRANS,
  CRM_OUT_QP_FALL, CRM_OUT_QP_SRC, CRM_OUT_QP_EVP, CRM_OUT_T_LS,
  CRM_NOUT
};
#define CRM_OUT_FIRST_3D CRM_OUT_PREC_CRM
#define CRM_OUT_FIRST_1D CRM_OUT_CLTOT
#define CRM_OUT_FIRST_2D CRM_OUT_CLDTOP

typedef struct crm_output_c {
  double *field[CRM_NOUT];      /* indexed by enum crm_output_field      */
} crm_output_c;

/* Hidden inputs of crm() made explicit (crm_module.F90:33,286-291,679):
 * get_gcol_p (random seed = gcol*1000), get_nstep (setperturb when
 * igstep <= 1), get_rlat_p/get_rlon_p (only feed the Coriolis terms, which
 * are off: docoriolis = .false.). */
typedef struct crm_call_desc {
  int lchnk;
  int ncrms;                    /* columns in this call                  */
  int ld;                       /* leading dimension (pcols) of arrays   */
  double dt_gl;                 /* GCM timestep [s]                      */
  int igstep;                   /* GCM step number (get_nstep())        */
  const int *gcol;              /* (ncrms) global column ids             */
  /* Optional (ncrms) column slots, 0-based and distinct, < ld: column c of
   * the call reads and writes slot col_map[c] of every (ld, ...) array, so a
   * caller can integrate any subset of a resident batch; col_status and gcol
   * stay indexed by c.  NULL: slot c.  A device pointer for crm_run_device,
   * host for crm_run; not accepted by crm_run_device_noalloc.  No
   * counterpart in the reference (ncrms always covers 1..ncrms). */
  const int *col_map;
} crm_call_desc;

typedef struct crm_ctx crm_ctx;

/* Create a handle for one (nx, ny, nz, dx, dt, microphysics, precision)
 * configuration on the current CUDA device.  Replaces the CPP build-time
 * specialisation (crmdims.F90) and the per-call allocate_* of the module
 * globals (crm_module.F90:199-266).  Returns NULL and sets *status on error. */
crm_ctx *crm_create(const crm_config *cfg, int *status);
void crm_destroy(crm_ctx *ctx);

/* The drop-in for subroutine crm() (crm_module.F90:45-1718): host arrays in,
 * host arrays out; state and rad updated in place.  col_status (ncrms, may be
 * NULL) receives a crm_status per column.  Synchronous. */
int crm_run(crm_ctx *ctx, const crm_call_desc *desc, const crm_input_c *in,
            crm_state_c *state, crm_rad_c *rad, crm_output_c *out,
            int *col_status);

/* Device-resident variant of crm_run: every array pointer in desc (gcol),
 * in, state, rad and out is a device pointer with the same layout, and
 * col_status (ncrms ints) is a device pointer or NULL.  The work is enqueued
 * on `stream` (a cudaStream_t, NULL for the handle's stream) and the call
 * returns without synchronising; argument errors are returned at once.  This
 * is the path a GCM that keeps its physics state on the GPU would call.  The
 * enqueued work is kernel launches and event records only (plus a memset in
 * reference-batch mode), so a call can be captured into a CUDA graph and the
 * graph replayed; crm_last_kernel_ms is not defined for a captured call. */
int crm_run_device(crm_ctx *ctx, const crm_call_desc *desc, const crm_input_c *in,
                   crm_state_c *state, crm_rad_c *rad, crm_output_c *out,
                   int *col_status, void *stream);

/* Size of the fixed device scratch used by crm_run_device_noalloc [bytes]. */
#define CRM_NOALLOC_SCRATCH_BYTES (32u << 20)
#define CRM_NOALLOC_MAX_NX 1024

/* crm_run_device without a handle and without any device allocation.  No
 * counterpart in the reference (its crm() allocates the module arrays on
 * every call, crm_module.F90:199-266).
 *
 * For callers that cannot allocate device memory at the point of the call:
 * a host model whose own pool allocator has reserved the GPU's memory up
 * front (so a cudaMalloc here would fail or fragment that pool), or a time
 * step loop that must not pay the implicit device-wide synchronisation that
 * cudaMalloc/cudaFree can cause while other streams are busy.
 *
 * Arguments are those of crm_run_device with the configuration in place of
 * the handle: every array pointer is a device pointer, col_status (ncrms ints,
 * device) is required, and the work is enqueued on `stream` (NULL: the legacy
 * default stream) without synchronising.  cfg->max_ncrms is ignored.
 *
 * Scratch: one static device array of CRM_NOALLOC_SCRATCH_BYTES (32 MiB) in
 * the library, holding the per-configuration constants (FP64 trig tables and
 * Laplacian eigenvalues), the per-column set-up values (8 * (1 + 5 * nx)
 * bytes per column) and as many per-column working slabs as fit; the column
 * kernel then runs with that many CTAs (fewer than crm_run_device uses, so
 * it is slower).  A call whose constants, per-column values and one slab do
 * not fit, or with crm_nx > CRM_NOALLOC_MAX_NX, returns CRM_ERR_TOO_LARGE
 * before touching the device.  The 3D CRM (crm_ny > 1) is taken by the
 * handle entry points only: here it returns CRM_ERR_UNSUPPORTED.
 *
 * The array is part of the library's device code, so every device on which
 * the library's kernels are loaded holds these 32 MiB until the process exits,
 * whether or not this entry point is ever called.
 *
 * The array's device address is looked up once per device, by the first call
 * made with that device current; make that first call before any stream
 * capture begins.  The address is kept for the life of the process: it
 * assumes the device's primary context is never reset (cudaDeviceReset) and
 * that calls come from that primary context.  Every device operation of a call is a kernel launch on
 * `stream` (the per-configuration constants travel as kernel parameters), so
 * later calls can be captured into a CUDA graph and replayed.  Every call on a device shares the one array and leaves its
 * last contents behind; nothing in it needs to start at zero (the kernel
 * clears a column's slab when it starts the column, and the set-up values and
 * constants are rewritten by every call).  Calls that overlap in time on the
 * same device (different streams or host threads) race on the array: order
 * them on one stream. */
int crm_run_device_noalloc(const crm_config *cfg, const crm_call_desc *desc,
                           const crm_input_c *in, crm_state_c *state, crm_rad_c *rad,
                           crm_output_c *out, int *col_status, void *stream);

/* Handle services with no counterpart in the reference (its crm() runs on
 * the calling thread with no stream, timer or status API; errors go to
 * endrun, e.g. kurant.F90:66-75). */

/* Number of kernel launches issued by the last crm_run on this handle. */
int crm_last_launch_count(const crm_ctx *ctx);
/* Duration of the compute kernels of the last crm_run [ms] (CUDA events on
 * the handle's stream), excluding host<->device copies. */
double crm_last_kernel_ms(const crm_ctx *ctx);
/* Bind the handle to a CUDA stream (cudaStream_t passed as void*). */
int crm_set_stream(crm_ctx *ctx, void *stream);
/* Text of a crm_status (what the reference would have passed to endrun). */
const char *crm_status_string(int status);
/* Per-phase cycle counters of the column kernel, summed over its CTAs since
 * the last read, in a profiling build of the library (compiled with
 * -DCRM_PHASE_TIMERS); returns the number of phases written, or -1 in a
 * normal build.  No counterpart in the reference (its GPTL timers
 * t_startf/t_stopf time the whole CRM call, crm_module.F90:377,1598). */
int crm_debug_phase_cycles(crm_ctx *ctx, unsigned long long *out, int n);
/* Launch shapes of the column kernel (threads per CTA, CTAs per SM the
 * register budget is sized for, scratch planes in shared memory): the search
 * space of an autotuner (crm_gb300/autotune.py).  FP64 results do not
 * depend on the shape; FP32-mixed results agree to FP32 rounding.  No
 * counterpart in the reference (its OpenACC schedule is the compiler's).  By default a handle chooses per call: the shape with the
 * most threads per column among those that hold the whole call at once
 * (latency), else the measured throughput default.  crm_set_launch_shape
 * fixes one for later calls (-1: back to the per-call choice); CRM_ERR_ARG
 * when out of range or not launchable for this configuration. */
int crm_num_launch_shapes(void);
int crm_launch_shape_info(int shape, int *threads, int *ctas_per_sm, int *smem_planes);
int crm_set_launch_shape(crm_ctx *ctx, int shape);
int crm_get_launch_shape(const crm_ctx *ctx);
/* Test hook of the reference-batch grid barrier (no counterpart in the
 * reference): every wait at the barrier gives up after spin_limit polls
 * (default 2^24, about 4 s) and the column then reports CRM_ERR_TIMEOUT;
 * withhold_column >= 0 makes the column at that call position skip its
 * arrival at the first barrier, so the other columns' waits run out.  Lets a
 * test drive the timeout path without a GPU fault; -1 restores normal
 * arrivals.  Applies to later calls on the handle. */
int crm_debug_barrier_test(crm_ctx *ctx, long long spin_limit, int withhold_column);
/* Device memory a handle holds [bytes]: its column slabs, per-column set-up
 * values and constants from crm_create on, plus the staging buffers of host
 * arguments from its first crm_run on (a handle driven only through
 * crm_run_device never allocates those).  crm_plan_device_bytes gives what
 * crm_create would allocate for cfg without allocating anything, so a
 * serving loop can admit a new configuration against an HBM budget before
 * it creates the handle.  No counterpart in the reference (its crm()
 * allocates and frees the module arrays on every call,
 * crm_module.F90:199-266,1666-1716). */
unsigned long long crm_device_bytes(const crm_ctx *ctx);
int crm_plan_device_bytes(const crm_config *cfg, unsigned long long *bytes);
/* ------------------------------------------------------------ serving
 * Continuous batching for C and Fortran hosts.  No counterpart in the
 * reference, which integrates each chunk synchronously inside
 * crm_physics_tend (cam/crm_physics.F90:1145-1156) and keeps each column's
 * CRM state in the physics buffer between GCM steps (crm_physics.F90:126-191,
 * pbuf 'global' fields).  A server keeps that state on the device: a pool of
 * `capacity` column slots of one configuration and `nhandles` column-kernel
 * handles with their own streams.  A chunk of GCM columns is admitted into
 * free slots (crm_chunk_open copies its CRM state in); each GCM step of a
 * chunk is a request (crm_submit) carrying only the chunk's new input
 * profiles.  An engine thread gathers the waiting requests, at most one per
 * chunk (a chunk's next step waits for its current one) and all of one
 * (dt_gl, first-step) kind, and runs ONE column-kernel launch over the union
 * of their slots on an idle handle; requests that arrive meanwhile join the
 * next launch, and launches on different handles overlap on the device.
 * Per-column mode (the only mode served) makes a chunk's results the same
 * alone and in any mix.  All calls are thread-safe. */
typedef struct crm_server crm_server;

/* hbm_budget_bytes bounds the device memory the server holds (slot arrays,
 * handles, staging): a configuration that does not fit gets NULL and
 * *status = CRM_ERR_BUDGET before anything is allocated.  cfg->max_ncrms
 * is ignored (capacity takes its place); batch_mode must be
 * CRM_PER_COLUMN. */
crm_server *crm_server_create(const crm_config *cfg, int capacity, int nhandles,
                              unsigned long long hbm_budget_bytes, int *status);
/* Stops the engine after the launches in flight; requests not yet
 * launched are dropped. */
void crm_server_destroy(crm_server *srv);
/* Device bytes the server holds; launches it has issued. */
unsigned long long crm_server_device_bytes(const crm_server *srv);
long long crm_server_launches(const crm_server *srv);

/* Admit ncols GCM columns whose CRM state is columns 0..ncols-1 of host
 * arrays of leading dimension ld (crm_state_c, and rad->qrad; the other rad
 * pointers are not read); gcol: their global column ids (the setperturb seed
 * of their first step).  *chunk receives the chunk id.  CRM_ERR_BUDGET when
 * fewer than ncols slots are free (retry after closing chunks). */
int crm_chunk_open(crm_server *srv, int ncols, const int *gcol, int ld, const crm_state_c *st,
                   const crm_rad_c *rad, int *chunk);
/* Copy a chunk's resident CRM state (and, if qrad is not NULL, its
 * radiative heating) to host arrays of leading dimension ld, e.g. for a
 * restart file; CRM_ERR_ARG while a step of the chunk is queued. */
int crm_chunk_read_state(crm_server *srv, int chunk, int ld, crm_state_c *st, double *qrad);
/* Release a chunk's slots; CRM_ERR_ARG while a step of it is queued. */
int crm_chunk_close(crm_server *srv, int chunk);

/* Submit one GCM step of a chunk: `in` holds its new GCM input profiles as
 * host arrays of leading dimension ld (columns 0..ncols-1; the fields
 * crm_run reads), qrad (may be NULL: keep the resident heating) its new
 * radiative heating (ld, nx_rad, ny_rad, nz).  The results are written, when
 * the step completes, into the caller's host arrays: every non-NULL field of
 * `out` (ld, ...), the non-NULL rad means of `rad_means` (its qrad is not
 * used) and col_status (ncols; may be NULL).  Those arrays must stay valid
 * until crm_poll reports completion.  Returns at once with a ticket.  The
 * first step of a chunk runs setperturb (igstep 1). */
int crm_submit(crm_server *srv, int chunk, const crm_input_c *in, const double *qrad, int ld,
               double dt_gl, crm_output_c *out, crm_rad_c *rad_means, int *col_status,
               long long *ticket);
/* CRM_PENDING while the step runs (wait = 0), else the step's worst column
 * status once its results are in the caller's arrays (wait != 0 blocks until
 * then).  A completed ticket is released by the call that reports it. */
int crm_poll(crm_server *srv, long long ticket, int wait);

/* The 3D pressure solve's x/y transforms on the tensor cores (the FP32-mixed
 * form's path for crm_nx = crm_ny in {16, 32}), on their own: one CTA
 * transforms nlev levels of ff, each (n + 2) x (n + 2) floats, x fastest, in
 * the layout of the solve: dir = -1 forward (rows j = 1..n, columns i = 1..n
 * of each level in; the fft991 coefficients of the 2D real transform out in
 * columns 1..n+1, rows 1..n+2), dir = +1 inverse (back to rows and columns
 * 1..n).  Host arrays; for tests. */
int crm_debug_tc_transform(int n, int nlev, int dir, const float *in, float *out);

/* Library version string. */
const char *crm_version(void);

#ifdef __cplusplus
}
#endif
#endif /* CRM_GB300_H */
