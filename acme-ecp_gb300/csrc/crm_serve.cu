// crm_serve.cu -- the continuous-batching service of include/crm_gb300.h
// (crm_server_create, crm_chunk_open/close/read_state, crm_submit,
// crm_poll) for C and Fortran hosts.
//
// The reference integrates each GCM chunk synchronously inside
// crm_physics_tend (cam/crm_physics.F90:1145-1156) and keeps every column's
// CRM state in the physics buffer between GCM steps (crm_physics.F90:126-191).
// The service keeps that state on the device instead: one pool of column
// slots per server (arrays of leading dimension `capacity`, the slot index
// fastest, exactly the (ld, ...) layout crm_run_device reads), and a set of
// column-kernel handles, each with its own stream.  A chunk is admitted into
// free slots; each step request carries only the chunk's new GCM input
// profiles.  One engine thread owns every device operation: it gathers the
// waiting requests, takes at most one per chunk (a chunk's later step
// depends on the earlier one and would integrate the same slots) and all of
// one (dt_gl, first-step) kind, scatters their inputs into the slots, runs
// ONE column-kernel launch over the union of their slots (crm_run_device with
// a col_map) on an idle handle, gathers the requested outputs, and completes
// each request when its launch's event has passed.  Requests that arrive
// while launches run join the next launch; launches on different handles
// overlap on the device.  Per-column mode makes a chunk's results the same
// alone and in any mix.
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/crm_gb300.h"

namespace {

constexpr int kMaxCopyFields = 80;

// Copy of `nf` fields between the slot arrays (ld, rows) and a packed buffer
// (n, rows), column index fastest in both: packed(c, r) <-> slot(slots[c], r).
struct SlotCopy {
  int nf, n, ld, to_slots;
  const int *slots;
  double *slot_arr[kMaxCopyFields];
  double *packed[kMaxCopyFields];
  int rows[kMaxCopyFields];
};

__global__ void slot_copy_kernel(const __grid_constant__ SlotCopy c) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (int f = 0; f < c.nf; ++f) {
    const size_t tot = (size_t)c.rows[f] * c.n;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += stride) {
      const size_t r = e / c.n, col = e % c.n;
      double *s = c.slot_arr[f] + (size_t)c.slots[col] + (size_t)c.ld * r;
      double *p = c.packed[f] + e;
      if (c.to_slots) *s = *p;
      else *p = *s;
    }
  }
}

enum InField { I_ZMID, I_ZINT, I_TL, I_QL, I_QCCL, I_QIIL, I_PMID, I_PINT, I_PDEL, I_UL, I_VL,
               I_TAU00, I_BFLXLS, I_WNDLS, I_NIN };

struct Request {
  long long ticket = 0;
  int chunk = -1;
  std::vector<int> slots, gcol;    // the chunk's, copied when the launch is chosen
  double dt_gl = 0.;
  bool first = false;
  std::vector<double> in;          // packed inputs of this chunk's columns (ncols, in_rows)
  bool has_qrad = false;
  std::vector<double> qrad;        // packed new radiative heating (ncols, nxr*nz), optional
  crm_output_c out{};              // caller's host arrays (ld, ...); NULL fields are not returned
  crm_rad_c rad{};                 // caller's rad means (temperature .. cld), optional
  int *col_status = nullptr;       // caller's (ncols) status, optional
  int ld = 0;
  int done = 0;                    // 0 pending, 1 launched, 2 complete
  int status = CRM_OK;
};

struct ChunkRec {
  std::vector<int> slots, gcol;
  int steps = 0;
  bool open = false;
  bool busy = false;               // a step in flight
  int queued = 0;                  // requests not yet complete
};

struct Handle {
  crm_ctx *ctx = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  bool busy = false;
  // device staging
  int *d_map = nullptr, *d_gcol = nullptr, *d_status = nullptr;
  double *d_in = nullptr;          // (capacity, in_rows)
  double *d_q = nullptr;           // (capacity, rad rows): new radiative heating
  double *d_out = nullptr;         // (capacity, out rows of the launch), grown on demand
  size_t out_cap = 0;              // doubles
  // pinned host staging
  double *h_in = nullptr, *h_out = nullptr, *h_q = nullptr;
  int *h_map = nullptr, *h_gcol = nullptr, *h_status = nullptr;
  size_t h_out_cap = 0;
  // the launch in flight
  std::vector<Request *> reqs;
  std::vector<int> fields;         // output field ids gathered (CRM_NOUT + 0..4: rad means)
  int n = 0;
};

}  // namespace

struct crm_server {
  crm_config cfg;
  int device = 0, capacity = 0;
  unsigned long long budget = 0;
  // pool arrays (device), leading dimension capacity
  double *in_arr[I_NIN] = {};
  double *state[7] = {};
  double *rad[6] = {};               // qrad, temperature, qv, qc, qi, cld
  double *out[CRM_NOUT] = {};
  std::vector<Handle> handles;
  cudaStream_t io_stream = nullptr;  // chunk state in/out
  std::vector<int> free_slots;
  std::map<int, ChunkRec> chunks;
  int next_chunk = 0;
  long long next_ticket = 1;
  std::deque<Request *> pending;
  std::map<long long, std::unique_ptr<Request>> requests;
  std::mutex mu;
  std::condition_variable cv;
  std::thread engine;
  bool stop = false;
  std::atomic<long long> launches{0};
  std::atomic<unsigned long long> used_bytes{0};   // device bytes held (grows with output staging)

  size_t in_rows(int f) const {
    if (f == I_ZINT || f == I_PINT) return (size_t)cfg.plev + 1;
    if (f >= I_TAU00) return 1;
    return (size_t)cfg.plev;
  }
  size_t in_rows_total() const {
    size_t r = 0;
    for (int f = 0; f < I_NIN; ++f) r += in_rows(f);
    return r;
  }
  size_t out_rows(int f) const {   // f < CRM_NOUT: crm_output; CRM_NOUT + 0..4: rad means
    if (f >= CRM_NOUT) return (size_t)cfg.crm_nx_rad * cfg.crm_ny_rad * cfg.crm_nz;
    if (f < CRM_OUT_FIRST_3D) return (size_t)cfg.crm_nx * cfg.crm_ny * cfg.crm_nz;
    if (f < CRM_OUT_FIRST_1D) return (size_t)cfg.crm_nx * cfg.crm_ny;
    if (f < CRM_OUT_FIRST_2D) return 1;
    return (size_t)cfg.plev;
  }
  size_t state_rows() const { return (size_t)cfg.crm_nx * cfg.crm_ny * cfg.crm_nz; }
  size_t rad_rows() const { return (size_t)cfg.crm_nx_rad * cfg.crm_ny_rad * cfg.crm_nz; }
  size_t pool_doubles() const {
    size_t r = in_rows_total() + 7 * state_rows() + 6 * rad_rows();
    for (int f = 0; f < CRM_NOUT; ++f) r += out_rows(f);
    return r * (size_t)capacity;
  }
};

namespace {

int copy_slots(crm_server *s, cudaStream_t st, int n, const int *d_slots, bool to_slots,
               const std::vector<double *> &slot_arr, const std::vector<double *> &packed,
               const std::vector<int> &rows) {
  for (size_t f0 = 0; f0 < slot_arr.size(); f0 += kMaxCopyFields) {
    SlotCopy c;
    memset(&c, 0, sizeof c);
    c.n = n; c.ld = s->capacity; c.to_slots = to_slots ? 1 : 0; c.slots = d_slots;
    for (size_t f = f0; f < slot_arr.size() && f < f0 + kMaxCopyFields; ++f) {
      c.slot_arr[c.nf] = slot_arr[f];
      c.packed[c.nf] = packed[f];
      c.rows[c.nf] = rows[f];
      ++c.nf;
    }
    slot_copy_kernel<<<4 * 152, 256, 0, st>>>(c);
  }
  return cudaGetLastError() == cudaSuccess ? CRM_OK : CRM_ERR_CUDA;
}

// Columns 0..n-1 of caller arrays with leading dimension ld -> packed (n, rows).
void pack(const double *src, int ld, int n, size_t rows, double *dst) {
  for (size_t r = 0; r < rows; ++r) memcpy(dst + r * n, src + r * (size_t)ld, sizeof(double) * n);
}
void unpack(const double *src, int n_tot, int off, int n, size_t rows, double *dst, int ld) {
  for (size_t r = 0; r < rows; ++r) memcpy(dst + r * (size_t)ld, src + r * (size_t)n_tot + off, sizeof(double) * n);
}

void free_handle(Handle &h) {
  if (h.ctx) crm_destroy(h.ctx);
  if (h.stream) cudaStreamDestroy(h.stream);
  if (h.done) cudaEventDestroy(h.done);
  cudaFree(h.d_map); cudaFree(h.d_gcol); cudaFree(h.d_status); cudaFree(h.d_in); cudaFree(h.d_out);
  cudaFree(h.d_q);
  cudaFreeHost(h.h_in); cudaFreeHost(h.h_out); cudaFreeHost(h.h_map); cudaFreeHost(h.h_gcol);
  cudaFreeHost(h.h_q);
  cudaFreeHost(h.h_status);
  h = Handle();
}

// Issue one launch for `reqs` on handle h (engine thread, lock not held).
int issue(crm_server *s, Handle &h) {
  int n = 0;
  for (Request *r : h.reqs) n += (int)r->slots.size();
  h.n = n;
  // output fields: the union of what the requests asked for
  std::vector<char> want(CRM_NOUT + 5, 0);
  for (Request *r : h.reqs) {
    for (int f = 0; f < CRM_NOUT; ++f)
      if (r->out.field[f]) want[f] = 1;
    double *rp[5] = {r->rad.temperature, r->rad.qv, r->rad.qc, r->rad.qi, r->rad.cld};
    for (int f = 0; f < 5; ++f)
      if (rp[f]) want[CRM_NOUT + f] = 1;
  }
  h.fields.clear();
  size_t orows = 0;
  for (int f = 0; f < CRM_NOUT + 5; ++f)
    if (want[f]) { h.fields.push_back(f); orows += s->out_rows(f); }
  const size_t need = orows * (size_t)n;
  if (need > h.out_cap) {
    // output staging grows to the largest launch seen, within the budget
    const unsigned long long extra = sizeof(double) * (unsigned long long)(need - h.out_cap);
    if (s->used_bytes.load() + extra > s->budget) return CRM_ERR_BUDGET;
    s->used_bytes += extra;
    cudaFree(h.d_out);
    cudaFreeHost(h.h_out);
    h.d_out = nullptr; h.h_out = nullptr; h.out_cap = 0;
    if (cudaMalloc(&h.d_out, sizeof(double) * need) != cudaSuccess) return CRM_ERR_CUDA;
    if (cudaMallocHost(&h.h_out, sizeof(double) * need) != cudaSuccess) return CRM_ERR_CUDA;
    h.out_cap = need;
  }
  // inputs: requests' packed columns side by side -> (n, rows) per field
  const size_t irows = s->in_rows_total();
  {
    int off = 0;
    for (Request *r : h.reqs) {
      const int m = (int)r->slots.size();
      size_t base = 0;
      for (int f = 0; f < I_NIN; ++f) {
        const size_t rows = s->in_rows(f);
        for (size_t row = 0; row < rows; ++row)
          memcpy(h.h_in + (base + row) * n + off, r->in.data() + (base + row) * m, sizeof(double) * m);
        base += rows;
      }
      for (int i = 0; i < m; ++i) {
        h.h_map[off + i] = r->slots[i];
        h.h_gcol[off + i] = r->gcol[i];
      }
      off += m;
    }
  }
  cudaStream_t st = h.stream;
  if (cudaMemcpyAsync(h.d_in, h.h_in, sizeof(double) * irows * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(h.d_map, h.h_map, sizeof(int) * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(h.d_gcol, h.h_gcol, sizeof(int) * n, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return CRM_ERR_CUDA;
  {
    std::vector<double *> sa, pk;
    std::vector<int> rows;
    size_t base = 0;
    for (int f = 0; f < I_NIN; ++f) {
      sa.push_back(s->in_arr[f]);
      pk.push_back(h.d_in + base * n);
      rows.push_back((int)s->in_rows(f));
      base += s->in_rows(f);
    }
    int rc = copy_slots(s, st, n, h.d_map, true, sa, pk, rows);
    if (rc != CRM_OK) return rc;
  }
  // new radiative heating of the requests that carry one, into their slots
  {
    const size_t rows = s->rad_rows();
    int off = 0;
    for (Request *r : h.reqs) {
      const int m = (int)r->slots.size();
      if (r->has_qrad) {
        memcpy(h.h_q + rows * off, r->qrad.data(), sizeof(double) * rows * m);
        if (cudaMemcpyAsync(h.d_q + rows * off, h.h_q + rows * off, sizeof(double) * rows * m,
                            cudaMemcpyHostToDevice, st) != cudaSuccess)
          return CRM_ERR_CUDA;
        std::vector<double *> sa{s->rad[0]}, pk{h.d_q + rows * off};
        std::vector<int> rw{(int)rows};
        int rc = copy_slots(s, st, m, h.d_map + off, true, sa, pk, rw);
        if (rc != CRM_OK) return rc;
      }
      off += m;
    }
  }
  // the column kernel over the union of slots
  crm_input_c in;
  memset(&in, 0, sizeof in);
  in.zmid = s->in_arr[I_ZMID]; in.zint = s->in_arr[I_ZINT]; in.tl = s->in_arr[I_TL];
  in.ql = s->in_arr[I_QL]; in.qccl = s->in_arr[I_QCCL]; in.qiil = s->in_arr[I_QIIL];
  in.pmid = s->in_arr[I_PMID]; in.pint = s->in_arr[I_PINT]; in.pdel = s->in_arr[I_PDEL];
  in.ul = s->in_arr[I_UL]; in.vl = s->in_arr[I_VL]; in.tau00 = s->in_arr[I_TAU00];
  in.bflxls = s->in_arr[I_BFLXLS]; in.wndls = s->in_arr[I_WNDLS];
  crm_state_c stt{s->state[0], s->state[1], s->state[2], s->state[3], s->state[4], s->state[5], s->state[6]};
  crm_rad_c rd{s->rad[0], s->rad[1], s->rad[2], s->rad[3], s->rad[4], s->rad[5]};
  crm_output_c out;
  for (int f = 0; f < CRM_NOUT; ++f) out.field[f] = s->out[f];
  crm_call_desc d;
  memset(&d, 0, sizeof d);
  d.ncrms = n; d.ld = s->capacity; d.dt_gl = h.reqs[0]->dt_gl;
  d.igstep = h.reqs[0]->first ? 1 : 2;
  d.gcol = h.d_gcol; d.col_map = h.d_map;
  int rc = crm_run_device(h.ctx, &d, &in, &stt, &rd, &out, h.d_status, st);
  if (rc != CRM_OK) return rc;
  // gather the requested outputs of the launched slots
  {
    std::vector<double *> sa, pk;
    std::vector<int> rows;
    size_t base = 0;
    for (int f : h.fields) {
      sa.push_back(f < CRM_NOUT ? s->out[f] : s->rad[1 + (f - CRM_NOUT)]);
      pk.push_back(h.d_out + base * n);
      rows.push_back((int)s->out_rows(f));
      base += s->out_rows(f);
    }
    rc = copy_slots(s, st, n, h.d_map, false, sa, pk, rows);
    if (rc != CRM_OK) return rc;
    if (cudaMemcpyAsync(h.h_out, h.d_out, sizeof(double) * base * n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(h.h_status, h.d_status, sizeof(int) * n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaEventRecord(h.done, st) != cudaSuccess)
      return CRM_ERR_CUDA;
  }
  return CRM_OK;
}

// Copy a finished launch's results into the callers' arrays (lock held).
void complete(crm_server *s, Handle &h, int rc) {
  int off = 0;
  for (Request *r : h.reqs) {
    ChunkRec &c = s->chunks[r->chunk];
    const int m = (int)r->slots.size();
    if (rc == CRM_OK) {
      size_t base = 0;
      for (int f : h.fields) {
        const size_t rows = s->out_rows(f);
        double *dst = nullptr;
        if (f < CRM_NOUT) dst = r->out.field[f];
        else {
          double *rp[5] = {r->rad.temperature, r->rad.qv, r->rad.qc, r->rad.qi, r->rad.cld};
          dst = rp[f - CRM_NOUT];
        }
        if (dst) unpack(h.h_out + base * h.n, h.n, off, m, rows, dst, r->ld);
        base += rows;
      }
      int worst = CRM_OK;
      for (int i = 0; i < m; ++i) {
        const int st = h.h_status[off + i];
        if (r->col_status) r->col_status[i] = st;
        if (st != CRM_OK) worst = st;
      }
      r->status = worst;
    } else {
      r->status = rc;
    }
    c.steps += 1;
    c.busy = false;
    c.queued -= 1;
    r->done = 2;
    off += m;
  }
  h.reqs.clear();
  h.busy = false;
}

void engine_loop(crm_server *s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (!s->stop) {
    bool progressed = false;
    // completions
    for (Handle &h : s->handles) {
      if (!h.busy || h.reqs.empty()) continue;
      cudaError_t q = cudaEventQuery(h.done);
      if (q == cudaErrorNotReady) continue;
      complete(s, h, q == cudaSuccess ? CRM_OK : CRM_ERR_CUDA);
      progressed = true;
    }
    if (progressed) s->cv.notify_all();
    // new launches: one per idle handle while requests can go
    for (Handle &h : s->handles) {
      if (h.busy || s->pending.empty()) continue;
      Request *head = nullptr;
      for (Request *r : s->pending)
        if (!s->chunks[r->chunk].busy) { head = r; break; }
      if (!head) break;
      std::vector<Request *> take;
      std::deque<Request *> rest;
      for (Request *r : s->pending) {
        ChunkRec &c = s->chunks[r->chunk];
        if (!c.busy && r->dt_gl == head->dt_gl && (c.steps == 0) == (s->chunks[head->chunk].steps == 0)) {
          c.busy = true;
          r->first = c.steps == 0;
          r->slots = c.slots;
          r->gcol = c.gcol;
          r->done = 1;
          take.push_back(r);
        } else {
          rest.push_back(r);
        }
      }
      s->pending.swap(rest);
      h.reqs = take;
      h.busy = true;
      lk.unlock();
      int rc = issue(s, h);
      lk.lock();
      if (rc != CRM_OK) {
        complete(s, h, rc);
        s->cv.notify_all();
      } else {
        s->launches += 1;
      }
    }
    bool inflight = false;
    for (Handle &h : s->handles) inflight = inflight || h.busy;
    if (inflight) {
      lk.unlock();
      std::this_thread::sleep_for(std::chrono::microseconds(100));
      lk.lock();
    } else {
      s->cv.wait_for(lk, std::chrono::milliseconds(20));
    }
  }
}

void destroy_server(crm_server *s) {
  for (Handle &h : s->handles) free_handle(h);
  for (double *&p : s->in_arr) cudaFree(p);
  for (double *&p : s->state) cudaFree(p);
  for (double *&p : s->rad) cudaFree(p);
  for (double *&p : s->out) cudaFree(p);
  if (s->io_stream) cudaStreamDestroy(s->io_stream);
  delete s;
}

}  // namespace

extern "C" {

crm_server *crm_server_create(const crm_config *cfg, int capacity, int nhandles,
                              unsigned long long hbm_budget_bytes, int *status) {
  auto fail = [&](int rc, crm_server *s) -> crm_server * {
    if (s) destroy_server(s);
    if (status) *status = rc;
    return nullptr;
  };
  if (!cfg || capacity < 1 || nhandles < 1 || nhandles > 16) return fail(CRM_ERR_ARG, nullptr);
  if (cfg->batch_mode != CRM_PER_COLUMN) return fail(CRM_ERR_UNSUPPORTED, nullptr);
  crm_config g = *cfg;
  g.max_ncrms = capacity;
  if (g.crm_nx_rad < 1) g.crm_nx_rad = g.crm_nx;
  if (g.crm_ny_rad < 1) g.crm_ny_rad = 1;
  unsigned long long hb = 0;
  int rc = crm_plan_device_bytes(&g, &hb);
  if (rc != CRM_OK) return fail(rc, nullptr);
  crm_server *s = new crm_server();
  s->cfg = g;
  s->capacity = capacity;
  s->budget = hbm_budget_bytes;
  if (cudaGetDevice(&s->device) != cudaSuccess) return fail(CRM_ERR_NO_DEVICE, s);
  // charged before anything is allocated: pool arrays, handles, staging
  const unsigned long long per_handle_staging =
      (unsigned long long)capacity * (3 * sizeof(int) + sizeof(double) * (s->in_rows_total() + s->rad_rows()));
  const unsigned long long need = sizeof(double) * (unsigned long long)s->pool_doubles() +
                                  (unsigned long long)nhandles * (hb + per_handle_staging);
  if (need > s->budget) return fail(CRM_ERR_BUDGET, s);
  s->used_bytes = need;
  auto dalloc = [&](double *&p, size_t rows) {
    return cudaMalloc(&p, sizeof(double) * rows * (size_t)capacity) == cudaSuccess &&
           cudaMemset(p, 0, sizeof(double) * rows * (size_t)capacity) == cudaSuccess;
  };
  for (int f = 0; f < I_NIN; ++f)
    if (!dalloc(s->in_arr[f], s->in_rows(f))) return fail(CRM_ERR_CUDA, s);
  for (int f = 0; f < 7; ++f)
    if (!dalloc(s->state[f], s->state_rows())) return fail(CRM_ERR_CUDA, s);
  for (int f = 0; f < 6; ++f)
    if (!dalloc(s->rad[f], s->rad_rows())) return fail(CRM_ERR_CUDA, s);
  for (int f = 0; f < CRM_NOUT; ++f)
    if (!dalloc(s->out[f], s->out_rows(f))) return fail(CRM_ERR_CUDA, s);
  if (cudaStreamCreateWithFlags(&s->io_stream, cudaStreamNonBlocking) != cudaSuccess) return fail(CRM_ERR_CUDA, s);
  s->handles.resize(nhandles);
  for (Handle &h : s->handles) {
    int st = 0;
    h.ctx = crm_create(&g, &st);
    if (!h.ctx) return fail(st, s);
    if (cudaStreamCreateWithFlags(&h.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h.done, cudaEventDisableTiming) != cudaSuccess)
      return fail(CRM_ERR_CUDA, s);
    crm_set_stream(h.ctx, h.stream);
    const size_t irows = s->in_rows_total();
    if (cudaMalloc(&h.d_map, sizeof(int) * capacity) != cudaSuccess ||
        cudaMalloc(&h.d_gcol, sizeof(int) * capacity) != cudaSuccess ||
        cudaMalloc(&h.d_status, sizeof(int) * capacity) != cudaSuccess ||
        cudaMalloc(&h.d_in, sizeof(double) * irows * capacity) != cudaSuccess ||
        cudaMalloc(&h.d_q, sizeof(double) * s->rad_rows() * capacity) != cudaSuccess ||
        cudaMallocHost(&h.h_in, sizeof(double) * irows * capacity) != cudaSuccess ||
        cudaMallocHost(&h.h_q, sizeof(double) * s->rad_rows() * capacity) != cudaSuccess ||
        cudaMallocHost(&h.h_map, sizeof(int) * capacity) != cudaSuccess ||
        cudaMallocHost(&h.h_gcol, sizeof(int) * capacity) != cudaSuccess ||
        cudaMallocHost(&h.h_status, sizeof(int) * capacity) != cudaSuccess)
      return fail(CRM_ERR_CUDA, s);
  }
  for (int i = capacity - 1; i >= 0; --i) s->free_slots.push_back(i);
  s->engine = std::thread(engine_loop, s);
  if (status) *status = CRM_OK;
  return s;
}

void crm_server_destroy(crm_server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  if (s->engine.joinable()) s->engine.join();
  for (Handle &h : s->handles)
    if (h.stream) cudaStreamSynchronize(h.stream);
  destroy_server(s);
}

unsigned long long crm_server_device_bytes(const crm_server *s) { return s ? s->used_bytes.load() : 0ull; }

long long crm_server_launches(const crm_server *s) { return s ? s->launches.load() : 0; }

int crm_chunk_open(crm_server *s, int ncols, const int *gcol, int ld, const crm_state_c *st,
                   const crm_rad_c *rad, int *chunk) {
  if (!s || ncols < 1 || !gcol || ld < ncols || !st || !rad || !rad->qrad || !chunk) return CRM_ERR_ARG;
  const double *sp[7] = {st->u_wind, st->v_wind, st->w_wind, st->temperature, st->qt, st->qp, st->qn};
  for (const double *p : sp)
    if (!p) return CRM_ERR_ARG;
  std::vector<int> slots;
  int id;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if ((int)s->free_slots.size() < ncols) return CRM_ERR_BUDGET;
    for (int i = 0; i < ncols; ++i) {
      slots.push_back(s->free_slots.back());
      s->free_slots.pop_back();
    }
    id = s->next_chunk++;
    ChunkRec &c = s->chunks[id];
    c.slots = slots;
    c.gcol.assign(gcol, gcol + ncols);
  }
  // the chunk's state and heating into its slots (the slots were free: no
  // launch touches them)
  cudaSetDevice(s->device);
  const size_t srows = s->state_rows(), rrows = s->rad_rows();
  std::vector<double> packed((size_t)ncols * (7 * srows + rrows));
  std::vector<double *> sa, pk;
  std::vector<int> rows;
  double *d_pk = nullptr;
  int *d_slots = nullptr;
  int rc = CRM_OK;
  if (cudaMalloc(&d_pk, sizeof(double) * packed.size()) != cudaSuccess ||
      cudaMalloc(&d_slots, sizeof(int) * ncols) != cudaSuccess)
    rc = CRM_ERR_CUDA;
  if (rc == CRM_OK) {
    for (int f = 0; f < 7; ++f) {
      pack(sp[f], ld, ncols, srows, packed.data() + (size_t)f * srows * ncols);
      sa.push_back(s->state[f]);
      pk.push_back(d_pk + (size_t)f * srows * ncols);
      rows.push_back((int)srows);
    }
    pack(rad->qrad, ld, ncols, rrows, packed.data() + 7 * srows * ncols);
    sa.push_back(s->rad[0]);
    pk.push_back(d_pk + 7 * srows * ncols);
    rows.push_back((int)rrows);
    if (cudaMemcpyAsync(d_pk, packed.data(), sizeof(double) * packed.size(), cudaMemcpyHostToDevice, s->io_stream) != cudaSuccess ||
        cudaMemcpyAsync(d_slots, slots.data(), sizeof(int) * ncols, cudaMemcpyHostToDevice, s->io_stream) != cudaSuccess)
      rc = CRM_ERR_CUDA;
  }
  if (rc == CRM_OK) rc = copy_slots(s, s->io_stream, ncols, d_slots, true, sa, pk, rows);
  if (rc == CRM_OK && cudaStreamSynchronize(s->io_stream) != cudaSuccess) rc = CRM_ERR_CUDA;
  cudaFree(d_pk);
  cudaFree(d_slots);
  std::lock_guard<std::mutex> lk(s->mu);
  if (rc != CRM_OK) {
    for (int sl : slots) s->free_slots.push_back(sl);
    s->chunks.erase(id);
    return rc;
  }
  s->chunks[id].open = true;
  *chunk = id;
  return CRM_OK;
}

int crm_chunk_read_state(crm_server *s, int chunk, int ld, crm_state_c *st, double *qrad) {
  if (!s || !st) return CRM_ERR_ARG;
  std::vector<int> slots;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->chunks.find(chunk);
    if (it == s->chunks.end() || !it->second.open) return CRM_ERR_ARG;
    if (it->second.queued > 0) return CRM_ERR_ARG;      // steps still to run
    slots = it->second.slots;
  }
  const int n = (int)slots.size();
  if (ld < n) return CRM_ERR_ARG;
  double *sp[7] = {st->u_wind, st->v_wind, st->w_wind, st->temperature, st->qt, st->qp, st->qn};
  cudaSetDevice(s->device);
  const size_t srows = s->state_rows(), rrows = s->rad_rows();
  std::vector<double> packed((size_t)n * (7 * srows + rrows));
  double *d_pk = nullptr;
  int *d_slots = nullptr;
  int rc = CRM_OK;
  if (cudaMalloc(&d_pk, sizeof(double) * packed.size()) != cudaSuccess ||
      cudaMalloc(&d_slots, sizeof(int) * n) != cudaSuccess ||
      cudaMemcpyAsync(d_slots, slots.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s->io_stream) != cudaSuccess)
    rc = CRM_ERR_CUDA;
  std::vector<double *> sa, pk;
  std::vector<int> rows;
  for (int f = 0; f < 7; ++f) {
    sa.push_back(s->state[f]);
    pk.push_back(d_pk + (size_t)f * srows * n);
    rows.push_back((int)srows);
  }
  sa.push_back(s->rad[0]);
  pk.push_back(d_pk + 7 * srows * n);
  rows.push_back((int)rrows);
  if (rc == CRM_OK) rc = copy_slots(s, s->io_stream, n, d_slots, false, sa, pk, rows);
  if (rc == CRM_OK &&
      (cudaMemcpyAsync(packed.data(), d_pk, sizeof(double) * packed.size(), cudaMemcpyDeviceToHost, s->io_stream) != cudaSuccess ||
       cudaStreamSynchronize(s->io_stream) != cudaSuccess))
    rc = CRM_ERR_CUDA;
  cudaFree(d_pk);
  cudaFree(d_slots);
  if (rc != CRM_OK) return rc;
  for (int f = 0; f < 7; ++f)
    if (sp[f]) unpack(packed.data() + (size_t)f * srows * n, n, 0, n, srows, sp[f], ld);
  if (qrad) unpack(packed.data() + 7 * srows * n, n, 0, n, rrows, qrad, ld);
  return CRM_OK;
}

int crm_chunk_close(crm_server *s, int chunk) {
  if (!s) return CRM_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->chunks.find(chunk);
  if (it == s->chunks.end() || !it->second.open) return CRM_ERR_ARG;
  if (it->second.queued > 0) return CRM_ERR_ARG;        // steps still to run
  for (int sl : it->second.slots) s->free_slots.push_back(sl);
  s->chunks.erase(it);
  return CRM_OK;
}

int crm_submit(crm_server *s, int chunk, const crm_input_c *in, const double *qrad, int ld, double dt_gl,
               crm_output_c *out, crm_rad_c *rad_means, int *col_status, long long *ticket) {
  if (!s || !in || !ticket || !(dt_gl > 0)) return CRM_ERR_ARG;
  const double *src[I_NIN] = {in->zmid, in->zint, in->tl, in->ql, in->qccl, in->qiil, in->pmid,
                              in->pint, in->pdel, in->ul, in->vl, in->tau00, in->bflxls, in->wndls};
  for (const double *p : src)
    if (!p) return CRM_ERR_ARG;
  std::unique_ptr<Request> r(new Request());
  int m;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->chunks.find(chunk);
    if (it == s->chunks.end() || !it->second.open) return CRM_ERR_ARG;
    m = (int)it->second.slots.size();
  }
  if (ld < m) return CRM_ERR_ARG;
  r->in.resize(s->in_rows_total() * (size_t)m);
  size_t base = 0;
  for (int f = 0; f < I_NIN; ++f) {
    pack(src[f], ld, m, s->in_rows(f), r->in.data() + base * m);
    base += s->in_rows(f);
  }
  if (qrad) {
    r->has_qrad = true;
    r->qrad.resize(s->rad_rows() * (size_t)m);
    pack(qrad, ld, m, s->rad_rows(), r->qrad.data());
  }
  if (out) r->out = *out;
  if (rad_means) {
    r->rad = *rad_means;
    r->rad.qrad = nullptr;
  }
  r->col_status = col_status;
  r->ld = ld;
  r->dt_gl = dt_gl;
  r->chunk = chunk;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->chunks.find(chunk);
    if (it == s->chunks.end() || !it->second.open) return CRM_ERR_ARG;
    it->second.queued += 1;
    r->ticket = s->next_ticket++;
    *ticket = r->ticket;
    s->pending.push_back(r.get());
    s->requests[r->ticket] = std::move(r);
  }
  s->cv.notify_all();
  return CRM_OK;
}

int crm_poll(crm_server *s, long long ticket, int wait) {
  if (!s) return CRM_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    auto it = s->requests.find(ticket);
    if (it == s->requests.end()) return CRM_ERR_ARG;
    if (it->second->done == 2) {
      int st = it->second->status;
      s->requests.erase(it);
      return st;
    }
    if (!wait) return CRM_PENDING;
    s->cv.wait_for(lk, std::chrono::milliseconds(50));
  }
}

}  // extern "C"
