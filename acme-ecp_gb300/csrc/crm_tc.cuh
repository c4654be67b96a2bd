// crm_tc.cuh -- the x/y transforms of the 3D pressure solve on the tensor
// cores (tcgen05, kind::tf32, 3xTF32), for the FP32-mixed form with
// nx = ny = n in {16, 32}.
//
// pressure.F90:97-310 transforms every level of the right-hand side with
// fft991 in x (rows j = 1..ny) and then in y (x coefficients i = 1..nx+1),
// solves a tridiagonal system per (i, j) coefficient, and transforms back.
// fft991 of a real row is linear: forward, x (n values) -> (n + 2) values
// [Re X_0, Im X_0, Re X_1, Im X_1, ..., Re X_n/2, Im X_n/2] of X = rfft(x)/n;
// inverse, the row back from the n + 2 values.  So each direction is a
// product with a fixed real matrix,
//   Bf (n+2 rows, n cols):  Bf[2k][i] = cos(2 pi i k / n) / n,
//                           Bf[2k+1][i] = -sin(2 pi i k / n) / n;
//   Bi (n rows, n+2 cols):  Bi[i][2k] = w_k cos(2 pi i k / n),
//                           Bi[i][2k+1] = -w_k sin(2 pi i k / n),
//                           w_0 = w_n/2 = 1, else 2;
// and a level's 2D transform is F = Bf P Bf^T, P = Bi F Bi^T (x and y have
// the same length).  Each one-direction pass over a tile of L = 128 / n
// levels is one GEMM with M = 128 rows:
//   forward x:  rows (level, j), K = i,      N = n + 2 -> D[(l, j)][c]
//   forward y:  rows (level, c), K = j,      N = n + 2 -> D[(l, c)][jj]
//                 (c = 0..n-1 on the tensor cores; the Nyquist column
//                  c = n on the CUDA cores; c = n + 1 is Im X_n/2 = 0)
//   inverse y:  rows (level, c), K = jj,     N = n     -> D[(l, c)][j]
//   inverse x:  rows (level, j), K = c,      N = n     -> D[(l, j)][i]
// Operands are staged in shared memory in the no-swizzle K-major core-matrix
// layout (8 rows x 16 bytes per core matrix, K-adjacent core matrices 128
// bytes apart, 8-row groups (K/4) x 128 bytes apart); the accumulator is a
// 128-lane x N-column fp32 tile in tensor memory, read back with tcgen05.ld.
// Split TF32: every operand is split into three TF32 parts (head, middle,
// tail: each the remainder rounded to nearest), x = x0 + x1 + x2 to 2^-33,
// and D = sum of the six products A_p B_q with p + q <= 2 (smallest first),
// which carries the products to FP32 accuracy (a two-part split, the usual
// 3xTF32, leaves 2^-22 per product: measured 1.5e-4 against 9e-5 relative L2
// on a GCM tendency where the FP32 FFT stays within 1e-4).
// Means: an FFT's first butterflies subtract pairs of inputs, so a row's
// mean never enters its other coefficients; a product with the DFT matrix
// would spread eps |mean| into every one of them (and the pressure field's
// horizontal mean is large against its perturbations).  Every pass therefore
// takes the mean out of the operand rows and adds it back exactly: forward,
// each row's mean (computed on the CUDA cores) is subtracted and becomes the
// X_0 coefficient; inverse, the X_0 input is left out of the product and
// added to every output.
//
// One thread issues the MMAs and commits them to an mbarrier; every wait on
// it is bounded (a timeout marks the column CRM_ERR_TIMEOUT and skips the
// remaining products).  Tensor memory is allocated once per CTA by warp 0
// before the column loop and released after it.
#pragma once

#include <cstdint>

namespace crm {
namespace tc {

constexpr int kSplit = 3;      // TF32 parts per operand element

// dimensions of the transform of length n (n = 16 or 32)
struct Dims {
  int n, L, nf, ki;     // L = 128 / n levels per tile; nf = N of the forward
                        // passes (n + 2 rounded up to 16); ki = K of the
                        // inverse passes (n + 2 rounded up to 8)
  __host__ __device__ explicit Dims(int n_) : n(n_), L(128 / n_), nf((n_ + 2 + 15) / 16 * 16), ki((n_ + 2 + 7) / 8 * 8) {}
  // float offsets of the shared-memory regions (each a multiple of 32 floats)
  __host__ __device__ int a_elems() const { return 128 * ki; }
  __host__ __device__ int bf_elems() const { return nf * n; }
  __host__ __device__ int bi_elems() const { return n * ki; }
  __host__ __device__ int gny_elems() const { return (L * n + 31) / 32 * 32; }
  __host__ __device__ int aux_elems() const { return 2 * 128; }       // row means / X_0 terms
  // part p of the staged operand A, of Bf, of Bi
  __host__ __device__ int off_a(int p) const { return p * a_elems(); }
  __host__ __device__ int off_bf(int p) const { return kSplit * a_elems() + p * bf_elems(); }
  __host__ __device__ int off_bi(int p) const { return kSplit * (a_elems() + bf_elems()) + p * bi_elems(); }
  __host__ __device__ int off_gny() const { return kSplit * (a_elems() + bf_elems() + bi_elems()); }
  __host__ __device__ int off_aux() const { return off_gny() + gny_elems(); }
  __host__ __device__ int total_elems() const { return off_aux() + aux_elems(); }
};

// shared-memory bytes of the tensor-core transform (0: not used)
__host__ __device__ inline size_t smem_bytes(int n) { return n ? sizeof(float) * (size_t)Dims(n).total_elems() + 128 : 0; }

// float index of element (r, q) of an R x K operand in the core-matrix layout
__device__ __forceinline__ int cm_index(int r, int q, int K) {
  return ((r >> 3) * (K >> 2) + (q >> 2)) * 32 + (r & 7) * 4 + (q & 3);
}
// the element a linear index e of that layout holds
__device__ __forceinline__ void cm_coords(int e, int K, int &r, int &q) {
  const int cm = e >> 5, w = e & 31, kq = K >> 2;
  r = (cm / kq) * 8 + (w >> 2);
  q = (cm % kq) * 4 + (w & 3);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ float tf32_head(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}
// x = v[0] + v[1] + v[2], each TF32 (every remainder exact in FP32)
__device__ __forceinline__ void splitk(float x, float *v) {
  v[0] = tf32_head(x);
  const float r1 = x - v[0];
  v[1] = tf32_head(r1);
  v[2] = tf32_head(r1 - v[1]);
}

// shared-memory matrix descriptor: no swizzle, K-major
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;                       // descriptor version of tcgen05
  return d;                                     // base offset 0, layout 0 (no swizzle)
}
// instruction descriptor: kind::tf32, D fp32, A and B tf32 K-major, M = 128
__device__ __forceinline__ uint32_t idesc_tf32(int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint32_t mbar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// wait for the phase with the given parity to complete; false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, long long limit) {
  for (long long it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred P1;\n\tmbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, P1;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// tensor memory: warp-wide allocation of ncols columns, address into *slot
__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols) : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
// 16 consecutive fp32 columns of this thread's lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int m = 0; m < 16; ++m) v[m] = __uint_as_float(r[m]);
}

constexpr uint32_t kTmemCols = 64;           // D tiles use at most 48 columns
constexpr long long kWaitLimit = 1ll << 24;  // mbarrier polls before a timeout

// The transform engine of one CTA.  sm: the dynamic shared-memory region
// (128-byte aligned); mats: Bf (nf x n) then Bi (n x ki), row-major, zero
// rows / columns beyond n + 2; state: the CTA's tensor-memory address,
// mbarrier and phase (in the kernel's static shared memory).
struct Engine {
  Dims d;
  float *sm;
  uint32_t tmem;
  uint32_t mbar;
  uint32_t *phase;
  int *fail;
  int tid, nt;

  __device__ Engine(int n, float *sm_, uint32_t tmem_, uint32_t mbar_, uint32_t *phase_, int *fail_, int tid_, int nt_)
      : d(n), sm(sm_), tmem(tmem_), mbar(mbar_), phase(phase_), fail(fail_), tid(tid_), nt(nt_) {}

  __device__ float *gny() const { return sm + d.off_gny(); }
  __device__ float *aux0() const { return sm + d.off_aux(); }
  __device__ float *aux1() const { return sm + d.off_aux() + 128; }

  // element e of operand A (or of a matrix at part offsets off(p)): split
  // store, and the value back
  __device__ void put_a(int e, float x) const {
    float v[kSplit];
    splitk(x, v);
#pragma unroll
    for (int p = 0; p < kSplit; ++p) sm[d.off_a(p) + e] = v[p];
  }
  __device__ float get_a(int e) const {
    float x = 0.f;
#pragma unroll
    for (int p = kSplit - 1; p >= 0; --p) x += sm[d.off_a(p) + e];
    return x;
  }

  // the mean of each of the 128 rows of the staged operand (n valid
  // columns, layout K = kl) into m[], then those rows minus their mean;
  // one thread per row
  __device__ void center_rows(int kl, float *m) const {
    for (int r = tid; r < 128; r += nt) {
      float sum = 0.f;
      for (int q = 0; q < d.n; ++q) sum += get_a(cm_index(r, q, kl));
      const float mean = sum / (float)d.n;
      m[r] = mean;
      for (int q = 0; q < d.n; ++q) {
        const int e = cm_index(r, q, kl);
        put_a(e, get_a(e) - mean);
      }
    }
  }

  // the constant matrices into shared memory, split (once per CTA)
  __device__ void load_mats(const float *mats) const {
    const float *bf = mats, *bi = mats + (size_t)d.nf * d.n;
    for (int e = tid; e < d.bf_elems(); e += nt) {
      int r, q;
      cm_coords(e, d.n, r, q);
      float v[kSplit];
      splitk(bf[r * d.n + q], v);
#pragma unroll
      for (int p = 0; p < kSplit; ++p) sm[d.off_bf(p) + e] = v[p];
    }
    for (int e = tid; e < d.bi_elems(); e += nt) {
      int r, q;
      cm_coords(e, d.ki, r, q);
      float v[kSplit];
      splitk(bi[r * d.ki + q], v);
#pragma unroll
      for (int p = 0; p < kSplit; ++p) sm[d.off_bi(p) + e] = v[p];
    }
  }
  __device__ float bf(int r, int q) const {       // Bf[r][q]
    const int e = cm_index(r, q, d.n);
    float x = 0.f;
#pragma unroll
    for (int p = kSplit - 1; p >= 0; --p) x += sm[d.off_bf(p) + e];
    return x;
  }
  __device__ float bi(int r, int q) const {       // Bi[r][q]
    const int e = cm_index(r, q, d.ki);
    float x = 0.f;
#pragma unroll
    for (int p = kSplit - 1; p >= 0; --p) x += sm[d.off_bi(p) + e];
    return x;
  }

  // D (128 x N) = A (128 x K, staged) . B^T (B: N x K, parts at boff(p)):
  // the products A_p B_q with p + q < kSplit, smallest first; every thread
  // returns once D is in tensor memory
  template <typename BOff>
  __device__ void gemm(int K, int N, BOff boff) {
    fence_async_smem();          // the operands written by this thread, to the tensor cores
    __syncthreads();
    if (tid == 0 && !*fail) {
      fence_after();
      const uint32_t id = idesc_tf32(N);
      const uint32_t sbo = (uint32_t)(K / 4) * 128u;
      bool first = true;
      for (int order = kSplit - 1; order >= 0; --order)
        for (int pa = order; pa >= 0; --pa) {
          const int pb = order - pa;
          const uint32_t a = smem_u32(sm + d.off_a(pa)), b = smem_u32(sm + boff(pb));
          for (int s = 0; s < K / 8; ++s) {
            const uint32_t o = (uint32_t)s * 256u;
            mma_tf32(tmem, sdesc(a + o, 128u, sbo), sdesc(b + o, 128u, sbo), id, first ? 0u : 1u);
            first = false;
          }
        }
      commit(mbar);
    }
    if (!*fail) {
      if (!mbar_wait(mbar, *phase & 1u, kWaitLimit)) *fail = 1;
    }
    __syncthreads();
    if (tid == 0) *phase ^= 1u;
    fence_after();
  }
  __device__ void gemm_fwd(int K, int N) {
    gemm(K, N, [&](int p) { return d.off_bf(p); });
  }
  __device__ void gemm_inv(int K, int N) {
    gemm(K, N, [&](int p) { return d.off_bi(p); });
  }

  // each warp of the first four per column block reads its lane quarter:
  // calls f(row, col0, v[16]) for column blocks col0 = 0, 16, ... < N
  template <typename F>
  __device__ void read_d(int N, F f) const {
    const int warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
    const int nblk = (N + 15) / 16;
    for (int wb = warp; wb < 4 * nblk; wb += nw) {
      const int lq = wb & 3, cb = wb >> 2;
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(32 * lq) << 16) + (uint32_t)(16 * cb), v);
      f(32 * lq + lane, 16 * cb, v);
    }
    fence_before();
  }

  // Forward transform of levels [k0, k0 + L) of FF (FF(i, j, k): 1-based,
  // x fastest, rows of n + 2, n + 2 rows per level), in place; levels > nzm
  // are read as zero and not written.
  template <typename FFT>
  __device__ void forward_tile(FFT FF, int k0, int nzm) {
    const int n = d.n, L = d.L;
    float *G = gny(), *mx = aux0(), *my = aux1();
    // x pass: A[(l, j)][i] = P(i, j, k)
    for (int e = tid; e < 128 * n; e += nt) {
      int r, q;
      cm_coords(e, n, r, q);
      const int l = r / n, j = r % n, k = k0 + l;
      put_a(e, k <= nzm ? FF(q + 1, j + 1, k) : 0.f);
    }
    __syncthreads();
    center_rows(n, mx);
    gemm_fwd(n, d.nf);
    // the x coefficients c < n become the rows of the y pass (X_0 with the
    // row mean added back); c = n (the Nyquist column) goes to G
    read_d(d.nf, [&](int r, int c0, const float *v) {
      const int l = r / n, j = r % n;
      for (int m = 0; m < 16; ++m) {
        const int c = c0 + m;
        if (c < n) put_a(cm_index(l * n + c, j, n), c == 0 ? v[m] + mx[r] : v[m]);
        else if (c == n) G[l * n + j] = v[m];
      }
    });
    __syncthreads();
    center_rows(n, my);
    gemm_fwd(n, d.nf);
    read_d(d.nf, [&](int r, int c0, const float *v) {
      const int l = r / n, c = r % n, k = k0 + l;
      if (k > nzm) return;
      for (int m = 0; m < 16; ++m) {
        const int jj = c0 + m;
        if (jj < n + 2) FF(c + 1, jj + 1, k) = jj == 0 ? v[m] + my[r] : v[m];
      }
    });
    // the Nyquist column's y transform on the CUDA cores
    for (int e = tid; e < L * (n + 2); e += nt) {
      const int l = e / (n + 2), jj = e % (n + 2), k = k0 + l;
      if (k > nzm) continue;
      float s = 0.f;
      for (int j = 0; j < n; ++j) s = fmaf(bf(jj, j), G[l * n + j], s);
      FF(n + 1, jj + 1, k) = s;
    }
    __syncthreads();
  }

  // Inverse transform of levels [k0, k0 + L), in place (the coefficients of
  // x index n + 2, Im X_n/2, are not read).
  template <typename FFT>
  __device__ void inverse_tile(FFT FF, int k0, int nzm) {
    const int n = d.n, L = d.L, ki = d.ki;
    float *G = gny(), *f0 = aux0(), *g0 = aux1();
    // y pass: A[(l, c)][jj] = F(c + 1, jj + 1, k), c < n, K padded to ki; X_0
    // (jj = 0) is left out and added to every output
    for (int e = tid; e < 128 * ki; e += nt) {
      int r, q;
      cm_coords(e, ki, r, q);
      const int l = r / n, c = r % n, k = k0 + l;
      const float x = (k <= nzm && q < n + 2) ? FF(c + 1, q + 1, k) : 0.f;
      if (q == 0) f0[r] = x;
      put_a(e, q == 0 ? 0.f : x);
    }
    // the Nyquist column back to grid rows j on the CUDA cores
    for (int e = tid; e < L * n; e += nt) {
      const int l = e / n, j = e % n, k = k0 + l;
      float s = 0.f;
      if (k <= nzm)
        for (int jj = 0; jj < n + 2; ++jj) s = fmaf(bi(j, jj), FF(n + 1, jj + 1, k), s);
      G[l * n + j] = s;
    }
    __syncthreads();
    gemm_inv(ki, n);
    // x pass: A[(l, j)][c] = D[(l, c)][j] + X_0 for c < n (c = 0 left out and
    // added to every output), G for c = n, 0 beyond
    read_d(n, [&](int r, int j0, const float *v) {
      const int l = r / n, c = r % n;
      for (int m = 0; m < 16; ++m) {
        const int j = j0 + m;
        if (j < n) {
          const float x = v[m] + f0[r];
          if (c == 0) g0[l * n + j] = x;
          put_a(cm_index(l * n + j, c, ki), c == 0 ? 0.f : x);
        }
      }
    });
    for (int e = tid; e < 128 * (ki - n); e += nt) {
      const int r = e / (ki - n), c = n + e % (ki - n);
      put_a(cm_index(r, c, ki), c == n ? G[r] : 0.f);
    }
    __syncthreads();
    gemm_inv(ki, n);
    read_d(n, [&](int r, int i0, const float *v) {
      const int l = r / n, j = r % n, k = k0 + l;
      if (k > nzm) return;
      for (int m = 0; m < 16; ++m) {
        const int i = i0 + m;
        if (i < n) FF(i + 1, j + 1, k) = v[m] + g0[r];
      }
    });
    __syncthreads();
  }
};

}  // namespace tc
}  // namespace crm
