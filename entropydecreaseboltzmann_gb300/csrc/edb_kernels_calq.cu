// Collision sum Q-hat (QCalculator::calQ, CalQ/QCalculator.h:231-257).
//
// FP64 drop-in path (one solve, the reference's B table streamed from HBM):
//   Q_c[kflat] = sum_l f_l f_m B[lflat * KC + kflat]
// with the per-dimension index maps of QParams (both index modes).  The grid
// is (k tiles) x (l chunks); every l chunk writes its partial sums and a
// second kernel adds the chunks in a fixed order (deterministic) and applies
// the output permutation of convertQ (:144-155).
//
// Batched FP32 path (many solves sharing one B table, ALIASED mode): see the
// comment above calq32_kernel.
#include <cuda.h>

#include <algorithm>
#include <mutex>
#include <map>
#include <cstring>
#include <vector>

#include "edb_internal.cuh"

namespace edb {

QParams make_qparams(int N, int mode) {
  QParams p;
  p.N = N;
  p.n = (N - 1) / 2;
  p.mode = mode;
  if (mode == EDB_INDEX_REFERENCE) {
    p.P = 2 * p.n + 1;
    p.sL = p.n + 1;
    p.sM = 2 * p.n + 1;
  } else {
    p.P = N;
    p.sL = N - p.n;
    p.sM = 0;
  }
  p.NQ = (long long)N * N * N;
  p.KC = (long long)p.P * p.P * p.P;
  return p;
}

static const int CALQ64_THREADS = 256;

int calq64_nchunk(const QParams &p) {
  long long tiles = (p.KC + CALQ64_THREADS - 1) / CALQ64_THREADS;
  long long want = (4LL * device_sm_count() + tiles - 1) / tiles;
  if (want < 1) want = 1;
  if (want > 64) want = 64;
  if (want > p.NQ) want = p.NQ;
  return (int)want;
}

__global__ void __launch_bounds__(CALQ64_THREADS)
    calq64_kernel(QParams p, long long rows_per_chunk, const double *__restrict__ B,
                  const double2 *__restrict__ fin, double2 *__restrict__ partial) {
  const int N = p.N, P = p.P;
  const long long kc = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int chunk = blockIdx.y;
  const long long r0 = chunk * rows_per_chunk;
  long long r1 = r0 + rows_per_chunk;
  if (r1 > p.NQ) r1 = p.NQ;
  if (kc >= p.KC) return;
  const int j1 = (int)(kc / ((long long)P * P)), j2 = (int)((kc / P) % P), j3 = (int)(kc % P);
  int i1 = (int)(r0 / ((long long)N * N)), i2 = (int)((r0 / N) % N), i3 = (int)(r0 % N);
  // f_l index parts (i + sL) mod N and f_m parts (j - i + sM) mod N
  int a1 = (i1 + p.sL) % N, a2 = (i2 + p.sL) % N, a3 = (i3 + p.sL) % N;
  int b1 = ((j1 - i1 + p.sM) % N + N) % N, b2 = ((j2 - i2 + p.sM) % N + N) % N,
      b3 = ((j3 - i3 + p.sM) % N + N) % N;
  double accr = 0.0, acci = 0.0;
  const double *Bp = B + r0 * p.KC + kc;
  for (long long r = r0; r < r1; ++r) {
    const double2 fl = __ldg(&fin[((long long)a1 * N + a2) * N + a3]);
    const double2 fm = __ldg(&fin[((long long)b1 * N + b2) * N + b3]);
    const double bb = __ldg(Bp);
    Bp += p.KC;
    const double pr = fl.x * fm.x - fl.y * fm.y;
    const double pi = fl.x * fm.y + fl.y * fm.x;
    accr += pr * bb;
    acci += pi * bb;
    // advance i3 (and carry into i2, i1): a_d increments, b_d decrements mod N
    if (++i3 == N) {
      i3 = 0;
      a3 = p.sL % N;
      b3 = (j3 + p.sM) % N;
      if (++i2 == N) {
        i2 = 0;
        a2 = p.sL % N;
        b2 = (j2 + p.sM) % N;
        ++i1;
        a1 = (a1 + 1 == N) ? 0 : a1 + 1;
        b1 = (b1 == 0) ? N - 1 : b1 - 1;
      } else {
        a2 = (a2 + 1 == N) ? 0 : a2 + 1;
        b2 = (b2 == 0) ? N - 1 : b2 - 1;
      }
    } else {
      a3 = (a3 + 1 == N) ? 0 : a3 + 1;
      b3 = (b3 == 0) ? N - 1 : b3 - 1;
    }
  }
  partial[(long long)chunk * p.KC + kc] = make_double2(accr, acci);
}

// Sums the chunks in order and writes Q in FFTW order.  REFERENCE mode
// follows convertQ (:144-155) literally: kq_d = k_d + n if k_d < n+1 else
// k_d - n - 1, flat index with stride N into the (2n+1)^3-filled array.
// ALIASED mode: the centred index of FFTW index k is (k + n) mod N.
__global__ void calq64_reduce_kernel(QParams p, int nchunk, const double2 *__restrict__ partial,
                                     double2 *__restrict__ Q) {
  const int N = p.N, n = p.n;
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= p.NQ) return;
  int k1 = (int)(k / ((long long)N * N)), k2 = (int)((k / N) % N), k3 = (int)(k % N);
  int q1, q2, q3;
  if (p.mode == EDB_INDEX_REFERENCE) {
    q1 = (k1 < n + 1) ? k1 + n : k1 - (n + 1);
    q2 = (k2 < n + 1) ? k2 + n : k2 - (n + 1);
    q3 = (k3 < n + 1) ? k3 + n : k3 - n - 1;
  } else {
    q1 = (k1 + n) % N;
    q2 = (k2 + n) % N;
    q3 = (k3 + n) % N;
  }
  long long q = ((long long)q1 * N + q2) * N + q3;
  double sr = 0.0, si = 0.0;
  if (q < p.KC) {
    for (int c = 0; c < nchunk; ++c) {
      double2 v = partial[(long long)c * p.KC + q];
      sr += v.x;
      si += v.y;
    }
  }
  Q[k] = make_double2(sr, si);
}

edb_status launch_calq64(const QParams &p, const double *d_B, const double2 *d_fin,
                         double2 *d_partial, double2 *d_Q, cudaStream_t st) {
  int nchunk = calq64_nchunk(p);
  long long rows = (p.NQ + nchunk - 1) / nchunk;
  dim3 grid((unsigned)((p.KC + CALQ64_THREADS - 1) / CALQ64_THREADS), (unsigned)nchunk);
  calq64_kernel<<<grid, CALQ64_THREADS, 0, st>>>(p, rows, d_B, d_fin, d_partial);
  EDB_LAUNCHED();
  calq64_reduce_kernel<<<(unsigned)((p.NQ + 255) / 256), 256, 0, st>>>(p, nchunk, d_partial, d_Q);
  EDB_LAUNCHED();
  return EDB_OK;
}

// The ordered chunk reduction and output permutation alone, for the
// double-float kernel (edb_kernels_calq64x.cu), which writes the same partial
// layout.
edb_status launch_calq64_reduce(const QParams &p, int nchunk, const double2 *d_partial,
                                double2 *d_Q, cudaStream_t st) {
  calq64_reduce_kernel<<<(unsigned)((p.NQ + 255) / 256), 256, 0, st>>>(p, nchunk, d_partial, d_Q);
  EDB_LAUNCHED();
  return EDB_OK;
}

// ---------------------------------------------------------------------------
// Batched FP32 kernel (ALIASED mode, many solves sharing one table).
//
// Work: Q^s_K = sum_L B[L][K] f^s_L f^s_((K-L) mod N) for S solves; every index
// in FFTW order.  The terms L and M = K - L carry the same product, so B32 is
// the symmetric pair table B[L][K] + B[M][K] written by genB_kernel, and only
// the l1 planes with l1 <= (k1 - l1) mod N are summed: [0, k1/2] and
// [k1+1, (k1+N)/2], about half of them.  The table holds just those planes,
// laid out [k1][visited line][l3][k2][k3] (c32_table_floats).
//
// CTA = (group of SG = 2 WS solves) x (one k1, a tile of K2T k2 values, all
// k3) x (a chunk of those l1 planes).  Thread = (solve pair {w, w+WS}, k2, run of
// A = 8 or 4 consecutive k3).  WS = 8 (16-solve groups) for throughput; WS = 2
// (4-solve groups) for the few live solves of a serving table.  The CTA walks
// the l-lines (l1, l2) of its chunk in order; for each line it needs
//   B[(l1,l2,l3)][k1, k2-tile, all k3]  N rows of K2T*N floats (the B tile),
//   f^s[l1][l2][:]                       N complex per solve (the f_l line),
//   f^s[m1][:][:], m1 = k1 - l1          the m1-plane, kept while l1 is fixed.
// Tile and line live in NST = 2-4 shared-memory stages.  One warp (rotating
// with the line) issues the TMA copies of line i + NST - 1 (two tensor copies,
// cp.async.bulk.tensor ... mbarrier::complete_tx; or 1-D bulk copies, one per
// row and per solve) while every warp computes line i; a "full" mbarrier per
// stage says the data landed, an "empty" mbarrier per stage (one arrival per
// warp) says every warp is done with it, so warps never wait for each other
// inside an l1-plane.  All waits are bounded: a wait that runs out marks the
// thread, the block leaves together at the next block barrier
// (__syncthreads_or), drains its copies and sets a device status word.
// Widths that are not multiples of 16 bytes or below 8 (N % 4 != 0, N < 8)
// take the same compute path with cooperative plain loads instead of TMA.
//
// Arithmetic, per term and solve, in three packed f32x2 instructions that carry
// the six FP32 operations of the term:
//   q    = (b, b) * f_m                 mul.rn.f32x2
//   accA = (f_l.x, f_l.x) * q + accA    fma.rn.f32x2
//   accB = (f_l.y, f_l.y) * q + accB    fma.rn.f32x2
// so that sum b f_l f_m = (accA.x - accB.y, accA.y + accB.x).  Along l3 the
// needed f_m = f[m1][m2][k3+a-l3] slide down by one, so they live in a ring of A
// registers.  Sums are plain FP32 FMA across FOLD_LINES l-lines (FOLD_LINES * N
// terms per output), then combined and folded into a (hi, lo) two-sum pair:
// blocked compensated summation.
//
// Chunks: with C > 1 the visited l1 planes are split into C consecutive chunks
// so that a few solves still fill the GPU; each chunk writes its (hi, lo) pairs
// and calq32_reduce_kernel adds the chunks in order in FP64 (a chunk may be
// empty: it writes zeros).  The chunk boundaries depend only on (N, C, k1),
// never on S or the variant, so a solve's result does not depend on what else
// is in the batch.
// ---------------------------------------------------------------------------
namespace {
constexpr int SC = 2;                     // solves per thread: w and w + WS
constexpr int ROWPAD = 8;                 // floats after each B-tile row
constexpr int FLPAD = 2;                  // complex after each f_l line
constexpr int PLPAD = 2;                  // complex after each solve's plane
constexpr int FOLD_LINES = 4;             // l-lines per compensated fold
// Limit of the drain after a wait ran out: the block then waits this long at
// most for each copy it issued, so none lands after it exits.
constexpr unsigned long long DRAIN_LIMIT_NS = 1000000000ull;

__device__ int g_calq32_status;  // nonzero: a bounded wait ran out

constexpr int MAX_ST = 4;                 // pipeline stages (l-lines in flight)
// the 128-byte header: (2 MAX_ST + 2) barriers, MAX_ST fill counts, and at
// byte 120 the grouped launch's current work item
static_assert((2 * MAX_ST + 2) * 8 + MAX_ST * 4 <= 120, "shared-memory header");

struct C32Geom {
  int N, A, R, RA, K2T, BROW, FLS, PSTR, NST, NPL, HLT, SG, EL;
  int BSTG, FSTG;  // per-stage sizes: B tile (floats), f_l lines (float2)
  size_t off_B, off_fl, off_pl, off_hl, bytes;
};

// Shared-memory layout for a CTA: NST stages of (B tile, f_l lines), NPL
// m1-planes and, when HLT > 0, the compensated (hi, lo) sums of HLT threads
// (2 * A * SC packed pairs each, thread-fastest so accesses never conflict).
// The first 128 bytes: barriers full[MAX_ST], empty[MAX_ST], plane[2] (80 B),
// then the fill count of each stage, int[MAX_ST] (the abort drain waits for
// each stage's last fill).  SG data units (solves, or
// solve pairs) of EL float2 per element (1: (re, im); 2: (re_a, re_b),
// (im_a, im_b) of a pair).
__host__ __device__ inline C32Geom c32_geom(int N, int A, int K2T, int NST, int NPL, int HLT,
                                            int SG, int EL, bool TMA) {
  C32Geom g;
  g.SG = SG;
  g.EL = EL;
  g.A = A;
  g.N = N;
  g.R = (N + A - 1) / A;
  g.RA = g.R * A;
  g.K2T = K2T;
  g.NST = NST;
  g.NPL = NPL;
  g.HLT = HLT;
  // TMA: tensor copies write dense boxes (B rows of K2T*N floats) to 128-byte
  // aligned stage buffers
  g.BROW = TMA ? K2T * N : K2T * N + ROWPAD;
  if (EL == 1) {
    g.FLS = g.RA + FLPAD;
    g.PSTR = N * N + PLPAD;
  } else {
    // 16-byte pair elements: a row stride of 1 mod 8 elements (4 mod 32
    // words) puts the 8 solve lanes of a quarter-warp on distinct banks
    g.FLS = (g.RA + (9 - g.RA % 8) % 8) * EL;
    g.PSTR = (N * N + (9 - (N * N) % 8) % 8) * EL;
  }
  size_t o = 128;  // 2*MAX_ST + 2 mbarriers, MAX_ST fill counts (+ pad)
  g.BSTG = g.RA * g.BROW;
  g.FSTG = SG * g.FLS;
  if (TMA) {
    g.BSTG = (g.BSTG + 31) / 32 * 32;
    g.FSTG = (g.FSTG + 15) / 16 * 16;
  }
  g.off_B = o;
  o += sizeof(float) * (size_t)NST * g.BSTG;
  g.off_fl = o;
  o += sizeof(float2) * (size_t)NST * g.FSTG;
  g.off_pl = o;
  o += sizeof(float2) * (size_t)NPL * SG * g.PSTR;
  g.off_hl = o;
  o += sizeof(unsigned long long) * 2 * A * SC * (size_t)HLT;
  g.bytes = o;
  return g;
}

__device__ __forceinline__ uint32_t s_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(s_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(s_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(s_addr(bar)) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(s_addr(dst)),
      "l"(src), "r"(bytes), "r"(s_addr(bar))
      : "memory");
}
// Lanes of the calling warp that exist (the last warp of a CTA may be partial).
__device__ __forceinline__ unsigned warp_mask() {
  const int wl = min(32, (int)blockDim.x - (int)(threadIdx.x & ~31u));
  return wl == 32 ? 0xffffffffu : ((1u << wl) - 1u);
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(s_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long gtimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// Wait for the phase with this parity, for at most limit_ns (0: every wait
// runs out at once, without polling).  A thread that already timed out does
// not wait again (its data are discarded at the next block barrier).
__device__ __forceinline__ void mbar_wait(uint64_t *bar, uint32_t parity, bool &to,
                                          unsigned long long limit_ns) {
  if (to) return;
  if (limit_ns == 0) {
    to = true;
    return;
  }
  if (mbar_try_wait(bar, parity)) return;
  const unsigned long long t0 = gtimer_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (gtimer_ns() - t0 >= limit_ns) {
      to = true;
      return;
    }
  }
}

typedef unsigned long long u64;
__device__ __forceinline__ u64 pk(float a, float b) {
  u64 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
// Shared-memory loads by 32-bit shared address (explicit ld.shared, so no
// generic-address resolution in the inner loops)
__device__ __forceinline__ u64 lds_u64(uint32_t a) {
  u64 v;
  asm volatile("ld.shared.u64 %0, [%1];" : "=l"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ ulonglong2 lds_u64x2(uint32_t a) {
  ulonglong2 v;
  asm volatile("ld.shared.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "r"(a));
  return v;
}
__device__ __forceinline__ float4 lds_f4(uint32_t a) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(a));
  return v;
}
__device__ __forceinline__ float lds_f32(uint32_t a) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ float2 lds_f2(uint32_t a) {
  float2 v;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
  return v;
}
__device__ __forceinline__ float2 upk(u64 v) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
__device__ __forceinline__ u64 mul2(u64 a, u64 b) {
  u64 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ void fma2(u64 &acc, u64 a, u64 b) {
  asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(acc) : "l"(a), "l"(b));
}
__device__ __forceinline__ u64 fma2r(u64 a, u64 b, u64 c) {
  u64 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ u64 add2(u64 a, u64 b) {
  u64 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ u64 sub2(u64 a, u64 b) {
  u64 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
// (x.y, x.x)
__device__ __forceinline__ u64 swp(u64 v) {
  float2 f = upk(v);
  return pk(f.y, f.x);
}
// Two-sum fold of a packed pair of partial sums into packed (hi, lo).
__device__ __forceinline__ void two_sum_fold2(u64 &hi, u64 &lo, u64 x) {
  const u64 s = add2(hi, x);
  const u64 bb = sub2(s, hi);
  const u64 e = add2(sub2(hi, sub2(s, bb)), sub2(x, bb));
  hi = s;
  lo = add2(lo, e);
}


// Tensor copies (one elected thread): the B tile of a line is one 5-D box
// {k3: N, k2: K2T, l3: N, line: 1, k1: 1} of the pair table, stored as
// [k1][visited line][l3][k2][k3] so the tile's rows lie within N^3 floats;
// the f_l lines of the group are one 3-D box
// {FLS floats x 2, 1 line, SG units} of the input viewed as [unit][line][l3],
// whose columns past N*EL complex are out of bounds and land as zeros.
__device__ __forceinline__ void tma_load_5d(void *dst, const CUtensorMap *tm, int c0, int c1,
                                            int c2, int c3, int c4, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(s_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4),
      "r"(s_addr(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *tm, int c0, int c1,
                                            int c2, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(s_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1), "r"(c2), "r"(s_addr(bar))
      : "memory");
}

// Issue (TMA: one whole warp; tensor copies from its lane 0, or one bulk copy
// per B row and f_l line from each lane) or perform (plain: all threads) the
// staging of the B tile and f_l line of line li into buffer `st`; vl is the
// line's index in k1's visited list (its row block of the pair table).
template <bool TMA>
__device__ __forceinline__ void stage_line(const C32Geom &g, int li, int vl, int st, int k1,
                                           int k2_0,
                                           int k2n, int s0, int nval, long long NQ,
                                           const float *__restrict__ B32,
                                           const float2 *__restrict__ fin, float *Bs,
                                           float2 *fls, uint64_t *full, bool tmap,
                                           const CUtensorMap *tmB, const CUtensorMap *tmF) {
  const int N = g.N;
  float *Bd = Bs + (size_t)st * g.BSTG;
  float2 *fd = fls + (size_t)st * g.FSTG;
  // table layout [k1][visited line][l3][k2][k3]: the tile's rows l3 are N^2 apart
  const float *Bsrc =
      B32 + ((long long)k1 * c32_maxlist(N) * N + vl) * NQ + (long long)k2_0 * N;
  const long long NN = (long long)N * N;
  const int EL = g.EL;  // s0 / nval count data units of EL float2 per element
  const float2 *fsrc = fin + ((long long)s0 * NQ + (long long)li * N) * EL;
  const int rowlen = k2n * N;
  if (TMA && tmap) {  // called by the issuing warp only
    if ((threadIdx.x & 31) == 0) {
      mbar_expect_tx(full + st, (uint32_t)(N * g.K2T * N * 4 + g.SG * g.FLS * 8));
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tma_load_5d(Bd, tmB, 0, k2_0, 0, vl, k1, full + st);
      tma_load_3d(fd, tmF, 0, li, s0, full + st);
    }
    __syncwarp(warp_mask());
  } else if (TMA) {  // called by the issuing warp only (a full warp)
    const int lane = threadIdx.x & 31;
    if (lane == 0) mbar_expect_tx(full + st, (uint32_t)(N * rowlen * 4 + nval * N * 8 * EL));
    __syncwarp(warp_mask());
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    for (int l3 = lane; l3 < N; l3 += 32)
      bulk_g2s(Bd + (size_t)l3 * g.BROW, Bsrc + (long long)l3 * NN, rowlen * 4, full + st);
    for (int s = lane; s < nval; s += 32)
      bulk_g2s(fd + (size_t)s * g.FLS, fsrc + (long long)s * NQ * EL, N * 8 * EL, full + st);
  } else {
    for (int e = threadIdx.x; e < N * rowlen; e += blockDim.x) {
      int l3 = e / rowlen, c = e % rowlen;
      Bd[(size_t)l3 * g.BROW + c] = __ldg(Bsrc + (long long)l3 * NN + c);
    }
    for (int e = threadIdx.x; e < nval * N * EL; e += blockDim.x) {
      int s = e / (N * EL), j = e % (N * EL);
      fd[(size_t)s * g.FLS + j] = __ldg(fsrc + (long long)s * NQ * EL + j);
    }
  }
}

template <bool TMA>
__device__ __forceinline__ void stage_plane(const C32Geom &g, int m1, int s0, int nval,
                                            long long NQ, const float2 *__restrict__ fin,
                                            float2 *pl, uint64_t *bar) {
  const int NN = g.N * g.N, EL = g.EL;
  const float2 *src = fin + ((long long)s0 * NQ + (long long)m1 * NN) * EL;
  if (TMA) {  // warp 0 only
    const int lane = threadIdx.x & 31;
    if (lane == 0) mbar_expect_tx(bar, (uint32_t)(nval * NN * 8 * EL));
    __syncwarp(warp_mask());
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    for (int s = lane; s < nval; s += 32)
      bulk_g2s(pl + (size_t)s * g.PSTR, src + (long long)s * NQ * EL, NN * 8 * EL, bar);
  } else {
    for (int e = threadIdx.x; e < nval * NN * EL; e += blockDim.x) {
      int s = e / (NN * EL), p = e % (NN * EL);
      pl[(size_t)s * g.PSTR + p] = __ldg(src + (long long)s * NQ * EL + p);
    }
  }
}

// One l-line for this thread: A outputs x SC solves.  BIGN: N >= A, so one
// conditional add brings a ring index back into [0, N).  VEC: N % 4 == 0, so
// every B-tile row offset is 16-byte aligned and B is read with float4 loads;
// otherwise with scalar loads.  Each output's sum runs over l3 in order
// whatever A is, so every A gives the same bits.
template <bool BIGN, bool VEC, int A>
__device__ __forceinline__ void compute_line(const C32Geom &g, const float *Bt, const float2 *fl0,
                                             const float2 *fl1, const float2 *p0,
                                             const float2 *p1, int k3_0, u64 (&accA)[A][SC],
                                             u64 (&accB)[A][SC]) {
  const int N = g.N;
  const uint32_t sp0 = s_addr(p0), sp1 = s_addr(p1), sf0 = s_addr(fl0), sf1 = s_addr(fl1);
  const uint32_t sB = s_addr(Bt), brow = 4u * g.BROW;
  u64 ring[A][SC];
#pragma unroll
  for (int a = 0; a < A; ++a) {
    int idx = k3_0 + a;
    if (BIGN) {
      idx -= (idx >= N) ? N : 0;
    } else {
      while (idx >= N) idx -= N;
    }
    ring[a][0] = lds_u64(sp0 + 8u * idx);
    ring[a][1] = lds_u64(sp1 + 8u * idx);
  }
  for (int gg = 0; gg < g.R; ++gg) {
    int base = k3_0 - gg * A;
    if (BIGN) {
      base += (base < 0) ? N : 0;
    } else {
      while (base < 0) base += N;
    }
#pragma unroll
    for (int t = 0; t < A; ++t) {
      const int l3 = gg * A + t;
      if (t > 0 || gg > 0) {
        int idx = base - t;
        if (BIGN) {
          idx += (idx < 0) ? N : 0;
        } else {
          while (idx < 0) idx += N;
        }
        const int slot = (A - t) % A;
        ring[slot][0] = lds_u64(sp0 + 8u * idx);
        ring[slot][1] = lds_u64(sp1 + 8u * idx);
      }
      float bv[A];
      if (VEC) {
#pragma unroll
        for (int q4 = 0; q4 < A / 4; ++q4) {
          const float4 b = lds_f4(sB + brow * l3 + 16u * q4);
          bv[4 * q4] = b.x;
          bv[4 * q4 + 1] = b.y;
          bv[4 * q4 + 2] = b.z;
          bv[4 * q4 + 3] = b.w;
        }
      } else {
#pragma unroll
        for (int a = 0; a < A; ++a) bv[a] = lds_f32(sB + brow * l3 + 4u * a);
      }
      const float2 f0 = lds_f2(sf0 + 8u * l3), f1 = lds_f2(sf1 + 8u * l3);
      const u64 flx[SC] = {pk(f0.x, f0.x), pk(f1.x, f1.x)};
      const u64 fly[SC] = {pk(f0.y, f0.y), pk(f1.y, f1.y)};
#pragma unroll
      for (int a = 0; a < A; ++a) {
        const int slot = (a - t + A) % A;
        const u64 bb = pk(bv[a], bv[a]);
#pragma unroll
        for (int c = 0; c < SC; ++c) {
          const u64 q = mul2(bb, ring[slot][c]);
          fma2(accA[a][c], flx[c], q);
          fma2(accB[a][c], fly[c], q);
        }
      }
    }
  }
}

// compute_line for a solve pair (PAIR layout: element = (re_a, re_b),
// (im_a, im_b)).  The packed lanes are the two solves, so f_l and f_m need no
// broadcast and one 16-byte load brings both components of both solves.  The
// four sums per output keep the per-solve operation order of compute_line:
//   accA[a][0] = sum f_l.re q.re    accA[a][1] = sum f_l.re q.im
//   accB[a][0] = sum f_l.im q.re    accB[a][1] = sum f_l.im q.im
// (lanes = solves), so both layouts give the same bits.
template <bool BIGN, bool VEC, int A>
__device__ __forceinline__ void compute_line_pair(const C32Geom &g, const float *Bt,
                                                  const float2 *fl, const float2 *p, int k3_0,
                                                  u64 (&accA)[A][SC], u64 (&accB)[A][SC]) {
  const int N = g.N;
  const uint32_t sp = s_addr(p), sf = s_addr(fl), sB = s_addr(Bt), brow = 4u * g.BROW;
  ulonglong2 ring[A];
#pragma unroll
  for (int a = 0; a < A; ++a) {
    int idx = k3_0 + a;
    if (BIGN) {
      idx -= (idx >= N) ? N : 0;
    } else {
      while (idx >= N) idx -= N;
    }
    ring[a] = lds_u64x2(sp + 16u * idx);
  }
  for (int gg = 0; gg < g.R; ++gg) {
    int base = k3_0 - gg * A;
    if (BIGN) {
      base += (base < 0) ? N : 0;
    } else {
      while (base < 0) base += N;
    }
#pragma unroll
    for (int t = 0; t < A; ++t) {
      const int l3 = gg * A + t;
      if (t > 0 || gg > 0) {
        int idx = base - t;
        if (BIGN) {
          idx += (idx < 0) ? N : 0;
        } else {
          while (idx < 0) idx += N;
        }
        ring[(A - t) % A] = lds_u64x2(sp + 16u * idx);
      }
      float bv[A];
      if (VEC) {
#pragma unroll
        for (int q4 = 0; q4 < A / 4; ++q4) {
          const float4 b = lds_f4(sB + brow * l3 + 16u * q4);
          bv[4 * q4] = b.x;
          bv[4 * q4 + 1] = b.y;
          bv[4 * q4 + 2] = b.z;
          bv[4 * q4 + 3] = b.w;
        }
      } else {
#pragma unroll
        for (int a = 0; a < A; ++a) bv[a] = lds_f32(sB + brow * l3 + 4u * a);
      }
      const ulonglong2 f = lds_u64x2(sf + 16u * l3);
#pragma unroll
      for (int a = 0; a < A; ++a) {
        const ulonglong2 m = ring[(a - t + A) % A];
        const u64 bb = pk(bv[a], bv[a]);
        const u64 qr = mul2(bb, m.x), qi = mul2(bb, m.y);
        fma2(accA[a][0], f.x, qr);
        fma2(accA[a][1], f.x, qi);
        fma2(accB[a][0], f.y, qr);
        fma2(accB[a][1], f.y, qi);
      }
    }
  }
}

// compute_line and compute_line_pair for N % A == 0 on the tensor-copy path:
// the same operations in the same order (so the same bits), with the shared-
// memory addresses built once per group of A l3 steps.  At group gg the
// ring's base index (k3_0 - gg A) mod N is a multiple of A, so for t >= 1 the
// new ring entry sits at qq - t with qq = base (N when base = 0) and needs no
// wrap; the B-tile row pointer advances by one row pitch per l3 step.  With
// the per-step index wrap and the row multiply gone, fewer integer
// multiply-adds compete with the packed math for the FMA pipe.
// RC > 0: N = RC A known at compile time (the workload sizes, see
// compute_line_al_n); the line's RC groups are then unrolled, so loads of one
// group are scheduled under the arithmetic of the one before (4096 x N = 24:
// 104 -> 99 ms).
template <int A, int RC = 0>
__device__ __forceinline__ void compute_line_al(const C32Geom &g, const float *Bt,
                                                const float2 *fl0, const float2 *fl1,
                                                const float2 *p0, const float2 *p1, int k3_0,
                                                u64 (&accA)[A][SC], u64 (&accB)[A][SC]) {
  const int N = RC > 0 ? RC * A : g.N;
  const uint32_t sp0 = s_addr(p0), sp1 = s_addr(p1);
  uint32_t sf0 = s_addr(fl0), sf1 = s_addr(fl1), bB = s_addr(Bt);
  const uint32_t brow = 4u * g.BROW;
  // f-hat values move in 16-byte pairs: every plane row, line and stage
  // offset is an even number of complex values here (N % 4 == 0, even
  // paddings), so pair loads are aligned.  A quarter-warp's 8 solve lanes then
  // hit 8 distinct 16-byte bank groups (plane pitch N^2 + 2 complex = an odd
  // number of pairs), where single-value loads of two windows 4 apart met
  // pairwise in the same banks.
  u64 ring[A][SC];
  {
    const uint32_t a0 = sp0 + 8u * k3_0, a1 = sp1 + 8u * k3_0;
#pragma unroll
    for (int a = 0; a < A; a += 2) {
      const ulonglong2 v0 = lds_u64x2(a0 + 8u * a), v1 = lds_u64x2(a1 + 8u * a);
      ring[a][0] = v0.x;
      ring[a + 1][0] = v0.y;
      ring[a][1] = v1.x;
      ring[a + 1][1] = v1.y;
    }
  }
  u64 held[SC] = {0ull, 0ull};  // f_m at qq - t for the next even step (or next group's t = 0)
  int base = k3_0;
#pragma unroll(RC > 0 ? RC : 1)
  for (int gg = 0; gg < (RC > 0 ? RC : g.R); ++gg) {
    const int qq = base == 0 ? N : base;
    const uint32_t qa = sp0 + 8u * qq, qb = sp1 + 8u * qq;
    ulonglong2 fp0 = make_ulonglong2(0ull, 0ull), fp1 = fp0;  // f_l of steps (t, t + 1)
#pragma unroll
    for (int t = 0; t < A; ++t) {
      // the ring entry of step t: f_m at qq - t (t = 0: base, held over)
      if (t == 0) {
        if (gg > 0) {
          ring[0][0] = held[0];
          ring[0][1] = held[1];
        }
      } else if (t & 1) {  // pair (qq - t - 1, qq - t)
        const ulonglong2 v0 = lds_u64x2(qa - 8u * (t + 1)), v1 = lds_u64x2(qb - 8u * (t + 1));
        ring[(A - t) % A][0] = v0.y;
        ring[(A - t) % A][1] = v1.y;
        held[0] = v0.x;
        held[1] = v1.x;
      } else {
        ring[(A - t) % A][0] = held[0];
        ring[(A - t) % A][1] = held[1];
      }
      float bv[A];
#pragma unroll
      for (int q4 = 0; q4 < A / 4; ++q4) {
        const float4 b = lds_f4(bB + 16u * q4);
        bv[4 * q4] = b.x;
        bv[4 * q4 + 1] = b.y;
        bv[4 * q4 + 2] = b.z;
        bv[4 * q4 + 3] = b.w;
      }
      bB += brow;
      if ((t & 1) == 0) {
        fp0 = lds_u64x2(sf0 + 8u * t);
        fp1 = lds_u64x2(sf1 + 8u * t);
      }
      const float2 f0 = upk((t & 1) ? fp0.y : fp0.x), f1 = upk((t & 1) ? fp1.y : fp1.x);
      const u64 flx[SC] = {pk(f0.x, f0.x), pk(f1.x, f1.x)};
      const u64 fly[SC] = {pk(f0.y, f0.y), pk(f1.y, f1.y)};
#pragma unroll
      for (int a = 0; a < A; ++a) {
        const int slot = (a - t + A) % A;
        const u64 bb = pk(bv[a], bv[a]);
#pragma unroll
        for (int c = 0; c < SC; ++c) {
          const u64 q = mul2(bb, ring[slot][c]);
          fma2(accA[a][c], flx[c], q);
          fma2(accB[a][c], fly[c], q);
        }
      }
    }
    sf0 += 8u * A;
    sf1 += 8u * A;
    base -= A;
    if (base < 0) base += N;
  }
}

template <int A, int RC = 0>
__device__ __forceinline__ void compute_line_pair_al(const C32Geom &g, const float *Bt,
                                                     const float2 *fl, const float2 *p, int k3_0,
                                                     u64 (&accA)[A][SC], u64 (&accB)[A][SC]) {
  const int N = RC > 0 ? RC * A : g.N;
  const uint32_t sp = s_addr(p);
  uint32_t sf = s_addr(fl), bB = s_addr(Bt);
  const uint32_t brow = 4u * g.BROW;
  ulonglong2 ring[A];
  {
    const uint32_t a0 = sp + 16u * k3_0;
#pragma unroll
    for (int a = 0; a < A; ++a) ring[a] = lds_u64x2(a0 + 16u * a);
  }
  int base = k3_0;
#pragma unroll(RC > 0 ? RC : 1)
  for (int gg = 0; gg < (RC > 0 ? RC : g.R); ++gg) {
    const int qq = base == 0 ? N : base;
    const uint32_t t0 = sp + 16u * base, qa = sp + 16u * qq;
#pragma unroll
    for (int t = 0; t < A; ++t) {
      if (t > 0)
        ring[(A - t) % A] = lds_u64x2(qa - 16u * t);
      else if (gg > 0)
        ring[0] = lds_u64x2(t0);
      float bv[A];
#pragma unroll
      for (int q4 = 0; q4 < A / 4; ++q4) {
        const float4 b = lds_f4(bB + 16u * q4);
        bv[4 * q4] = b.x;
        bv[4 * q4 + 1] = b.y;
        bv[4 * q4 + 2] = b.z;
        bv[4 * q4 + 3] = b.w;
      }
      bB += brow;
      const ulonglong2 f = lds_u64x2(sf + 16u * t);
#pragma unroll
      for (int a = 0; a < A; ++a) {
        const ulonglong2 m = ring[(a - t + A) % A];
        const u64 bb = pk(bv[a], bv[a]);
        const u64 qr = mul2(bb, m.x), qi = mul2(bb, m.y);
        fma2(accA[a][0], f.x, qr);
        fma2(accA[a][1], f.x, qi);
        fma2(accB[a][0], f.y, qr);
        fma2(accB[a][1], f.y, qi);
      }
    }
    sf += 16u * A;
    base -= A;
    if (base < 0) base += N;
  }
}

// The aligned lines with N fixed at compile time for the workload sizes
// N = 16, 24, 32 (the serving mix and the uniform batch), generic otherwise.
// The branch is uniform over the CTA.
template <int A>
__device__ __forceinline__ void compute_line_al_n(const C32Geom &g, const float *Bt,
                                                  const float2 *fl0, const float2 *fl1,
                                                  const float2 *p0, const float2 *p1, int k3_0,
                                                  u64 (&accA)[A][SC], u64 (&accB)[A][SC]) {
  if (g.N == 24)
    compute_line_al<A, 24 / A>(g, Bt, fl0, fl1, p0, p1, k3_0, accA, accB);
  else if (g.N == 32)
    compute_line_al<A, 32 / A>(g, Bt, fl0, fl1, p0, p1, k3_0, accA, accB);
  else if (g.N == 16)
    compute_line_al<A, 16 / A>(g, Bt, fl0, fl1, p0, p1, k3_0, accA, accB);
  else
    compute_line_al<A>(g, Bt, fl0, fl1, p0, p1, k3_0, accA, accB);
}
template <int A>
__device__ __forceinline__ void compute_line_pair_al_n(const C32Geom &g, const float *Bt,
                                                       const float2 *fl, const float2 *p,
                                                       int k3_0, u64 (&accA)[A][SC],
                                                       u64 (&accB)[A][SC]) {
  if (g.N == 24)
    compute_line_pair_al<A, 24 / A>(g, Bt, fl, p, k3_0, accA, accB);
  else if (g.N == 32)
    compute_line_pair_al<A, 32 / A>(g, Bt, fl, p, k3_0, accA, accB);
  else if (g.N == 16)
    compute_line_pair_al<A, 16 / A>(g, Bt, fl, p, k3_0, accA, accB);
  else
    compute_line_pair_al<A>(g, Bt, fl, p, k3_0, accA, accB);
}

// Solve pairs for the PAIR variants: out[P][e] = (re_2P, re_2P+1, im_2P,
// im_2P+1); a missing odd partner reads as zero.
__global__ void c32_pairs_kernel(int S, long long NQ, const float2 *__restrict__ fin,
                                 float4 *__restrict__ out) {
  const long long n = (long long)((S + 1) / 2) * NQ;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long P = i / NQ, e = i - P * NQ;
    const float2 a = __ldg(fin + 2 * P * NQ + e);
    const float2 b = (2 * P + 1 < S) ? __ldg(fin + (2 * P + 1) * NQ + e) : make_float2(0.f, 0.f);
    out[i] = make_float4(a.x, b.x, a.y, b.y);
  }
}
}  // namespace

// MAXT bounds the CTA size: 256 threads keep at most two warps per SM
// sub-partition, so up to 255 registers per thread; 384 allow more warps at
// 168 registers.  HLS: keep the compensated (hi, lo) pairs in shared memory
// instead of registers, which frees 64 registers per thread for more resident
// warps.  WS: solve lanes (group of 2 WS solves).  PAIR: fin is in the
// solve-pair layout (c32_pairs_kernel) and lane w holds solves 2w, 2w+1 of
// the group; otherwise fin is plain and lane w holds solves w, w+WS.  The
// autotuner picks the variant per (table, S).
// The work of one CTA: CTA number lin of a grid of U x GY x GZ = (solve
// groups x chunks, N, k2 tiles) CTAs over one table (see calq32_kernel).
// Returns false when a bounded wait ran out (the CTA drained its copies and
// set the status word); every thread returns at the same point.
template <bool TMA, int MAXT, bool HLS, int WS, int A, int MINB, bool PAIR>
__device__ __forceinline__ bool calq32_cta(int N, int S, int K2T, int NST, int NPL, int C, int GB,
                                           const float *__restrict__ B32,
                                           const float2 *__restrict__ fin,
                                           float2 *__restrict__ Q, float4 *__restrict__ partial,
                                           int tmap, unsigned long long wait_ns,
                                           const CUtensorMap *tmB, const CUtensorMap *tmF, int U,
                                           int GY, int GZ, long long lin, int nthr) {
  constexpr int SG = SC * WS;  // solves per group
  extern __shared__ __align__(128) unsigned char smem[];
  const C32Geom g =
      c32_geom(N, A, K2T, NST, NPL, HLS ? (int)blockDim.x : 0, PAIR ? WS : SG, PAIR ? 2 : 1,
               TMA && tmap);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);  // [MAX_ST]
  uint64_t *empty = full + MAX_ST;                       // [MAX_ST]
  uint64_t *pbar = full + 2 * MAX_ST;                    // [2] planes
  int *fills = reinterpret_cast<int *>(pbar + 2);        // [MAX_ST] copies issued per stage
  float *Bs = reinterpret_cast<float *>(smem + g.off_B);
  float2 *fls = reinterpret_cast<float2 *>(smem + g.off_fl);
  float2 *plb = reinterpret_cast<float2 *>(smem + g.off_pl);
  const long long NQ = (long long)N * N * N;
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int nwarps = (blockDim.x + 31) >> 5;
  const int nfull = max(1, (int)blockDim.x / 32);  // warps with 32 lanes
  const int w = tid % WS;
  const int rest = tid / WS;
  const int r = rest % g.R;
  const int k2l = rest / g.R;
  // CTA -> (unit = solve group x chunk, k1, k2 tile).  Blocks of GB units walk
  // every (k1, tile) before the next block starts, so a block's f-hat stays in
  // L2 while the table streams once per block (the grid is (units, N, tiles)).
  const int NT = GY * GZ;
  const int blk = (int)(lin / ((long long)GB * NT));
  const int gsz = min(GB, U - blk * GB);
  const long long off = lin - (long long)blk * GB * NT;
  const int kt = (int)(off / gsz);
  const int unit = blk * GB + (int)(off % gsz);
  const int k1 = kt % GY;
  const int k2_0 = (kt / GY) * K2T;
  const int k2n = min(K2T, N - k2_0);
  const int k2 = k2_0 + k2l;
  // threads past nthr (a grouped launch's block is its largest table's) take
  // part in the barriers only
  const bool act = tid < nthr;
  const bool k_ok = act && (k2l < k2n);
  const int k2c = k_ok ? k2 : k2_0;
  const int k3_0 = r * A;
  const int chunk = unit % C;
  const int s0 = (unit / C) * SG;
  // staged data units (solves, or solve pairs) of this group
  const int u0 = PAIR ? s0 / 2 : s0;
  const int nval = PAIR ? min(WS, (S - s0 + 1) / 2) : min(SG, S - s0);
  // The table is the symmetric pair table (see genB_kernel): only the l1
  // planes with l1 <= m1 = (k1 - l1) mod N are visited, in increasing l1:
  // [0, k1 / 2] and [k1 + 1, (k1 + N) / 2].  Plane p of that list is
  // l1 = plane_l1(p).  This chunk takes list entries [P0, P1) and walks their
  // l-lines j = 0 .. nlines - 1 (line j: plane P0 + j / N, l2 = j mod N).
  const int plo = k1 / 2;
  const int nlist = c32_nlist(N, k1);
  auto plane_l1 = [&](int p) { return p <= plo ? p : k1 + 1 + (p - plo - 1); };
  const int PPC = (nlist + C - 1) / C;
  const int P0 = min(nlist, chunk * PPC), P1 = min(nlist, P0 + PPC);
  const int nplanes = P1 - P0;
  const int nlines = nplanes * N;
  auto line_li = [&](int j) { return plane_l1(P0 + j / N) * N + j % N; };
  const size_t plane_sz = (size_t)g.SG * g.PSTR;
  const bool ring_al = (N % A) == 0;  // compute_line*_al apply (tensor-copy path)
  // the compile-time-N lines, except in the solve-pair variants under the
  // 128-register cap or with the sums in shared memory (there they spill more)
  constexpr bool FIXN = !(PAIR && (MINB == 2 || HLS));

  // zero the tile/line buffers once: padded rows (l3 >= N), row tails and the
  // f_l tails are never written by the copies and must read as zeros
  {
    const size_t nz = ((size_t)(g.off_pl - g.off_B)) / sizeof(float);
    for (size_t e = tid; e < nz; e += blockDim.x) Bs[e] = 0.f;
  }
  if (tid == 0) {
    for (int i = 0; i < MAX_ST; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], nwarps);
    }
    mbar_init(&pbar[0], 1);
    mbar_init(&pbar[1], 1);
    for (int i = 0; i < MAX_ST; ++i) fills[i] = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  u64 accA[A][SC], accB[A][SC];            // packed (re, im) partial sums
  u64 hi[HLS ? 1 : A][SC], lo[HLS ? 1 : A][SC];  // compensated sums (registers)
  u64 *hl = reinterpret_cast<u64 *>(smem + g.off_hl);  // or [2*A*SC][threads] in smem
#pragma unroll
  for (int a = 0; a < A; ++a)
#pragma unroll
    for (int c = 0; c < SC; ++c) {
      accA[a][c] = 0ull;
      accB[a][c] = 0ull;
      if (HLS) {
        hl[(size_t)(2 * (a * SC + c)) * blockDim.x + tid] = 0ull;
        hl[(size_t)(2 * (a * SC + c) + 1) * blockDim.x + tid] = 0ull;
      } else {
        hi[HLS ? 0 : a][c] = 0ull;
        lo[HLS ? 0 : a][c] = 0ull;
      }
    }
  const u64 neg_re = pk(-1.f, 1.f), neg_one = pk(-1.f, -1.f);

  // Pipeline bookkeeping uses chunk-relative indices: j (line), pr (plane).
  // prologue: lines 0 .. NST-2 and the first plane
  int planes = 0;       // counted in warp 0
  if (TMA && warp == 0 && nlines > 0) {
    for (int j = 0; j < NST - 1 && j < nlines; ++j) {
      stage_line<true>(g, line_li(j), P0 * N + j, j % NST, k1, k2_0, k2n, u0, nval, NQ, B32, fin, Bs, fls,
                       full, tmap, tmB, tmF);
      if (lane == 0) ++fills[j % NST];
    }
    stage_plane<true>(g, (k1 - plane_l1(P0) + N) % N, u0, nval, NQ, fin, plb, &pbar[0]);
    ++planes;
  }
  bool to = false;
  bool aborted = false;
  // Line j = pr N + l2 of the chunk (plane l1 = plane_l1(P0 + pr)) in stage
  // st = j mod NST, fill parity fpar = (j / NST) & 1, and m2 = (k2c - l2) mod N
  // are advanced by counters at the end of each line, as is the issuing warp
  // iw = jn mod nfull of the refill line jn = j + NST - 1: no integer
  // division in the line loop.
  int l2 = 0, pr = 0, st = 0, fpar = 0, m2 = k2c;
  int l1 = nlines > 0 ? plane_l1(P0) : 0;
  int iw = (NST - 1) % nfull;
  for (int j = 0; j < nlines; ++j) {
    const int pb = (NPL == 2) ? (pr & 1) : 0;
    if (l2 == 0) {
      // every warp is done with the previous plane (and with its buffer)
      if (__syncthreads_or(to)) {
        aborted = true;
        break;
      }
      if (TMA) {
        if (NPL == 2) {
          if (warp == 0 && pr + 1 < nplanes) {
            stage_plane<true>(g, (k1 - plane_l1(P0 + pr + 1) + N) % N, u0, nval, NQ, fin,
                              plb + (size_t)((pr + 1) & 1) * plane_sz, &pbar[(pr + 1) & 1]);
            ++planes;
          }
          mbar_wait(&pbar[pr & 1], (uint32_t)((pr >> 1) & 1), to, wait_ns);
        } else {
          if (warp == 0 && pr > 0) {
            stage_plane<true>(g, (k1 - l1 + N) % N, u0, nval, NQ, fin, plb, &pbar[0]);
            ++planes;
          }
          mbar_wait(&pbar[0], (uint32_t)(pr & 1), to, wait_ns);
        }
      } else {
        stage_plane<false>(g, (k1 - l1 + N) % N, u0, nval, NQ, fin, plb, pbar);
      }
    }
    if (TMA) {
      // refill: line j+NST-1 goes into the stage line j-1 used.  The issuing
      // warp rotates over the full warps with the line, so the issue work
      // (and the wait for every warp to leave line j-1) does not make one warp
      // fall behind the rest.  Once one of its lanes has timed out the warp
      // issues nothing more: the stage's previous copy may still be landing.
      const int jn = j + NST - 1;
      if (warp == iw && jn < nlines) {
        // stage of line j - 1, whose fill (j - 1) / NST completes parity
        // fpar, or fpar ^ 1 when line j starts a new round of stages
        const int sn = st == 0 ? NST - 1 : st - 1;
        if (j >= 1) mbar_wait(&empty[sn], (uint32_t)(st > 0 ? fpar : fpar ^ 1), to, wait_ns);
        if (!__any_sync(warp_mask(), to)) {
          // line jn is row l2 + NST - 1 of plane pr, or of plane pr + 1 (NST <= N)
          int l2n = l2 + NST - 1, prn = pr;
          if (l2n >= N) {
            l2n -= N;
            ++prn;
          }
          stage_line<true>(g, plane_l1(P0 + prn) * N + l2n, P0 * N + jn, sn, k1, k2_0, k2n, u0,
                           nval, NQ, B32, fin, Bs, fls, full, tmap, tmB, tmF);
          if (lane == 0) ++fills[sn];
        }
      }
      mbar_wait(&full[st], (uint32_t)fpar, to, wait_ns);
    } else {
      __syncthreads();  // previous line's readers are done (single buffer)
      stage_line<false>(g, l1 * N + l2, P0 * N + j, st, k1, k2_0, k2n, u0, nval, NQ, B32, fin, Bs,
                        fls, full, tmap, tmB, tmF);
      __syncthreads();
    }

    // ---- compute line (l1, l2)
    if (act) {
    const float *Bt = Bs + (size_t)st * g.BSTG + k2l * N + k3_0;
    const float2 *fl0 = fls + (size_t)st * g.FSTG + (size_t)w * g.FLS;
    const float2 *p0 = plb + (size_t)pb * plane_sz + (size_t)w * g.PSTR + m2 * N * g.EL;
    if (PAIR) {
      if (TMA && ring_al && FIXN)
        compute_line_pair_al_n<A>(g, Bt, fl0, p0, k3_0, accA, accB);
      else if (TMA && ring_al)
        compute_line_pair_al<A>(g, Bt, fl0, p0, k3_0, accA, accB);
      else if (TMA)
        compute_line_pair<true, true, A>(g, Bt, fl0, p0, k3_0, accA, accB);
      else
        compute_line_pair<false, false, A>(g, Bt, fl0, p0, k3_0, accA, accB);
    } else {
      const float2 *fl1 = fl0 + (size_t)WS * g.FLS;
      const float2 *p1 = p0 + (size_t)WS * g.PSTR;
      if (TMA && ring_al && FIXN)
        compute_line_al_n<A>(g, Bt, fl0, fl1, p0, p1, k3_0, accA, accB);
      else if (TMA && ring_al)
        compute_line_al<A>(g, Bt, fl0, fl1, p0, p1, k3_0, accA, accB);
      else if (TMA)
        compute_line<true, true, A>(g, Bt, fl0, fl1, p0, p1, k3_0, accA, accB);
      else
        compute_line<false, false, A>(g, Bt, fl0, fl1, p0, p1, k3_0, accA, accB);
    }
    }
    if (TMA) {
      // a warp releases the stage only when every lane saw this line's copy
      // land, so a stage is refilled only after its previous copy completed
      // (at most one copy per stage is ever in flight)
      const bool bad = __any_sync(warp_mask(), to);
      if (lane == 0 && !bad) mbar_arrive(&empty[st]);
    }
    if ((l2 + 1) % FOLD_LINES == 0 || l2 == N - 1) {  // fold into the compensated pair
#pragma unroll
      for (int a = 0; a < A; ++a) {
        // (accA.x - accB.y, accA.y + accB.x) = accA + (-1, 1) * swap(accB);
        // PAIR: xs[0] the real parts, xs[1] the imaginary parts of both solves
        u64 xs[SC];
#pragma unroll
        for (int c = 0; c < SC; ++c)
          xs[c] = !PAIR ? fma2r(neg_re, swp(accB[a][c]), accA[a][c])
                  : c == 0 ? fma2r(neg_one, accB[a][1], accA[a][0])
                           : add2(accA[a][1], accB[a][0]);
#pragma unroll
        for (int c = 0; c < SC; ++c) {
          const u64 x = xs[c];
          if (HLS) {
            u64 *ph = hl + (size_t)(2 * (a * SC + c)) * blockDim.x + tid;
            u64 h = ph[0], l = ph[blockDim.x];
            two_sum_fold2(h, l, x);
            ph[0] = h;
            ph[blockDim.x] = l;
          } else {
            two_sum_fold2(hi[HLS ? 0 : a][c], lo[HLS ? 0 : a][c], x);
          }
          accA[a][c] = 0ull;
          accB[a][c] = 0ull;
        }
      }
    }
    // advance the line counters
    if (++st == NST) {
      st = 0;
      fpar ^= 1;
    }
    if (++l2 == N) {
      l2 = 0;
      m2 = k2c;
      if (++pr < nplanes) l1 = plane_l1(P0 + pr);
    } else {
      m2 = m2 == 0 ? N - 1 : m2 - 1;
    }
    if (++iw == nfull) iw = 0;
  }
  if (!aborted && __syncthreads_or(to)) aborted = true;
  if (aborted) {
    if (tid == 0) {
      atomicExch(&g_calq32_status, 1);
      // drain: wait for the last copy issued into every stage and plane
      // buffer, so none lands after the block exits.  Fill k of a stage
      // completes phase k of its full barrier, and a stage is refilled only
      // after its previous fill landed, so only the last fill can be pending.
      if (TMA) {
        for (int sx = 0; sx < NST; ++sx) {
          bool t2 = false;
          if (fills[sx] > 0)
            mbar_wait(&full[sx], (uint32_t)((fills[sx] - 1) & 1), t2, DRAIN_LIMIT_NS);
        }
        // plane x went to buffer (NPL == 2 ? x & 1 : 0); the last one issued into
        // each buffer is the only phase that can still be pending there
        for (int px = planes - NPL; px < planes; ++px) {
          if (px < 0) continue;
          const int b = (NPL == 2) ? (px & 1) : 0;
          const int use = (NPL == 2) ? (px >> 1) : px;
          bool t2 = false;
          mbar_wait(&pbar[b], (uint32_t)(use & 1), t2, DRAIN_LIMIT_NS);
        }
      }
    }
    __syncthreads();
    return false;
  }
#pragma unroll
  for (int c = 0; c < SC; ++c) {
    const int s = PAIR ? s0 + 2 * w + c : s0 + w + c * WS;
    if (!k_ok) break;
    if (s >= S) continue;
    const long long o = (long long)k1 * N * N + (long long)k2 * N;
#pragma unroll
    for (int a = 0; a < A; ++a) {
      const int k3 = k3_0 + a;
      if (k3 < N) {
        // (hi, lo) of this output: packed (re, im) at [a][c], or for PAIR
        // lane c of the packed real [a][0] and imaginary [a][1] sums
        u64 hv[SC], lv[SC];
#pragma unroll
        for (int j = 0; j < SC; ++j) {
          if (PAIR || j == c) {
            if (HLS) {
              hv[j] = hl[(size_t)(2 * (a * SC + j)) * blockDim.x + tid];
              lv[j] = hl[(size_t)(2 * (a * SC + j) + 1) * blockDim.x + tid];
            } else {
              hv[j] = hi[HLS ? 0 : a][j];
              lv[j] = lo[HLS ? 0 : a][j];
            }
          }
        }
        float2 h, l;
        if (PAIR) {
          const float2 hr = upk(hv[0]), hm = upk(hv[1]), lr = upk(lv[0]), lm = upk(lv[1]);
          h = c == 0 ? make_float2(hr.x, hm.x) : make_float2(hr.y, hm.y);
          l = c == 0 ? make_float2(lr.x, lm.x) : make_float2(lr.y, lm.y);
        } else {
          h = upk(hv[c]);
          l = upk(lv[c]);
        }
        if (C == 1)
          Q[(long long)s * NQ + o + k3] = make_float2(h.x + l.x, h.y + l.y);
        else
          partial[((long long)chunk * S + s) * NQ + o + k3] = make_float4(h.x, h.y, l.x, l.y);
      }
    }
  }
  return true;
}

// One table per launch: grid (solve groups x chunks, N, k2 tiles).
template <bool TMA, int MAXT, bool HLS, int WS, int A, int MINB, bool PAIR>
__global__ void __launch_bounds__(MAXT, MINB)
    calq32_kernel(int N, int S, int K2T, int NST, int NPL, int C, int GB,
                  const float *__restrict__ B32, const float2 *__restrict__ fin,
                  float2 *__restrict__ Q, float4 *__restrict__ partial, int tmap,
                  unsigned long long wait_ns, const __grid_constant__ CUtensorMap tmB,
                  const __grid_constant__ CUtensorMap tmF) {
  const long long lin =
      blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
  calq32_cta<TMA, MAXT, HLS, WS, A, MINB, PAIR>(N, S, K2T, NST, NPL, C, GB, B32, fin, Q, partial,
                                               tmap, wait_ns, &tmB, &tmF, gridDim.x, gridDim.y,
                                               gridDim.z, lin, (int)blockDim.x);
}

// Several tables in one persistent launch (uneven N, each table shared by its
// solves): a descriptor per table, indexed by work item.  Table t owns the
// items [begin, begin + U GY GZ) of one queue, each the work of one CTA of
// that table's own launch (same tile shape, same item order, so the same
// bits).  A grid of resident CTAs pulls items from the queue in order until it
// is empty; the block is the largest of the tables' (a smaller table leaves its
// extra threads idle).
struct C32Table {
  CUtensorMap tmB, tmF;  // 64-byte aligned
  const float *B32;
  const float2 *fin;
  float2 *Q;
  long long begin;
  float4 *partial;  // C > 1: chunk partial sums
  int N, S, K2T, NST, NPL, GB, U, GY, GZ, tmap, threads, C;
};
constexpr int C32_MULTI_MAX = 16;
struct C32Multi {
  C32Table t[C32_MULTI_MAX];
  int ntab;
  long long total;         // work items (CTAs of the tables' own launches)
  unsigned long long *queue;  // next item, zero at launch; null: item b + k gridDim.x
};

template <bool TMA, int MAXT, bool HLS, int WS, int A, int MINB, bool PAIR>
__global__ void __launch_bounds__(MAXT, MINB)
    calq32_multi_kernel(const __grid_constant__ C32Multi mt, unsigned long long wait_ns) {
  extern __shared__ __align__(128) unsigned char smem[];
  // the item number lives in the unused tail of the 128-byte barrier header
  // (barriers and fill counts take 96 bytes)
  long long *next = reinterpret_cast<long long *>(smem + 120);
  for (long long k = 0;; ++k) {
    // from the queue, in order, so the items in flight stay together (their
    // table slices and f-hat blocks are shared through L2) and CTAs that
    // finish short items early take the next ones; without a queue,
    // round-robin
    if (threadIdx.x == 0)
      *next = mt.queue ? (long long)atomicAdd(mt.queue, 1ull)
                       : (long long)blockIdx.x + k * (long long)gridDim.x;
    __syncthreads();
    const long long item = *next;
    if (item >= mt.total) break;
    int t = 0;
    while (t + 1 < mt.ntab && item >= mt.t[t + 1].begin) ++t;
    const C32Table &d = mt.t[t];
    const bool ok = calq32_cta<TMA, MAXT, HLS, WS, A, MINB, PAIR>(
        d.N, d.S, d.K2T, d.NST, d.NPL, d.C, d.GB, d.B32, d.fin, d.Q, d.partial, d.tmap, wait_ns,
        &d.tmB, &d.tmF, d.U, d.GY, d.GZ, item - d.begin, d.threads);
    if (!ok) break;  // uniform: the CTA drained its copies and set the status word
    // every thread is done with the item; the barriers (at the start of shared
    // memory) are invalidated before the next item initialises them again
    __syncthreads();
    if (threadIdx.x == 0) {
      uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
      for (int i = 0; i < 2 * MAX_ST + 2; ++i)
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(s_addr(bars + i)) : "memory");
    }
    __syncthreads();
  }
}

// Chunk reduction: Q = sum over chunks (in order) of hi + lo, in FP64.
__global__ void calq32_reduce_kernel(long long n, int C, const float4 *__restrict__ partial,
                                     float2 *__restrict__ Q) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double re = 0.0, im = 0.0;
    for (int c = 0; c < C; ++c) {
      const float4 v = partial[(long long)c * n + i];
      re += (double)v.x + (double)v.z;
      im += (double)v.y + (double)v.w;
    }
    Q[i] = make_float2((float)re, (float)im);
  }
}

// Variants the autotuner chooses from (solve lanes WS, k3 outputs per
// thread A, CTA-size bound, where the compensated sums live, CTAs per SM the
// register budget must allow):
//   0: WS 8, A 8, <= 256 threads, registers (<= 255 registers)
//   1: WS 8, A 8, <= 384 threads, shared memory (<= 168 registers)
//   2: WS 2, A 8, <= 256 threads, registers        (4-solve groups)
//   3: WS 8, A 4, <= 256 threads, registers, 2 CTAs per SM (<= 128 registers)
//   4: WS 8, A 4, <= 384 threads, registers (<= 168 registers)
//   5-9: 0-4 on the solve-pair layout (same bits, fewer operand moves and
//        shared-memory loads; needs a pair-layout copy of the input)
struct C32Variant {
  int ws, a, maxt;
  bool hls;
  int minb;
  bool pair;
};
constexpr C32Variant kC32Variants[] = {
    {8, 8, 256, false, 1, false}, {8, 8, 384, true, 1, false}, {2, 8, 256, false, 1, false},
    {8, 4, 256, false, 2, false}, {8, 4, 384, false, 1, false}, {8, 8, 256, false, 1, true},
    {8, 8, 384, true, 1, true},   {2, 8, 256, false, 1, true},  {8, 4, 256, false, 2, true},
    {8, 4, 384, false, 1, true}};
int calq32_variants() { return (int)(sizeof(kC32Variants) / sizeof(kC32Variants[0])); }
int calq32_group(int variant) { return SC * kC32Variants[variant].ws; }
bool calq32_pair(int variant) { return kC32Variants[variant].pair; }
size_t calq32_pair_bytes(int N, int S) { return (size_t)((S + 1) / 2) * N * N * N * sizeof(float4); }

// Tensor maps of one launch (tmap = 0: bulk copies, the maps are unused).
struct C32Maps {
  int tmap = 0;
  CUtensorMap B, F;
};

// cuTensorMapEncodeTiled from the driver (through the runtime's entry-point
// query, so the library links no driver stub).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
  static const EncodeTiledFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}
// FP32 tiled map, no swizzle, out-of-bounds elements read as zero.
static bool encode_map(CUtensorMap *m, int rank, const void *base, const cuuint64_t *dim,
                       const cuuint64_t *stride, const cuuint32_t *box) {
  const EncodeTiledFn fn = encode_tiled();
  if (!fn) return false;
  const cuuint32_t es[5] = {1, 1, 1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, (cuuint32_t)rank, const_cast<void *>(base), dim,
            stride, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <bool TMA, int MAXT, bool HLS, int WS, int A, int MINB, bool PAIR>
static edb_status launch_c32(dim3 grid, int threads, size_t smem, int N, int S, int K2T, int NST,
                             int NPL, int C, int GB, const float *B32, const float2 *fin,
                             float2 *Q, float4 *partial, const C32Maps &maps, cudaStream_t st) {
  // once per instantiation (thread-safe static initialisation: the serving
  // loop's thread and a caller's thread may launch concurrently)
  static const cudaError_t configured =
      cudaFuncSetAttribute(calq32_kernel<TMA, MAXT, HLS, WS, A, MINB, PAIR>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  if (configured != cudaSuccess) return cuda_fail(configured, "cudaFuncSetAttribute(calq32)");
  calq32_kernel<TMA, MAXT, HLS, WS, A, MINB, PAIR>
      <<<grid, threads, smem, st>>>(N, S, K2T, NST, NPL, C, GB, B32, fin, Q, partial, maps.tmap,
                                    wait_limit_ns(), maps.B, maps.F);
  EDB_LAUNCHED();
  return EDB_OK;
}

template <bool TMA>
static edb_status launch_c32_variant(int v, dim3 grid, int threads, size_t smem, int N, int S,
                                     int K2T, int NST, int NPL, int C, int GB, const float *B32,
                                     const float2 *fin, float2 *Q, float4 *partial,
                                     const C32Maps &maps, cudaStream_t st) {
#define EDB_C32(MAXT, HLS, WS, A, MINB, PAIR)                                                   \
  return launch_c32<TMA, MAXT, HLS, WS, A, MINB, PAIR>(grid, threads, smem, N, S, K2T, NST,    \
                                                       NPL, C, GB, B32, fin, Q, partial, maps, \
                                                       st)
  switch (v) {
    case 1: EDB_C32(384, true, 8, 8, 1, false);
    case 2: EDB_C32(256, false, 2, 8, 1, false);
    case 3: EDB_C32(256, false, 8, 4, 2, false);
    case 4: EDB_C32(384, false, 8, 4, 1, false);
    case 5: EDB_C32(256, false, 8, 8, 1, true);
    case 6: EDB_C32(384, true, 8, 8, 1, true);
    case 7: EDB_C32(256, false, 2, 8, 1, true);
    case 8: EDB_C32(256, false, 8, 4, 2, true);
    case 9: EDB_C32(384, false, 8, 4, 1, true);
    default: EDB_C32(256, false, 8, 8, 1, false);
  }
#undef EDB_C32
}

// Tile shape, staging path, tensor maps and pipeline depth of one table's
// launch (the same for a single-table and a grouped launch).  src: the input
// the f_l lines and planes are staged from (the solve-pair copy for PAIR).
struct C32Setup {
  int K2T, tiles, threads, NST, NPL, GB;
  bool tma;
  C32Maps maps;
  size_t bytes;
};

static edb_status c32_setup(int N, int S, const C32Variant &vr, int C, const float *d_B32,
                            const float2 *src, int block_threads, C32Setup *o) {
  const int maxt = vr.maxt, WS = vr.ws, A = vr.a;
  const int SG = SC * WS;
  const int R = (N + A - 1) / A;
  int K2T = maxt / (R * WS);
  if (K2T > N) K2T = N;
  if (K2T < 1) return fail(EDB_EINVAL, "calq32: N too large for the thread tile");
  const int tiles = (N + K2T - 1) / K2T;
  K2T = (N + tiles - 1) / tiles;
  o->K2T = K2T;
  o->tiles = tiles;
  o->threads = K2T * R * WS;
  const int bt = block_threads > 0 ? block_threads : o->threads;
  const int hlt = vr.hls ? bt : 0;
  // TMA bulk copies need 16-byte aligned sources: N % 4 == 0 makes every
  // row/line/plane offset a multiple of 16 bytes; the base pointers are checked
  const int units = vr.pair ? WS : SG, el = vr.pair ? 2 : 1;
  o->tma = (N % 4) == 0 && N >= A && ((uintptr_t)d_B32 % 16) == 0 && ((uintptr_t)src % 16) == 0;
  // line staging by two tensor copies when the f_l box fits (<= 256 floats a
  // row), else by one bulk copy per B row and f_l line
  o->maps = C32Maps{};
  if (o->tma && 2 * c32_geom(N, A, K2T, 1, 1, 0, units, el, true).FLS <= 256 && N <= 256) {
    const int FLS = c32_geom(N, A, K2T, 1, 1, 0, units, el, true).FLS;
    const long long NQ = (long long)N * N * N;
    // pair table [k1][visited line][l3][k2][k3]: dims k3, k2, l3, visited line, k1
    const long long VL = (long long)c32_maxlist(N) * N;
    const cuuint64_t bdim[5] = {(cuuint64_t)N, (cuuint64_t)N, (cuuint64_t)N, (cuuint64_t)VL,
                                (cuuint64_t)N};
    const cuuint64_t bstr[4] = {(cuuint64_t)N * 4, (cuuint64_t)N * N * 4, (cuuint64_t)NQ * 4,
                                (cuuint64_t)(VL * NQ * 4)};
    const cuuint32_t bbox[5] = {(cuuint32_t)N, (cuuint32_t)K2T, (cuuint32_t)N, 1, 1};
    const long long nunits = vr.pair ? (S + 1) / 2 : S;
    const cuuint64_t fdim[3] = {(cuuint64_t)N * 2 * el, (cuuint64_t)N * N, (cuuint64_t)nunits};
    const cuuint64_t fstr[2] = {(cuuint64_t)N * 8 * el, (cuuint64_t)NQ * 8 * el};
    const cuuint32_t fbox[3] = {(cuuint32_t)(2 * FLS), 1, (cuuint32_t)units};
    if (encode_map(&o->maps.B, 5, d_B32, bdim, bstr, bbox) &&
        encode_map(&o->maps.F, 3, src, fdim, fstr, fbox))
      o->maps.tmap = 1;
  }
  // deepest pipeline that fits: two planes with >= 3 stages if possible,
  // else one plane with up to MAX_ST stages (the plain path uses 1 + 1)
  const size_t cap = vr.minb == 2 ? 113 * 1024 : 227 * 1024;
  int NST = 1, NPL = 1;
  if (o->tma) {
    NST = 0;
    for (int ns = MAX_ST; ns >= 3 && !NST; --ns)
      if (c32_geom(N, A, K2T, ns, 2, hlt, units, el, o->maps.tmap).bytes <= cap) {
        NST = ns;
        NPL = 2;
      }
    for (int ns = MAX_ST; ns >= 2 && !NST; --ns)
      if (c32_geom(N, A, K2T, ns, 1, hlt, units, el, o->maps.tmap).bytes <= cap) {
        NST = ns;
        NPL = 1;
      }
    if (!NST) return fail(EDB_EINVAL, "calq32: this variant does not fit in shared memory");
  }
  const C32Geom g = c32_geom(N, A, K2T, NST, NPL, hlt, units, el, o->maps.tmap);
  if (g.bytes > cap) return fail(EDB_EINVAL, "calq32: this variant does not fit in shared memory");
  o->NST = NST;
  o->NPL = NPL;
  o->bytes = g.bytes;
  // solve-group block of the CTA order: about 32 MB of f-hat kept in L2
  const unsigned U = (unsigned)(((S + SG - 1) / SG) * C);
  const long long group_bytes = (long long)SG * N * N * N * (long long)sizeof(float2);
  int GB = (int)std::max<long long>(1, (32LL << 20) / group_bytes) * C;
  if (GB > (int)U) GB = (int)U;
  o->GB = GB;
  return EDB_OK;
}

edb_status launch_calq32_batch(int N, int S, const float *d_B32, const float2 *d_fin, float2 *d_Q,
                               cudaStream_t st, int variant, int C, float4 *d_partial,
                               float4 *d_pairs, int persist) {
  if (variant < 0 || variant >= calq32_variants()) variant = 0;
  if (C < 1 || C > N) return fail(EDB_EINVAL, "calq32: chunk count must be in [1, N]");
  if (C > 1 && !d_partial) return fail(EDB_EINVAL, "calq32: chunks need a partial-sum buffer");
  const C32Variant &vr = kC32Variants[variant];
  if (vr.pair && !d_pairs) return fail(EDB_EINVAL, "calq32: pair variants need a pair buffer");
  const int SG = SC * vr.ws;
  const float2 *src = vr.pair ? reinterpret_cast<const float2 *>(d_pairs) : d_fin;
  C32Setup su;
  EDB_TRY(c32_setup(N, S, vr, C, d_B32, src, 0, &su));
  if (!vr.pair && su.tma && su.maps.tmap && (persist > 0 || (persist < 0 && C == 1))) {
    // one persistent grid of resident CTAs pulls the launch's CTA work items
    // from a queue, in the launch's order (same CTA work, so the same bits;
    // 4096 x N = 24: 84.9 -> 83.0 ms).  Taken round-robin instead, the items
    // in flight drift apart (their costs differ by k1) and the table is read
    // from HBM twice as often (14.3 against 7.5 GB per launch).
    C32MultiIn one{N, S, d_B32, d_fin, d_Q};
    one.C = C;
    one.partial = d_partial;
    EDB_TRY(launch_calq32_multi(1, &one, variant, st, persist < 0));
    if (C == 1) return EDB_OK;
    const long long n = (long long)S * N * N * N;
    const long long blocks = std::min<long long>((n + 255) / 256, 16LL * device_sm_count());
    calq32_reduce_kernel<<<(unsigned)blocks, 256, 0, st>>>(n, C, d_partial, d_Q);
    EDB_LAUNCHED();
    return EDB_OK;
  }
  dim3 grid((unsigned)(((S + SG - 1) / SG) * C), (unsigned)N, (unsigned)su.tiles);
  if (vr.pair) {
    const long long n = (long long)((S + 1) / 2) * N * N * N;
    const long long blocks = std::min<long long>((n + 255) / 256, 16LL * device_sm_count());
    c32_pairs_kernel<<<(unsigned)blocks, 256, 0, st>>>(S, (long long)N * N * N, d_fin, d_pairs);
    EDB_LAUNCHED();
  }
  edb_status rc =
      su.tma ? launch_c32_variant<true>(variant, grid, su.threads, su.bytes, N, S, su.K2T, su.NST,
                                        su.NPL, C, su.GB, d_B32, src, d_Q, d_partial, su.maps, st)
             : launch_c32_variant<false>(variant, grid, su.threads, su.bytes, N, S, su.K2T,
                                         su.NST, su.NPL, C, su.GB, d_B32, src, d_Q, d_partial,
                                         su.maps, st);
  if (rc != EDB_OK || C == 1) return rc;
  const long long n = (long long)S * N * N * N;
  const long long blocks = std::min<long long>((n + 255) / 256, 16LL * device_sm_count());
  calq32_reduce_kernel<<<(unsigned)blocks, 256, 0, st>>>(n, C, d_partial, d_Q);
  EDB_LAUNCHED();
  return EDB_OK;
}

template <int V>
static edb_status launch_c32_multi_v(const C32Multi &mt, int block, size_t smem,
                                     cudaStream_t st) {
  constexpr C32Variant vr = kC32Variants[V];
  auto kern = calq32_multi_kernel<true, vr.maxt, vr.hls, vr.ws, vr.a, vr.minb, false>;
  static const cudaError_t configured = cudaFuncSetAttribute(
      kern, cudaFuncAttributeMaxDynamicSharedMemorySize, vr.minb == 2 ? 113 * 1024 : 227 * 1024);
  if (configured != cudaSuccess) return cuda_fail(configured, "cudaFuncSetAttribute(calq32 multi)");
  // persistent grid: the CTAs that fit on the device at once, at most one per
  // item (the occupancy is cached per device and shape, so a launch recorded
  // into a graph after a first direct launch makes no query)
  static std::mutex mu;
  static std::map<long long, int> occ_cache;
  int dev = 0;
  EDB_CUDA(cudaGetDevice(&dev));
  const long long key = ((long long)dev << 40) | ((long long)block << 24) | (long long)smem;
  int occ = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = occ_cache.find(key);
    if (it != occ_cache.end()) {
      occ = it->second;
    } else {
      EDB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, block, smem));
      occ_cache[key] = occ;
    }
  }
  if (occ < 1) return fail(EDB_EINVAL, "calq32 multi: the block does not fit on an SM");
  const long long blocks = std::min<long long>(mt.total, (long long)occ * device_sm_count());
  kern<<<(unsigned)blocks, block, smem, st>>>(mt, wait_limit_ns());
  EDB_LAUNCHED();
  return EDB_OK;
}

// Grouped launch: one plain-layout variant (0-4) for every table, tensor-copy
// staging required; tables ordered by descending N (their CTAs are the
// longest) in one work queue, each table's CTAs in its own launch's order,
// served by a persistent grid.
edb_status launch_calq32_multi(int ntab, const C32MultiIn *in, int variant, cudaStream_t st,
                               bool queue) {
  if (ntab < 1 || ntab > C32_MULTI_MAX)
    return fail(EDB_EINVAL, "calq32 multi: 1 to 16 tables per launch");
  if (variant < 0 || variant >= calq32_variants() || kC32Variants[variant].pair)
    return fail(EDB_EINVAL, "calq32 multi: a plain-layout variant (0-4)");
  const C32Variant &vr = kC32Variants[variant];
  const int SG = SC * vr.ws;
  std::vector<int> order(ntab);
  for (int i = 0; i < ntab; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return in[a].N > in[b].N; });
  // the block is the largest table's; every table's shared memory and
  // pipeline depth is chosen for that block
  int block = 0;
  for (int i = 0; i < ntab; ++i) {
    if (in[i].S < 1 || !in[i].B32 || !in[i].fin || !in[i].Q)
      return fail(EDB_EINVAL, "calq32 multi: bad table entry");
    C32Setup su;
    if (in[i].C < 1 || in[i].C > in[i].N || (in[i].C > 1 && !in[i].partial))
      return fail(EDB_EINVAL, "calq32 multi: bad chunk count");
    EDB_TRY(c32_setup(in[i].N, in[i].S, vr, in[i].C, in[i].B32, in[i].fin, 0, &su));
    block = std::max(block, su.threads);
  }
  C32Multi mt;
  memset(&mt, 0, sizeof(mt));
  mt.ntab = ntab;
  long long begin = 0;
  size_t smem = 0;
  for (int j = 0; j < ntab; ++j) {
    const C32MultiIn &e = in[order[j]];
    C32Setup su;
    EDB_TRY(c32_setup(e.N, e.S, vr, e.C, e.B32, e.fin, block, &su));
    if (!su.tma || !su.maps.tmap)
      return fail(EDB_EINVAL, "calq32 multi: every table needs the tensor-copy path (N % 4 == 0)");
    C32Table &d = mt.t[j];
    d.tmB = su.maps.B;
    d.tmF = su.maps.F;
    d.B32 = e.B32;
    d.fin = e.fin;
    d.Q = e.Q;
    d.begin = begin;
    d.N = e.N;
    d.S = e.S;
    d.K2T = su.K2T;
    d.NST = su.NST;
    d.NPL = su.NPL;
    d.GB = su.GB;
    d.U = (e.S + SG - 1) / SG * e.C;
    d.C = e.C;
    d.partial = e.partial;
    d.GY = e.N;
    d.GZ = su.tiles;
    d.tmap = 1;
    d.threads = su.threads;
    begin += (long long)d.U * d.GY * d.GZ;
    smem = std::max(smem, su.bytes);
  }
  mt.total = begin;
  // the work queue's counter, stream-ordered: allocated, zeroed, used, freed
  mt.queue = nullptr;
  if (queue) {
    EDB_CUDA(
        cudaMallocAsync(reinterpret_cast<void **>(&mt.queue), sizeof(unsigned long long), st));
    EDB_CUDA(cudaMemsetAsync(mt.queue, 0, sizeof(unsigned long long), st));
  }
  edb_status rc;
  switch (variant) {
    case 0: rc = launch_c32_multi_v<0>(mt, block, smem, st); break;
    case 1: rc = launch_c32_multi_v<1>(mt, block, smem, st); break;
    case 2: rc = launch_c32_multi_v<2>(mt, block, smem, st); break;
    case 3: rc = launch_c32_multi_v<3>(mt, block, smem, st); break;
    default: rc = launch_c32_multi_v<4>(mt, block, smem, st); break;
  }
  const cudaError_t fe = queue ? cudaFreeAsync(mt.queue, st) : cudaSuccess;
  if (rc != EDB_OK) return rc;
  if (fe != cudaSuccess) return cuda_fail(fe, "cudaFreeAsync(calq32 multi queue)");
  return EDB_OK;
}

edb_status read_calq32_status(int *status, bool clear) {
  int v = 0;
  EDB_CUDA(cudaMemcpyFromSymbol(&v, g_calq32_status, sizeof(int)));
  if (clear && v) {
    int z = 0;
    EDB_CUDA(cudaMemcpyToSymbol(g_calq32_status, &z, sizeof(int)));
  }
  *status = v;
  return EDB_OK;
}

}  // namespace edb
