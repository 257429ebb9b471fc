// FP64-accurate collision sum on the FP32 pipe (the drop-in path's fast
// kernel).
//
// GB300 runs native FP64 FMA at about 1.5 instructions per clock per SM, so
// the reference's six FP64 operations per term (QCalculator.h:247) would keep
// the B stream near a tenth of HBM bandwidth.  This kernel keeps FP64 accuracy
// with double-float arithmetic (every value as an unevaluated sum hi + lo of
// two floats, about 48 significant bits) built from error-free
// transformations: the product of two floats is split exactly as
// p + e with e = fma(a, b, -p) (FMA two-product), and sums are carried exactly
// by Knuth's two-sum.  Low-order cross terms (hi * lo) are added in plain
// FP32; their rounding is 2^-24 of a quantity already 2^-24 smaller.
//
// Data: B2 is the kernel table pre-split into (hi, lo) float pairs (8 bytes
// per term, the same stream as FP64), in the flat layout the FP64 kernel
// reads (row lflat, column kflat, row stride KC = P^3).  fdf is f-hat split
// into {re_hi, im_hi, re_lo, im_lo}.
//
// Per term, with u = b f_m (complex times real) and Q = sum f_l u:
//   u   = -nu_h + uc          nu_h = -(b_h f_m,h)  [mul],  uc = exact error +
//                             b_h f_m,l + b_l f_m,h        [3 fma]
//   accA += f_l.x u,  accB += f_l.y u   (each: two-product of the hi parts,
//                             two cross terms, two-sum into (hi, lo): 12 ops)
// with every operation a packed f32x2 instruction over (re, im) lanes; at the
// end Q = (A.re - B.im, A.im + B.re), combined in FP64.
//
// Pairs: with the aliased index shifts (ALIASED mode, or odd N) B2 is the
// split symmetric pair table (b2_pair_split_kernel) and each output plane
// visits only the l1 planes with l1 <= (k1 - l1) mod N, about half the B
// stream; otherwise every l-line is visited with B split as it is.  When N is
// a multiple of 4 the pair table is read by calq64p_kernel instead (the same
// sum with neighbouring outputs in the packed lanes; see there).
//
// Tiling: CTA = (output plane j1, a tile of j2, all j3) x (a chunk of its
// l-lines (i1, i2)).  Thread = (j2, run of 4 consecutive j3).  For each i1 the f-hat
// m1-plane (m1 = j1 - i1 + sM mod N) is staged in shared memory; along i3 the
// needed f_m slide down by one (a ring of 4).  The number of line chunks comes
// from a model of the schedule on the measured resident CTA slots (see
// c64x_plan_compute).  Each CTA writes
// FP64 partial sums per chunk; calq64_reduce_kernel adds the chunks in order.
//
// B stream: when every warp's row segment is a contiguous, 16-byte aligned run
// (P % 4 == 0 and whole j2 tiles), each warp streams its own 1 KB segment of
// the next D rows into a private shared-memory ring with 1-D TMA bulk copies
// (lane 0 issues; one mbarrier per slot; waits bounded by %globaltimer, a
// timeout sets the device status word).  Otherwise threads load their 32
// bytes per row with __ldg, one row ahead.
#include <algorithm>
#include <functional>
#include <map>
#include <mutex>
#include <queue>
#include <vector>

#include "edb_df.cuh"
#include "edb_internal.cuh"

namespace edb {

namespace {
using namespace df;
constexpr int RUN = 4;  // outputs per thread along j3

constexpr int DEPTH = 8;  // B rows in flight per warp
// Limit of the drain after a wait ran out: lane 0 then waits this long at
// most for each copy its warp issued, so none lands after the block exits.
constexpr unsigned long long DRAIN_LIMIT_NS = 1000000000ull;

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
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(s_addr(dst)),
      "l"(src), "r"(bytes), "r"(s_addr(bar))
      : "memory");
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
// runs out at once, without polling); a thread that timed out does not wait
// again.
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

// mbar_wait for a nonzero limit
__device__ __forceinline__ void mbar_wait_nz(uint64_t *bar, uint32_t parity, bool &to,
                                             unsigned long long limit_ns) {
  if (to || mbar_try_wait(bar, parity)) return;
  const unsigned long long t0 = gtimer_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (gtimer_ns() - t0 >= limit_ns) {
      to = true;
      return;
    }
  }
}

__device__ int g_calq64x_status;  // nonzero: a bounded wait ran out
}  // namespace

// Splits f-hat into {re_hi, im_hi, re_lo, im_lo}.
__global__ void fdf_split_kernel(long long n, const double2 *__restrict__ f, float4 *__restrict__ out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 v = f[i];
  const float rh = (float)v.x, ih = (float)v.y;
  const float rl = (float)(v.x - (double)rh), il = (float)(v.y - (double)ih);
  out[i] = make_float4(rh, ih, rl, il);
}

// The output-pair kernel's input: the split of f-hat rotated along the last
// axis by shift (see calq64p_kernel), and one zero float4 of padding.
__global__ void fdr_split_kernel(int N, int shift, const double2 *__restrict__ f,
                                 float4 *__restrict__ out) {
  const long long NQ = (long long)N * N * N;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > NQ) return;
  if (i == NQ) {
    out[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  const long long row = i / N;
  int c = (int)(i - row * N) + shift;
  if (c >= N) c -= N;
  const double2 v = f[row * N + c];
  const float rh = (float)v.x, ih = (float)v.y;
  out[i] = make_float4(rh, ih, (float)(v.x - (double)rh), (float)(v.y - (double)ih));
}

__global__ void b2_split_kernel(long long n, const double *__restrict__ B, float2 *__restrict__ B2) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = B[i];
  const float h = (float)v;
  B2[i] = make_float2(h, (float)(v - (double)h));
}

// The paired table of the double-float kernel (ALIASED, P = N): entry
// [l][k] (centred) is B[l][k] + B[m][k], m the partner row with
// m_d = (k_d - l_d + n) mod N, summed in FP64 and then split, or B[l][k]
// alone when l and m share the first index (both terms lie on one visited
// plane).  The terms l and m of a Q-hat sum carry the same product f_l f_m.
__global__ void b2_pair_split_kernel(int N, const double *__restrict__ B, float2 *__restrict__ B2) {
  const long long NQ = (long long)N * N * N;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NQ * NQ) return;
  const long long l = i / NQ, k = i - l * NQ;
  const int n = (N - 1) / 2;
  const int l1 = (int)(l / (N * N)), l2 = (int)((l / N) % N), l3 = (int)(l % N);
  const int k1 = (int)(k / (N * N)), k2 = (int)((k / N) % N), k3 = (int)(k % N);
  const int m1 = (k1 - l1 + n + N) % N, m2 = (k2 - l2 + n + N) % N, m3 = (k3 - l3 + n + N) % N;
  double v = B[i];
  if (m1 != l1) v += B[(((long long)m1 * N + m2) * N + m3) * NQ + k];
  const float h = (float)v;
  const float lo = (float)(v - (double)h);
  if (N % RUN == 0) {
    // output-pair layout (calq64p_kernel): each aligned group G of four
    // entries as the halves {h0, h1, l0, l1}, {h2, h3, l2, l3}, in swapped
    // order when bit 2 of G is set (the reader's 128-bit loads then spread
    // over all bank groups)
    float *o = reinterpret_cast<float *>(B2);
    const long long half = ((i >> 1) & 1) ^ ((i >> 4) & 1);
    const long long hp = 2 * (i & ~3ll) + half * 4 + (i & 1);
    o[hp] = h;
    o[hp + 2] = lo;
  } else {
    B2[i] = make_float2(h, lo);
  }
}

// TMA: per-warp bulk-copy ring for B (requires contiguous, aligned warp
// segments; see the launcher).  Otherwise __ldg one row ahead.
// MAXT, MINB: CTA size bound and minimum resident CTAs per SM the register
// allocation must allow (see kC64xShapes).  The kernel is bound by the latency
// of its dependent double-float chains, so resident warps matter: chosen per
// table by timing every shape (edb_qcalc_genB runs the comparison once).
template <bool TMA, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB)
    calq64x_kernel(QParams p, int J2T, int LC, int paired, const float2 *__restrict__ B2,
                   const float4 *__restrict__ fdf, double2 *__restrict__ partial,
                   unsigned long long wait_ns) {
  extern __shared__ __align__(128) unsigned char smem64[];
  const int N = p.N, P = p.P;
  const int R4 = (P + RUN - 1) / RUN;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
  const int wthreads = min(32, (int)blockDim.x - warp * 32);  // threads in this warp
  const unsigned wmask = wthreads == 32 ? 0xffffffffu : ((1u << wthreads) - 1u);
  const long long NN = (long long)N * N;
  // shared memory: [nwarps][DEPTH] mbarriers, B rings [nwarps][DEPTH][32 threads x 4 pairs],
  // then the f-hat plane [N][N]
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem64);
  float2 *rings = reinterpret_cast<float2 *>(smem64 + 16 * ((nwarps * DEPTH * 8 + 15) / 16));
  float4 *plane = reinterpret_cast<float4 *>(rings + (TMA ? (size_t)nwarps * DEPTH * 32 * RUN : 0));
  uint64_t *mybar = bars + warp * DEPTH;
  float2 *myring = rings + (size_t)warp * DEPTH * 32 * RUN;

  const int r = tid % R4;
  const int j2l = tid / R4;
  const int j1 = blockIdx.x;
  const int j2 = blockIdx.y * J2T + j2l;
  const bool ok = (j2l < J2T) && (j2 < P);
  const int j2c = ok ? j2 : 0;
  const int j3_0 = r * RUN;
  const int chunk = blockIdx.z;
  // l1 planes this output plane visits.  Paired table (ALIASED): the terms l
  // and m = k - l share the product f_l f_m and B2 holds B[l][k] + B[m][k], so
  // only the planes with a1 <= (k1 - a1) mod N are visited (a1, k1 in FFTW
  // order): [0, k1/2] and [k1+1, (k1+N)/2].  Otherwise every i1 in order.
  const int k1f = (j1 - p.n + N) % N;
  const int plo = k1f / 2;
  const int nlist = paired ? plo + 1 + max(0, (k1f + N) / 2 - k1f) : N;
  auto plane_i1 = [&](int pi) {
    if (!paired) return pi;
    const int a = pi <= plo ? pi : k1f + 1 + (pi - plo - 1);
    return (a + p.n) % N;  // a = (i1 - n) mod N
  };
  const int NL = nlist * N;  // l-lines (i1, i2) of those planes
  const int c0 = min(NL, chunk * LC), c1 = min(NL, c0 + LC);
  // B2 row of the chunk's qq-th row (line c0 + qq / N, i3 = qq mod N)
  auto row_of = [&](int qq) -> long long {
    const int t = c0 + qq / N;
    return ((long long)plane_i1(t / N) * N + t % N) * N + qq % N;
  };
  const long long kcol = ((long long)j1 * P + j2c) * P + j3_0;
  // columns past P (ragged last run) read a clamped, in-row column and are
  // masked out of the output
  int colc[RUN];
#pragma unroll
  for (int a = 0; a < RUN; ++a) colc[a] = (j3_0 + a < P) ? a : 0;

  // the warp's B segment: threads [32 warp, 32 warp + wthreads) are consecutive
  // 4-pair runs, contiguous in the row (checked by the launcher)
  const long long wcol = ((long long)j1 * P + (blockIdx.y * J2T + (warp * 32) / R4)) * P +
                         ((warp * 32) % R4) * RUN;
  const uint32_t seg_bytes = (uint32_t)(wthreads * RUN * sizeof(float2));
  const int nrows = (c1 - c0) * N;  // rows this CTA streams
  bool to = false;
  int issued = 0;  // lane 0: rows its warp has issued into the ring
  // refill cursor (lane 0): row q + DEPTH of the chunk as (list plane, i2, i3),
  // advanced by one row per refill so the per-row path has no division
  int rf_pi = 0, rf_i2 = 0, rf_i3 = 0;
  long long rf_base = 0;
  const float2 *rf_src = nullptr;  // source of row q + DEPTH: B2 + (rf_base + rf_i3) KC + wcol
  if (TMA && lane == 0 && DEPTH < nrows) {
    const int t = c0 + DEPTH / N;
    rf_pi = t / N;
    rf_i2 = t % N;
    rf_i3 = DEPTH % N;
    rf_base = ((long long)plane_i1(rf_pi) * N + rf_i2) * N;
    rf_src = B2 + (rf_base + rf_i3) * p.KC + wcol;
  }

  if (TMA) {
    if (lane == 0) {
      for (int d = 0; d < DEPTH; ++d) mbar_init(&mybar[d], 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp(wmask);
    if (lane == 0) {  // prologue: the first DEPTH rows
      for (int q = 0; q < DEPTH && q < nrows; ++q) {
        const long long lflat = row_of(q);
        mbar_expect_tx(&mybar[q], seg_bytes);
        bulk_g2s(myring + (size_t)q * 32 * RUN, B2 + lflat * p.KC + wcol, seg_bytes, &mybar[q]);
        ++issued;
      }
    }
  }

  DF2 accA[RUN], accB[RUN];
#pragma unroll
  for (int a = 0; a < RUN; ++a) {
    accA[a].h = accA[a].l = 0ull;
    accB[a].h = accB[a].l = 0ull;
  }

  const int base3 = (j3_0 + p.sM) % N;  // m3 of output a = 0 at i3 = 0
  const int fi0 = p.sL % N;             // f_l entry at i3 = 0
  int cur_i1 = -1;
  int q = 0;  // row counter within the chunk
  for (int line = c0; line < c1; ++line) {
    // line indices: i1, i2 (centred l); a1, a2 = (i + sL) mod N (f_l, FFTW
    // order); m2 = (j2 - i2 + sM) mod N.  Computed per line: counters kept
    // across the loop cost registers and measured slower here.
    const int i1 = plane_i1(line / N), i2 = line % N;
    const int a1 = (i1 + p.sL) % N, a2 = (i2 + p.sL) % N;
    const int m2 = ((j2c - i2 + p.sM) % N + N) % N;
    if (i1 != cur_i1) {  // stage the m1-plane
      cur_i1 = i1;
      const int m1 = ((j1 - i1 + p.sM) % N + N) % N;
      __syncthreads();
      for (long long e = tid; e < NN; e += blockDim.x) plane[e] = fdf[(long long)m1 * NN + e];
      __syncthreads();
    }
    const float4 *prow = plane + (long long)m2 * N;
    const float4 *flrow = fdf + ((long long)a1 * N + a2) * N;
    const long long lrow0 = ((long long)i1 * N + i2) * N;
    u64 rh[RUN], rl[RUN];  // f_m hi, lo (re, im lanes)
#pragma unroll
    for (int a = 0; a < RUN; ++a) {
      int m3 = base3 + a;
      while (m3 >= N) m3 -= N;
      const float4 v = prow[m3];
      rh[a] = pk(v.x, v.y);
      rl[a] = pk(v.z, v.w);
    }
    const float2 *brow = B2 + lrow0 * p.KC + kcol;
    float2 bcur[RUN], bnext[RUN];
    // running indices along i3: the new ring entry m3 = (j3_0 - i3 + sM) mod N
    // and the f_l entry fi = (i3 + sL) mod N, kept in range by one conditional
    int m3n = base3;  // value at i3 = 0
    int fi = fi0;
    float4 fl_next = __ldg(flrow + fi);
    if (!TMA) {
#pragma unroll
      for (int a = 0; a < RUN; ++a) bcur[a] = __ldg(brow + colc[a]);
    }
    for (int g = 0; g < N; g += RUN) {
#pragma unroll
      for (int t = 0; t < RUN; ++t, ++q) {
        const int i3 = g + t;
        if (i3 >= N) break;
        if (TMA) {
          const int slot = q % DEPTH;
          mbar_wait(&mybar[slot], (uint32_t)((q / DEPTH) & 1), to, wait_ns);
          const float4 *src = reinterpret_cast<const float4 *>(myring + ((size_t)slot * 32 + lane) * RUN);
#pragma unroll
          for (int h = 0; h < RUN / 2; ++h) {
            const float4 v = src[h];
            bcur[2 * h] = make_float2(v.x, v.y);
            bcur[2 * h + 1] = make_float2(v.z, v.w);
          }
          // every lane has read the slot; refill it with row q + DEPTH unless a
          // lane timed out (its copy may still be landing: the warp then
          // issues nothing more, so at most one copy per slot is in flight)
          const bool bad = __any_sync(wmask, to);
          if (lane == 0 && !bad && q + DEPTH < nrows) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_expect_tx(&mybar[slot], seg_bytes);
            bulk_g2s(myring + (size_t)slot * 32 * RUN, rf_src, seg_bytes, &mybar[slot]);
            // the next row is one row of the table further (KC entries) within
            // a line; a new line restarts from its own row block
            if (++rf_i3 == N) {
              rf_i3 = 0;
              if (++rf_i2 == N) {
                rf_i2 = 0;
                ++rf_pi;
              }
              rf_base = ((long long)plane_i1(rf_pi) * N + rf_i2) * N;
              rf_src = B2 + rf_base * p.KC + wcol;
            } else {
              rf_src += p.KC;
            }
            ++issued;
          }
        } else if (i3 + 1 < N) {
          const float2 *bn = brow + (long long)(i3 + 1) * p.KC;
#pragma unroll
          for (int a = 0; a < RUN; ++a) bnext[a] = __ldg(bn + colc[a]);
        }
        if (i3 > 0) {  // new ring value enters at a = 0
          m3n = (m3n == 0) ? N - 1 : m3n - 1;
          const float4 v = prow[m3n];
          const int slot = (RUN - t) % RUN;
          rh[slot] = pk(v.x, v.y);
          rl[slot] = pk(v.z, v.w);
        }
        // broadcast pairs of f_l.re and f_l.im (hi; and negated hi, lo)
        const float4 fl = fl_next;
        fi = (fi + 1 == N) ? 0 : fi + 1;
        fl_next = __ldg(flrow + fi);
        const u64 xr = pk(fl.x, fl.x), nxr = pk(-fl.x, -fl.x), nlr = pk(-fl.z, -fl.z);
        const u64 xi = pk(fl.y, fl.y), nxi = pk(-fl.y, -fl.y), nli = pk(-fl.w, -fl.w);
        u64 nuh[RUN], ucs[RUN];
#pragma unroll
        for (int a = 0; a < RUN; ++a) {
          const int slot = (a - t + RUN) % RUN;
          const float bh = bcur[a].x, bl = bcur[a].y;
          const u64 nbh2 = pk(-bh, -bh), bh2 = pk(bh, bh), bl2 = pk(bl, bl);
          // u = b * f_m:  nu_h = -(b_h f_m,h), uc = exact error + cross terms
          nuh[a] = mul2(nbh2, rh[slot]);
          const u64 ue = fma2(bh2, rh[slot], nuh[a]);
          ucs[a] = fma2(bh2, rl[slot], fma2(bl2, rh[slot], ue));
        }
#pragma unroll
        for (int a = 0; a < RUN; ++a) df_axpy(accA[a], xr, nxr, nlr, nuh[a], ucs[a]);
#pragma unroll
        for (int a = 0; a < RUN; ++a) df_axpy(accB[a], xi, nxi, nli, nuh[a], ucs[a]);
        if (!TMA) {
#pragma unroll
          for (int a = 0; a < RUN; ++a) bcur[a] = bnext[a];
        }
      }
    }
  }
  if (TMA) {
    if (__syncthreads_or(to)) {
      if (lane == 0) {
        atomicExch(&g_calq64x_status, 1);
        // drain: row r went into slot r % DEPTH as its fill r / DEPTH, and a
        // slot is refilled only after its previous copy landed, so only the
        // last row issued into each slot can still be in flight
        for (int sl = 0; sl < DEPTH && sl < issued; ++sl) {
          const int last = sl + ((issued - 1 - sl) / DEPTH) * DEPTH;
          bool t2 = false;
          mbar_wait(&mybar[sl], (uint32_t)((last / DEPTH) & 1), t2, DRAIN_LIMIT_NS);
        }
      }
      __syncwarp(wmask);
      return;
    }
  }
  if (!ok) return;
#pragma unroll
  for (int a = 0; a < RUN; ++a) {
    if (j3_0 + a >= P) continue;
    const float2 Ah = upk(accA[a].h), Al = upk(accA[a].l);
    const float2 Bh = upk(accB[a].h), Bl = upk(accB[a].l);
    const double re = ((double)Ah.x + (double)Al.x) - ((double)Bh.y + (double)Bl.y);
    const double im = ((double)Ah.y + (double)Al.y) + ((double)Bh.x + (double)Bl.x);
    partial[(long long)chunk * p.KC + kcol + a] = make_double2(re, im);
  }
}

// Output-pair form of calq64x_kernel (pair table, N % 4 == 0).  The f32x2
// lanes carry two neighbouring outputs (j3, j3 + 1) instead of the (re, im)
// parts of one, so the table's values enter the packed instructions as they
// are stored: each thread's four entries of a row are laid out as
// {h0, h1, l0, l1, h2, h3, l2, l3} (b2_pair_split_kernel), and no broadcast
// pair of b is formed (the two 16-byte halves of a thread's entries are
// stored swapped for every other run of four threads, and each thread loads
// them in its own order, so eight consecutive lanes cover all bank groups).
// Per term the arithmetic is the same double-float
// sequence: u = b f_m for the real and imaginary parts of f_m, then
//   R += f_l.re u.re + (-f_l.im) u.im,   I += f_l.re u.im + f_l.im u.re
// with four df_axpy per output pair.  f_m comes from a shared-memory copy of
// the m1-plane stored as neighbour pairs, E[x] = {re_h(x), re_h(x+1),
// im_h(x), im_h(x+1)}, {re_l(x), re_l(x+1), im_l(x), im_l(x+1)} (x + 1 mod N):
// at step i3 the pair (0, 1) reads E[x], the pair (2, 3) E[x + 2], x =
// (j3_0 - i3 + sM) mod N, so one new entry per step and a ring of four.  The
// hi and lo halves sit in two planes, each row stored transposed, E[x] at
// (x mod 4) N/4 + x/4: the lanes of a row read x four apart, which then fall
// in distinct 16-byte bank groups (at N = 32 every 128-bit load is
// conflict-free; untransposed, eight lanes shared one group).
// B stream: ROWS table rows per ring slot (one wait, one vote and one
// expect_tx per slot), PDEPTH rows in flight per warp.
constexpr int PDEPTH = 8;
struct __align__(16) P64Cursor {
  const float4 *src;
  int pi, i2, i3;
  int issued;  // slot fills the warp has issued
};

// fdr: f-hat split as for calq64x_kernel and rotated along the last axis by
// the f_l shift, fdr[a1][a2][i] = f[a1][a2][(i + sL) mod N], with one float4 of
// padding after the last row: the f_l of step i3 is entry i3 of its row (the
// read one step ahead touches entry N, the next row's first or the padding).
// An f_m entry x (FFTW order) sits at (x + n) mod N of its row.
// NC > 0: N fixed at compile time (the index arithmetic folds); 0: p.N.
template <bool TMA, int MAXT, int MINB, int ROWS, int NC>
__global__ void __launch_bounds__(MAXT, MINB)
    calq64p_kernel(QParams p, int J2T, int LC, const float4 *__restrict__ B2p,
                   const float4 *__restrict__ fdr, double2 *__restrict__ partial,
                   unsigned long long wait_ns) {
  constexpr int SLOTS = PDEPTH / ROWS;
  static_assert(SLOTS * ROWS == PDEPTH && RUN % ROWS == 0, "ring shape");
  extern __shared__ __align__(128) unsigned char smem64[];
  const int N = NC > 0 ? NC : p.N;  // == P
  const int n = (N - 1) / 2;
  const int R4 = N / RUN;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
  const int wthreads = min(32, (int)blockDim.x - warp * 32);
  const unsigned wmask = wthreads == 32 ? 0xffffffffu : ((1u << wthreads) - 1u);
  const int NN = N * N;
  const long long KC2 = (long long)NN * N / 2;  // float4 per table row
  // shared memory: [nwarps][SLOTS] mbarriers; [nwarps] refill cursors; B rings
  // [nwarps][PDEPTH rows][32 threads][2 float4]; the neighbour-pair planes (hi,
  // then lo) [N][N] float4
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem64);
  P64Cursor *curs =
      reinterpret_cast<P64Cursor *>(smem64 + 16 * ((nwarps * SLOTS * 8 + 15) / 16));
  float4 *rings = reinterpret_cast<float4 *>(reinterpret_cast<unsigned char *>(curs) +
                                             sizeof(P64Cursor) * nwarps);
  float4 *ehi = rings + (TMA ? (size_t)nwarps * PDEPTH * 32 * 2 : 0);
  float4 *elo = ehi + NN;
  uint64_t *mybar = bars + warp * SLOTS;
  float4 *myring = rings + (size_t)warp * PDEPTH * 32 * 2;

  const int r = tid % R4;
  const int j2l = tid / R4;
  const int j1 = blockIdx.x;
  const int j2 = blockIdx.y * J2T + j2l;
  const bool ok = (j2l < J2T) && (j2 < N);
  const int j2c = ok ? j2 : 0;
  const int j3_0 = r * RUN;
  const int chunk = blockIdx.z;
  // l1 planes this output plane visits (the pair table): a1 <= (k1 - a1) mod N
  const int k1f = (j1 - n + N) % N;
  const int plo = k1f / 2;
  const int nlist = plo + 1 + max(0, (k1f + N) / 2 - k1f);
  auto plane_i1 = [&](int pi) {
    const int a = pi <= plo ? pi : k1f + 1 + (pi - plo - 1);
    return (a + n) % N;
  };
  const int NL = nlist * N;
  const int c0 = min(NL, chunk * LC), c1 = min(NL, c0 + LC);
  auto row_of = [&](int qq) -> long long {
    const int t = c0 + qq / N;
    return ((long long)plane_i1(t / N) * N + t % N) * N + qq % N;
  };
  // entry index of the thread's run within a row (a multiple of 4: float4 kcol / 2)
  const long long kcol = ((long long)j1 * N + j2c) * N + j3_0;
  const int hsw = (int)((kcol >> 4) & 1);  // halves stored swapped
  const long long wcol = ((long long)j1 * N + (blockIdx.y * J2T + (warp * 32) / R4)) * N +
                         ((warp * 32) % R4) * RUN;
  const uint32_t seg_bytes = (uint32_t)(wthreads * RUN * sizeof(float2));
  const int nrows = (c1 - c0) * N;  // a multiple of 4
  // a zero limit: every wait has run out at once
  bool to = TMA && wait_ns == 0;
  // lane 0's cursor (kept in shared memory, off the registers of the loop):
  // the next row to issue as (list plane, i2, i3), its source, and the fills
  // issued so far
  if (TMA && lane == 0) {
    P64Cursor c;
    c.issued = 0;
    c.src = nullptr;
    c.pi = c.i2 = c.i3 = 0;
    if (PDEPTH < nrows) {
      const int t = c0 + PDEPTH / N;
      c.pi = t / N;
      c.i2 = t % N;
      c.i3 = PDEPTH % N;
      c.src = B2p + (((long long)plane_i1(c.pi) * N + c.i2) * N + c.i3) * KC2 + wcol / 2;
    }
    curs[warp] = c;
  }

  if (TMA) {
    if (lane == 0) {
      for (int d = 0; d < SLOTS; ++d) mbar_init(&mybar[d], 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp(wmask);
    if (lane == 0) {  // prologue: rows [0, PDEPTH)
      for (int s = 0; s < SLOTS && s * ROWS < nrows; ++s) {
        const int nr = min(ROWS, nrows - s * ROWS);
        mbar_expect_tx(&mybar[s], seg_bytes * nr);
        for (int rr = 0; rr < nr; ++rr) {
          const int qq = s * ROWS + rr;
          bulk_g2s(myring + (size_t)qq * 32 * 2, B2p + row_of(qq) * KC2 + wcol / 2, seg_bytes,
                   &mybar[s]);
        }
        ++curs[warp].issued;
      }
    }
  }

  DF2 accR[2], accI[2];  // lanes (j3_0 + 2h, j3_0 + 2h + 1)
#pragma unroll
  for (int h = 0; h < 2; ++h) accR[h].h = accR[h].l = accI[h].h = accI[h].l = 0ull;
  const u64 MONE = pk(-1.0f, -1.0f);
  const float4 *lring = myring + (size_t)lane * 2 + hsw;  // this lane's first half, ring row 0

  int cur_i1 = -1;
  int q = 0;  // chunk row of the current group's first step (a multiple of 4)
  for (int line = c0; line < c1; ++line) {
    const int i1 = plane_i1(line / N), i2 = line % N;
    // f_l row (a1, a2) = (i + sL) mod N with sL = N - n; m = k - l for k1 = j1, k2 = j2
    const int a1 = (i1 + N - n) % N, a2 = (i2 + N - n) % N;
    const int m2 = (j2c - i2 + N) % N;
    if (i1 != cur_i1) {  // stage the m1-plane as neighbour pairs
      cur_i1 = i1;
      const int m1 = (j1 - i1 + N) % N;
      const float4 *src = fdr + (long long)m1 * NN;
      __syncthreads();
      for (int e = tid; e < NN; e += blockDim.x) {
        const int row = e / N;
        const int c = e - row * N;
        int cr = c + n;
        if (cr >= N) cr -= N;
        const int cr1 = cr + 1 == N ? 0 : cr + 1;
        const float4 v0 = src[row * N + cr], v1 = src[row * N + cr1];
        const int d = row * N + (c & 3) * R4 + (c >> 2);
        ehi[d] = make_float4(v0.x, v1.x, v0.y, v1.y);
        elo[d] = make_float4(v0.z, v1.z, v0.w, v1.w);
      }
      __syncthreads();
    }
    // E[x] of the row at (x mod 4) R4 + x / 4.  Step i3 = g + t reads
    // x = (4r - i3) mod N: x / 4 = a (the group's a) at t = 0, and for t >= 1
    // x mod 4 = 4 - t with x / 4 = (a - 1) mod R4.
    const float4 *erh = ehi + m2 * N, *erl = elo + m2 * N;
    const float4 *flp = fdr + ((long long)a1 * N + a2) * N;
    const long long lrow0 = ((long long)i1 * N + i2) * N;
    u64 eh[4][2], el[4][2];  // ring[s]: E entry of step i3 with i3 mod 4 = s
    auto load_e = [&](int px, int s) {
      const float4 u = erh[px], w = erl[px];
      eh[s][0] = pk(u.x, u.y);
      eh[s][1] = pk(u.z, u.w);
      el[s][0] = pk(w.x, w.y);
      el[s][1] = pk(w.z, w.w);
    };
    load_e(r, 0);           // x = 4r
    load_e(R4 + r, 3);      // x = 4r + 1: E[x + 1] of step 0 = the entry of step -1
    load_e(2 * R4 + r, 2);  // x = 4r + 2: E[x + 2] of step 0 = the entry of step -2
    const float4 *brow = B2p + lrow0 * KC2 + kcol / 2;
    float4 bv0, bv1, bn0, bn1;
    if (!TMA) {
      bv0 = __ldg(brow + hsw);
      bv1 = __ldg(brow + 1 - hsw);
    }
    float4 fl_next = __ldg(flp);
    int am = r;
    // at N = 24 two groups per iteration (0.304 -> 0.298 ms per launch); at
    // N = 32 that measured 1% slower
#pragma unroll(NC == 24 ? 2 : 1)
    for (int g = 0; g < N; g += RUN, q += RUN) {
      const int an = am == 0 ? R4 - 1 : am - 1;
      const float4 *ring_g = lring + (size_t)(q & 4) * 64;  // ring row q mod 8 = (q & 4) + t
#pragma unroll
      for (int t = 0; t < RUN; ++t) {
        if (TMA) {
          const int slot = ((q & 4) + t) / ROWS;
          if (t % ROWS == 0) mbar_wait_nz(&mybar[slot], (uint32_t)((q >> 3) & 1), to, wait_ns);
          bv0 = ring_g[t * 64];
          bv1 = ring_g[t * 64 + 1 - 2 * hsw];
          if (t % ROWS == ROWS - 1) {
            // every lane has read the slot's rows; refill it with the next
            // ROWS rows unless a lane timed out
            const bool bad = __any_sync(wmask, to);
            const int first = q + t + 1 - ROWS + PDEPTH;
            if (lane == 0 && !bad && first < nrows) {
              const int nr = min(ROWS, nrows - first);
              P64Cursor c = curs[warp];
              asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
              mbar_expect_tx(&mybar[slot], seg_bytes * nr);
              for (int rr = 0; rr < nr; ++rr) {
                bulk_g2s(myring + ((size_t)(slot * ROWS + rr) * 32) * 2, c.src, seg_bytes,
                         &mybar[slot]);
                if (++c.i3 == N) {
                  c.i3 = 0;
                  if (++c.i2 == N) {
                    c.i2 = 0;
                    ++c.pi;
                  }
                  c.src = B2p + ((long long)plane_i1(c.pi) * N + c.i2) * N * KC2 + wcol / 2;
                } else {
                  c.src += KC2;
                }
              }
              ++c.issued;
              curs[warp] = c;
            }
          }
        } else if (g + t + 1 < N) {
          const float4 *bn = brow + (long long)(g + t + 1) * KC2;
          bn0 = __ldg(bn + hsw);
          bn1 = __ldg(bn + 1 - hsw);
        }
        if (t == 0) {
          if (g > 0) load_e(am, 0);
        } else {
          load_e((4 - t) * R4 + an, t);
        }
        const float4 fl = fl_next;
        fl_next = __ldg(flp + g + t + 1);
        const u64 xr = pk(fl.x, fl.x), nxr = pk(-fl.x, -fl.x), nlr = pk(-fl.z, -fl.z);
        const u64 xi = pk(fl.y, fl.y), nxi = pk(-fl.y, -fl.y), nli = pk(-fl.w, -fl.w);
        const u64 li = pk(fl.w, fl.w);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int s = (t + 2 * h) % RUN;
          const float4 bv = h ? bv1 : bv0;
          const u64 bh = pk(bv.x, bv.y), bl = pk(bv.z, bv.w);
          const u64 nbh = mul2(bh, MONE);
          // u = b f_m per part: -u_h rounded, and the exact error plus cross terms
          const u64 nure = mul2(nbh, eh[s][0]);
          const u64 ucre = fma2(bh, el[s][0], fma2(bl, eh[s][0], fma2(bh, eh[s][0], nure)));
          const u64 nuim = mul2(nbh, eh[s][1]);
          const u64 ucim = fma2(bh, el[s][1], fma2(bl, eh[s][1], fma2(bh, eh[s][1], nuim)));
          df_axpy(accR[h], xr, nxr, nlr, nure, ucre);  // + f_l.re u.re
          df_axpy(accR[h], nxi, xi, li, nuim, ucim);   // - f_l.im u.im
          df_axpy(accI[h], xr, nxr, nlr, nuim, ucim);  // + f_l.re u.im
          df_axpy(accI[h], xi, nxi, nli, nure, ucre);  // + f_l.im u.re
        }
        if (!TMA) {
          bv0 = bn0;
          bv1 = bn1;
        }
      }
      am = an;
    }
  }
  if (TMA) {
    if (__syncthreads_or(to)) {
      if (lane == 0) {
        atomicExch(&g_calq64x_status, 1);
        // drain: fill f went into slot f % SLOTS, and a slot is refilled only
        // after its previous fill landed, so only each slot's last fill can
        // still be in flight
        const int issued = curs[warp].issued;
        for (int sl = 0; sl < SLOTS && sl < issued; ++sl) {
          const int last = sl + ((issued - 1 - sl) / SLOTS) * SLOTS;
          bool t2 = false;
          mbar_wait(&mybar[sl], (uint32_t)((last / SLOTS) & 1), t2, DRAIN_LIMIT_NS);
        }
      }
      __syncwarp(wmask);
      return;
    }
  }
  if (!ok) return;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const float2 Rh = upk(accR[h].h), Rl = upk(accR[h].l);
    const float2 Ih = upk(accI[h].h), Il = upk(accI[h].l);
    double2 *o = partial + (long long)chunk * NN * N + kcol + 2 * h;
    o[0] = make_double2((double)Rh.x + (double)Rl.x, (double)Ih.x + (double)Il.x);
    o[1] = make_double2((double)Rh.y + (double)Rl.y, (double)Ih.y + (double)Il.y);
  }
}

struct C64xPlan {
  int J2T, tiles, threads, LC, nch;
  bool tma;
  size_t smem;
};

// Launch shapes (CTA size bound, CTAs per SM the registers must allow):
//   0: 256 threads, 2 CTAs (<= 128 registers)   1: 256, 1 (<= 255)
//   2: 128 threads, 3 CTAs (<= 168)            3: 128, 4 (<= 128)
//   4: 192 threads, 2 CTAs (<= 168)
struct C64xShape {
  int maxt, minb;
};
constexpr C64xShape kC64xShapes[] = {{256, 2}, {256, 1}, {128, 3}, {128, 4}, {192, 2}};
constexpr int kC64xNShapes = (int)(sizeof(kC64xShapes) / sizeof(kC64xShapes[0]));
// The output-pair kernel's shapes (same count): CTA size bound, CTAs per SM,
// table rows per ring slot.  N = 32 (ms per launch): 1.27, 1.37, 1.62, 1.54
// for the first four with 4, 2, 2, 2 rows; 1.45 with one row per slot.
struct C64pShape {
  int maxt, minb, rows;
};
constexpr C64pShape kC64pShapes[] = {{256, 2, 4}, {256, 2, 2}, {128, 3, 2}, {128, 4, 2}, {256, 2, 1}};
static_assert(sizeof(kC64pShapes) / sizeof(kC64pShapes[0]) == kC64xNShapes, "shape count");
// the output-pair kernel runs the pair table when N is a multiple of 4
static bool c64_op(const QParams &p, bool paired) { return paired && p.N % RUN == 0; }

// N fixed at compile time for the output-pair kernel's tensor-copy form at
// these sizes (0: runtime N)
static int c64_nc(const QParams &p, bool op, bool tma) {
  return (op && tma && (p.N == 24 || p.N == 32)) ? p.N : 0;
}
template <bool TMA, int S>
static const void *c64x_fn_s(bool op, int nc) {
  constexpr int T = kC64pShapes[S].maxt, B = kC64pShapes[S].minb, R = kC64pShapes[S].rows;
  if (op) {
    if constexpr (TMA) {
      if (nc == 24) return (const void *)calq64p_kernel<TMA, T, B, R, 24>;
      if (nc == 32) return (const void *)calq64p_kernel<TMA, T, B, R, 32>;
    }
    return (const void *)calq64p_kernel<TMA, T, B, R, 0>;
  }
  return (const void *)calq64x_kernel<TMA, kC64xShapes[S].maxt, kC64xShapes[S].minb>;
}
template <bool TMA>
static const void *c64x_fn(int shape, bool op, int nc) {
  switch (shape) {
    case 0: return c64x_fn_s<TMA, 0>(op, nc);
    case 1: return c64x_fn_s<TMA, 1>(op, nc);
    case 2: return c64x_fn_s<TMA, 2>(op, nc);
    case 3: return c64x_fn_s<TMA, 3>(op, nc);
    default: return c64x_fn_s<TMA, 4>(op, nc);
  }
}

static size_t c64x_smem(int N, int threads, bool tma, bool op, int rows) {
  const int nwarps = (threads + 31) / 32;
  if (op) {
    size_t o = 16 * (size_t)((nwarps * (PDEPTH / rows) * 8 + 15) / 16) + sizeof(P64Cursor) * nwarps;
    if (tma) o += 2 * sizeof(float4) * (size_t)nwarps * PDEPTH * 32;
    return o + 2 * sizeof(float4) * (size_t)N * N;
  }
  size_t o = 16 * (size_t)((nwarps * DEPTH * 8 + 15) / 16);
  if (tma) o += sizeof(float2) * (size_t)nwarps * DEPTH * 32 * RUN;
  return o + sizeof(float4) * (size_t)N * N;
}

// Tile shape, TMA eligibility and the line-chunk count that makes the grid
// whole waves of resident CTAs (cached per shape: the occupancy query is not
// free).
// l-lines of the longest plane list (all N^2 lines, or about half when paired)
static int c64x_lines(const QParams &p, bool paired) {
  if (!paired) return p.N * p.N;
  int m = 0;
  for (int k1 = 0; k1 < p.N; ++k1) m = std::max(m, k1 / 2 + 1 + std::max(0, (k1 + p.N) / 2 - k1));
  return m * p.N;
}

static C64xPlan c64x_plan_compute(const QParams &p, bool aligned, int shape, bool paired);
static C64xPlan c64x_plan(const QParams &p, bool aligned, int shape, bool paired) {
  static std::mutex mu;
  static std::map<long long, C64xPlan> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  const long long key =
      (((((long long)dev * 128 + p.N) * 4 + p.mode) * 2 + (aligned ? 1 : 0)) * 16 + shape) * 2 +
      (paired ? 1 : 0);
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  C64xPlan pl = c64x_plan_compute(p, aligned, shape, paired);
  cache[key] = pl;
  return pl;
}

// shape in [0, 2 kC64xNShapes): the kernel shape shape mod kC64xNShapes, with
// the line chunks sized by whole waves (first half) or by the schedule model
// (second half)
static C64xPlan c64x_plan_compute(const QParams &p, bool aligned, int shape_in, bool paired) {
  C64xPlan pl;
  const int shape = shape_in % kC64xNShapes;
  const bool model = shape_in >= kC64xNShapes;
  const bool op = c64_op(p, paired);
  const int R4 = (p.P + RUN - 1) / RUN;
  int J2T = std::max(1, (op ? kC64pShapes[shape].maxt : kC64xShapes[shape].maxt) / R4);
  if (J2T > p.P) J2T = p.P;
  const int tiles = (p.P + J2T - 1) / J2T;
  J2T = (p.P + tiles - 1) / tiles;
  pl.J2T = J2T;
  pl.tiles = tiles;
  pl.threads = J2T * R4;
  pl.tma = aligned && (p.P % RUN) == 0 && (p.P % J2T) == 0;
  pl.smem = c64x_smem(p.N, pl.threads, pl.tma, op, kC64pShapes[shape].rows);
  int occ = 1;
  const int nc = c64_nc(p, op, pl.tma);
  const void *fn = pl.tma ? c64x_fn<true>(shape, op, nc) : c64x_fn<false>(shape, op, nc);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, pl.threads, pl.smem);
  if (occ < 1) occ = 1;
  const int sms = device_sm_count();
  const long long wave = (long long)sms * occ;
  const long long per_chunk = (long long)p.P * tiles;
  // l-lines each output plane j1 visits (its plane list, or all N planes)
  std::vector<int> nlj(p.P);
  for (int j1 = 0; j1 < p.P; ++j1) {
    const int k1 = (j1 - p.n + p.N) % p.N;
    nlj[j1] = paired ? (k1 / 2 + 1 + std::max(0, (k1 + p.N) / 2 - k1)) * p.N : p.N * p.N;
  }
  const int NL = c64x_lines(p, paired);
  // Whole waves: the chunk count (at most 8 waves) maximising useful CTA-lines
  // / (waves * wave * lines per chunk), chunks sized by the longest list.
  // Schedule model: CTAs start in launch order (j1 fastest, then the j2 tile,
  // then the chunk) on the `wave` resident slots, each as soon as a slot
  // frees, and cost their own lines plus a quarter line; efficiency = useful
  // lines / (makespan * wave).  Neither predicts every table: measured at
  // N = 24 the model's plan is 4% faster, at N = 32 3% slower (1.163 against
  // 1.133 ms), so genB times both.
  double best_eff = -1.0;
  int best_lc = NL;
  for (int ch = 1; ch <= NL; ++ch) {
    const int lc = (NL + ch - 1) / ch;
    const int nch = (NL + lc - 1) / lc;
    if (nch != ch) continue;
    if (per_chunk * nch > 8 * wave) break;
    if (!model) {
      const long long waves = (per_chunk * nch + wave - 1) / wave;
      const double eff = (double)per_chunk * NL / ((double)waves * wave * lc);
      if (eff > best_eff + 1e-9) {
        best_eff = eff;
        best_lc = lc;
      }
      continue;
    }
    std::priority_queue<double, std::vector<double>, std::greater<double>> slots;
    for (long long s = 0; s < wave; ++s) slots.push(0.0);
    double useful = 0.0, makespan = 0.0;
    for (int c = 0; c < nch; ++c)
      for (int t = 0; t < tiles; ++t)
        for (int j1 = 0; j1 < p.P; ++j1) {
          const int w = std::max(0, std::min(lc, nlj[j1] - c * lc));
          useful += w;
          const double f = slots.top() + w + 0.25;
          slots.pop();
          slots.push(f);
          makespan = std::max(makespan, f);
        }
    const double eff = useful / (makespan * (double)wave);
    if (eff > best_eff + 1e-9) {
      best_eff = eff;
      best_lc = lc;
    }
  }
  pl.LC = best_lc;
  pl.nch = (NL + best_lc - 1) / best_lc;
  return pl;
}

int calq64x_nchunk(const QParams &p, int *J2T_out) {
  // upper bound over the variants, used to size the partial-sum buffer
  int n = 1;
  for (int shape = 0; shape < 2 * kC64xNShapes; ++shape)
    for (int al = 0; al <= 1; ++al)
      for (int pa = 0; pa <= 1; ++pa) {
        const C64xPlan pl = c64x_plan(p, al != 0, shape, pa != 0);
        if (J2T_out) *J2T_out = pl.J2T;
        if (pl.nch > n) n = pl.nch;
      }
  return n;
}

edb_status launch_split_f(long long n, const double2 *f, float4 *out, cudaStream_t st) {
  fdf_split_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, f, out);
  EDB_LAUNCHED();
  return EDB_OK;
}

edb_status launch_split_B(long long n, const double *B, float2 *B2, cudaStream_t st) {
  b2_split_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, B, B2);
  EDB_LAUNCHED();
  return EDB_OK;
}

edb_status launch_split_B_paired(int N, const double *B, float2 *B2, cudaStream_t st) {
  const long long n = (long long)N * N * N * N * N * N;
  b2_pair_split_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(N, B, B2);
  EDB_LAUNCHED();
  return EDB_OK;
}

int calq64x_shapes() { return 2 * kC64xNShapes; }

template <bool TMA, int S>
static void c64x_launch_s(dim3 grid, const C64xPlan &pl, const QParams &p, bool paired,
                          const float2 *d_B2, const float4 *d_fdf, double2 *d_partial,
                          cudaStream_t st) {
  constexpr int T = kC64pShapes[S].maxt, B = kC64pShapes[S].minb, R = kC64pShapes[S].rows;
  const float4 *B2p = reinterpret_cast<const float4 *>(d_B2);
  if (c64_op(p, paired)) {
    const int nc = c64_nc(p, true, TMA);
    bool done = false;
    if constexpr (TMA) {
      if (nc == 24) {
        calq64p_kernel<TMA, T, B, R, 24><<<grid, pl.threads, pl.smem, st>>>(
            p, pl.J2T, pl.LC, B2p, d_fdf, d_partial, wait_limit_ns());
        done = true;
      } else if (nc == 32) {
        calq64p_kernel<TMA, T, B, R, 32><<<grid, pl.threads, pl.smem, st>>>(
            p, pl.J2T, pl.LC, B2p, d_fdf, d_partial, wait_limit_ns());
        done = true;
      }
    }
    if (!done)
      calq64p_kernel<TMA, T, B, R, 0><<<grid, pl.threads, pl.smem, st>>>(
          p, pl.J2T, pl.LC, B2p, d_fdf, d_partial, wait_limit_ns());
  } else
    calq64x_kernel<TMA, kC64xShapes[S].maxt, kC64xShapes[S].minb>
        <<<grid, pl.threads, pl.smem, st>>>(p, pl.J2T, pl.LC, paired, d_B2, d_fdf, d_partial,
                                            wait_limit_ns());
}
template <bool TMA>
static void c64x_launch(int shape, dim3 grid, const C64xPlan &pl, const QParams &p, bool paired,
                        const float2 *d_B2, const float4 *d_fdf, double2 *d_partial,
                        cudaStream_t st) {
  switch (shape) {
    case 0: c64x_launch_s<TMA, 0>(grid, pl, p, paired, d_B2, d_fdf, d_partial, st); break;
    case 1: c64x_launch_s<TMA, 1>(grid, pl, p, paired, d_B2, d_fdf, d_partial, st); break;
    case 2: c64x_launch_s<TMA, 2>(grid, pl, p, paired, d_B2, d_fdf, d_partial, st); break;
    case 3: c64x_launch_s<TMA, 3>(grid, pl, p, paired, d_B2, d_fdf, d_partial, st); break;
    default: c64x_launch_s<TMA, 4>(grid, pl, p, paired, d_B2, d_fdf, d_partial, st); break;
  }
}

edb_status launch_calq64x(const QParams &p, const float2 *d_B2, const double2 *d_in,
                          float4 *d_fdf, double2 *d_partial, double2 *d_Q, cudaStream_t st,
                          int shape, bool paired) {
  if (shape < 0 || shape >= 2 * kC64xNShapes) shape = 0;
  if (paired && (p.P != p.N || (p.sM % p.N) != 0 || (p.sL % p.N) != p.N - p.n))
    return fail(EDB_EINVAL, "calq64x: pairs need the aliased index shifts");
  if (c64_op(p, paired)) {
    fdr_split_kernel<<<(unsigned)((p.NQ + 1 + 255) / 256), 256, 0, st>>>(p.N, p.sL % p.N, d_in,
                                                                        d_fdf);
  } else {
    fdf_split_kernel<<<(unsigned)((p.NQ + 255) / 256), 256, 0, st>>>(p.NQ, d_in, d_fdf);
  }
  EDB_LAUNCHED();
  const bool aligned = ((uintptr_t)d_B2 % 16) == 0;
  if (c64_op(p, paired) && !aligned)
    return fail(EDB_EINVAL, "calq64x: the output-pair table must be 16-byte aligned");
  const C64xPlan pl = c64x_plan(p, aligned, shape, paired);
  dim3 grid((unsigned)p.P, (unsigned)pl.tiles, (unsigned)pl.nch);
  if (pl.tma)
    c64x_launch<true>(shape % kC64xNShapes, grid, pl, p, paired, d_B2, d_fdf, d_partial, st);
  else
    c64x_launch<false>(shape % kC64xNShapes, grid, pl, p, paired, d_B2, d_fdf, d_partial, st);
  EDB_LAUNCHED();
  return launch_calq64_reduce(p, pl.nch, d_partial, d_Q, st);
}

edb_status read_calq64x_status(int *status, bool clear) {
  int v = 0;
  EDB_CUDA(cudaMemcpyFromSymbol(&v, g_calq64x_status, sizeof(int)));
  if (clear && v) {
    int z = 0;
    EDB_CUDA(cudaMemcpyToSymbol(g_calq64x_status, &z, sizeof(int)));
  }
  *status = v;
  return EDB_OK;
}

}  // namespace edb
