// FP64-accurate collision sum with the kernel table evaluated on the fly (no
// N^6 table).
//
// QCalculator::genB (CalQ/QCalculator.h:158-229) stores beta(l, k) for every
// (l, k): N^6 doubles, 8.6 GB at N = 32 and 550 GB at N = 64.  Yet beta depends
// on (l, m = k - l) only through the integer squared norms a = |l + m|^2 and
// b = |l - m|^2, the per-axis filter factors and the self-interaction term
// (QCalculator.h:204-224):
//   beta(l, k) = T(a, b) sigma(l) sigma(m) rval - Bmm[m],
//   T(a, b)    = F(lambda pi sqrt(a), lambda pi sqrt(b)),
// and the terms l and m of a Q-hat sum share the product f_l f_m, so the
// double-float kernel's pair entry (edb_kernels_calq64x.cu) is
//   beta(l, k) + beta(m, k) = 2 T(a, b) sigma(l) sigma(m) rval - Bmm[l] - Bmm[m]
// off the planes l1 = m1, and beta(l, k) alone on them.  This kernel forms that
// entry per term from three small tables instead of streaming it:
//   tc  T(a, b) rval split into {hi, lo}; (l + m)^2 - (l - m)^2 = 4 l.m, so
//       a = b mod 4 and only b = (a mod 4) + 4q is stored: row a, column q,
//       (amax + 1) x (amax / 4 + 1) entries (19 MB at N = 32, 302 MB at N = 64);
//   bs  per mode, in FFTW order: {Bmm hi, Bmm lo, sigma3 hi, sigma3 lo}, with
//       sigma3 = sigma(c1) sigma(c2) sigma(c3) (1 with the filter off);
// and the same (already split) f-hat as the streamed kernel.  The pair entry is
// formed in double-float arithmetic (sdf_* helpers), then the term runs exactly
// as in calq64x_kernel.  Only the aliased index shifts (ALIASED mode, or odd N)
// have the pair structure, as for the streamed pair table.
//
// Tiling as calq64x_kernel: CTA = (output plane j1, a tile of j2, all j3) x (a
// chunk of the visited l-lines); thread = (j2, a run of RUN consecutive j3).
// Per l1-plane the f-hat m1-plane and the bs m1-plane are staged in shared
// memory; along i3 the entries f_m and bs_m of each output slide down by one,
// so they live in a register ring (one new entry per step).  The tc entries
// are gathered from global memory (L2-resident) one step ahead of their use.
// Each CTA writes FP64 partial sums per chunk; calq64_reduce_kernel adds the
// chunks in order.  No waits: nothing here is staged asynchronously.
#include <algorithm>
#include <map>
#include <mutex>

#include "edb_df.cuh"
#include "edb_internal.cuh"

namespace edb {

namespace {
using namespace df;
constexpr int RUN = 4;  // outputs per thread along j3
constexpr int THREADS = 256;
// two CTAs per SM: at most 128 registers a thread (no spills), 16 warps per SM
// against 7 with 186 registers; N = 24: 0.714 -> 0.476 ms, N = 32: 2.30 ->
// 2.03 ms.  The kernel is bound by the latency of its double-float chains.
constexpr int MINB = 2;

// tc[a][q] = T[a][(a mod 4) + 4 q] * rval, split (0 past amax).
__global__ void tc_kernel(int amax, int rl, double rval, const double *__restrict__ T,
                          float2 *__restrict__ tc) {
  const long long n = (long long)(amax + 1) * rl;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(i / rl), q = (int)(i - (long long)a * rl);
    const int b = (a & 3) + 4 * q;
    const double v = b <= amax ? T[(long long)a * (amax + 1) + b] * rval : 0.0;
    const float h = (float)v;
    tc[i] = make_float2(h, (float)(v - (double)h));
  }
}

// bs[f] for FFTW flat index f: Bmm and sigma3 of the mode's centred index.
__global__ void bs_kernel(int N, int filter, const double *__restrict__ sigma,
                          const double *__restrict__ Bmm, float4 *__restrict__ bs) {
  const long long NQ = (long long)N * N * N;
  const long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= NQ) return;
  const int n = (N - 1) / 2;
  const int f1 = (int)(f / ((long long)N * N)), f2 = (int)((f / N) % N), f3 = (int)(f % N);
  const int c1 = (f1 + n) % N, c2 = (f2 + n) % N, c3 = (f3 + n) % N;
  const double bm = Bmm[((long long)c1 * N + c2) * N + c3];
  const double s3 = filter ? sigma[c1] * sigma[c2] * sigma[c3] : 1.0;
  const float bh = (float)bm, sh = (float)s3;
  bs[f] = make_float4(bh, (float)(bm - (double)bh), sh, (float)(s3 - (double)sh));
}

// FIL: the filter is on (sigma3 products enter the entry).
template <bool FIL>
__global__ void __launch_bounds__(THREADS, MINB)
    calq64f_kernel(QParams p, int J2T, int LC, int rl, const float2 *__restrict__ tc,
                   const float4 *__restrict__ bs, const float4 *__restrict__ fdf,
                   double2 *__restrict__ partial) {
  extern __shared__ __align__(16) unsigned char smem64f[];
  const int N = p.N, P = p.P, n = p.n;
  const int R4 = (P + RUN - 1) / RUN;
  const int tid = threadIdx.x;
  const long long NN = (long long)N * N;
  float4 *plane = reinterpret_cast<float4 *>(smem64f);  // f-hat m1-plane [N][N]
  float4 *planeb = plane + NN;                          // bs m1-plane [N][N]

  const int r = tid % R4;
  const int j2l = tid / R4;
  const int j1 = blockIdx.x;
  const int j2 = blockIdx.y * J2T + j2l;
  const bool ok = (j2l < J2T) && (j2 < P);
  const int j2c = ok ? j2 : 0;
  const int j3_0 = r * RUN;
  const int chunk = blockIdx.z;
  // visited l1 planes of the pair structure (see calq64x_kernel)
  const int k1f = (j1 - n + N) % N;
  const int plo = k1f / 2;
  const int nlist = plo + 1 + max(0, (k1f + N) / 2 - k1f);
  auto plane_i1 = [&](int pi) {
    const int a = pi <= plo ? pi : k1f + 1 + (pi - plo - 1);
    return (a + n) % N;
  };
  const int NL = nlist * N;
  const int c0 = min(NL, chunk * LC), c1 = min(NL, c0 + LC);
  const long long kcol = ((long long)j1 * P + j2c) * P + j3_0;

  DF2 accA[RUN], accB[RUN];
#pragma unroll
  for (int a = 0; a < RUN; ++a) {
    accA[a].h = accA[a].l = 0ull;
    accB[a].h = accB[a].l = 0ull;
  }

  const int base3 = j3_0 % N;  // FFTW m3 of output a = 0 at i3 = 0 (sM = 0)
  const int fi0 = p.sL % N;     // FFTW l3 at i3 = 0
  int cur_i1 = -1;
  bool pair = true;
  int x1 = 0, e1 = 0;
  // line indices advanced by counters (no division per line): list plane pi
  // with i1 = plane_i1(pi), row i2; a1, a2 = (i + sL) mod N; the FFTW index
  // m2f = (j2 - i2) mod N of m2
  int pi = c0 / N, i2 = c0 % N;
  int i1 = plane_i1(pi), a1 = (i1 + p.sL) % N, a2 = (i2 + p.sL) % N;
  int m2f = ((j2c - i2) % N + N) % N;
  for (int line = c0; line < c1; ++line) {
    if (line > c0) {
      if (++i2 == N) {
        i2 = 0;
        i1 = plane_i1(++pi);
        a1 = (i1 + p.sL) % N;
      }
      a2 = (a2 + 1 == N) ? 0 : a2 + 1;
      m2f = (m2f == 0) ? N - 1 : m2f - 1;
    }
    if (i1 != cur_i1) {  // stage the m1-planes of f-hat and bs
      cur_i1 = i1;
      const int m1f = ((j1 - i1) % N + N) % N;
      const int m1c = (j1 - i1 + n + N) % N;
      pair = (m1c != i1);
      x1 = i1 + m1c - 2 * n;
      e1 = i1 - m1c;
      __syncthreads();
      for (long long e = tid; e < NN; e += blockDim.x) {
        plane[e] = fdf[(long long)m1f * NN + e];
        planeb[e] = bs[(long long)m1f * NN + e];
      }
      __syncthreads();
    }
    const int m2c = (j2c - i2 + n + N) % N;
    const int x2 = i2 + m2c - 2 * n, e2 = i2 - m2c;
    const int A12 = x1 * x1 + x2 * x2, B12 = e1 * e1 + e2 * e2;
    const float4 *prow = plane + (long long)m2f * N;
    const float4 *brow = planeb + (long long)m2f * N;
    const float4 *flrow = fdf + ((long long)a1 * N + a2) * N;
    const float4 *blrow = bs + ((long long)a1 * N + a2) * N;
    // ring of f_m {hi, lo} pairs and bs_m per output; centred m3 per output
    u64 rh[RUN], rl_[RUN];
    float4 rb[RUN];
    int m3c[RUN];
#pragma unroll
    for (int a = 0; a < RUN; ++a) {
      int m3 = base3 + a;
      while (m3 >= N) m3 -= N;
      const float4 v = prow[m3];
      rh[a] = pk(v.x, v.y);
      rl_[a] = pk(v.z, v.w);
      rb[a] = brow[m3];
      m3c[a] = (m3 + n) % N;
    }
    // the tc entries of step i3 for each output: row a, column (b >> 2)
    auto tc_at = [&](int i3, int mc) {
      const int x3 = i3 + mc - 2 * n, e3 = i3 - mc;
      const int aa = A12 + x3 * x3, bb = B12 + e3 * e3;
      return __ldg(tc + (long long)aa * rl + (bb >> 2));
    };
    float2 tcur[RUN];
#pragma unroll
    for (int a = 0; a < RUN; ++a) tcur[a] = tc_at(0, m3c[a]);
    int m3n = base3;
    int fi = fi0;
    float4 fl_next = __ldg(flrow + fi), bl_next = __ldg(blrow + fi);
    for (int g = 0; g < N; g += RUN) {
#pragma unroll
      for (int t = 0; t < RUN; ++t) {
        const int i3 = g + t;
        if (i3 >= N) break;
        if (i3 > 0) {  // new ring entry at output a = 0
          m3n = (m3n == 0) ? N - 1 : m3n - 1;
          const float4 v = prow[m3n];
          const int slot = (RUN - t) % RUN;
          rh[slot] = pk(v.x, v.y);
          rl_[slot] = pk(v.z, v.w);
          rb[slot] = brow[m3n];
        }
        // prefetch the next step's tc entries (centred m3 of each output
        // moves down by one per step)
        float2 tnext[RUN];
#pragma unroll
        for (int a = 0; a < RUN; ++a) {
          m3c[a] = (m3c[a] == 0) ? N - 1 : m3c[a] - 1;
          if (i3 + 1 < N) tnext[a] = tc_at(i3 + 1, m3c[a]);
        }
        const float4 fl = fl_next, bl = bl_next;
        fi = (fi + 1 == N) ? 0 : fi + 1;
        fl_next = __ldg(flrow + fi);
        bl_next = __ldg(blrow + fi);
        const u64 xr = pk(fl.x, fl.x), nxr = pk(-fl.x, -fl.x), nlr = pk(-fl.z, -fl.z);
        const u64 xi = pk(fl.y, fl.y), nxi = pk(-fl.y, -fl.y), nli = pk(-fl.w, -fl.w);
        const float2 Bl = make_float2(bl.x, bl.y), sl = make_float2(bl.z, bl.w);
        u64 nuh[RUN], ucs[RUN];
#pragma unroll
        for (int a = 0; a < RUN; ++a) {
          const int slot = (a - t + RUN) % RUN;
          const float4 bm = rb[slot];
          // the pair entry: 2 T rval sigma(l) sigma(m) - Bmm[l] - Bmm[m], or
          // T rval sigma(l) sigma(m) - Bmm[m] on the self planes
          float2 q = tcur[a];
          if (FIL) q = sdf_mul(q, sdf_mul(sl, make_float2(bm.z, bm.w)));
          const float2 Bm = make_float2(bm.x, bm.y);
          const float2 e = pair ? sdf_add(make_float2(2.f * q.x, 2.f * q.y),
                                          sdf_neg(sdf_add(Bl, Bm)))
                                : sdf_add(q, sdf_neg(Bm));
          const float bh = e.x, blo = e.y;
          const u64 nbh2 = pk(-bh, -bh), bh2 = pk(bh, bh), bl2 = pk(blo, blo);
          // u = b * f_m:  nu_h = -(b_h f_m,h), uc = exact error + cross terms
          nuh[a] = mul2(nbh2, rh[slot]);
          const u64 ue = fma2(bh2, rh[slot], nuh[a]);
          ucs[a] = fma2(bh2, rl_[slot], fma2(bl2, rh[slot], ue));
        }
#pragma unroll
        for (int a = 0; a < RUN; ++a) df_axpy(accA[a], xr, nxr, nlr, nuh[a], ucs[a]);
#pragma unroll
        for (int a = 0; a < RUN; ++a) df_axpy(accB[a], xi, nxi, nli, nuh[a], ucs[a]);
#pragma unroll
        for (int a = 0; a < RUN; ++a)
          if (i3 + 1 < N) tcur[a] = tnext[a];
      }
    }
  }
  if (!ok) return;
#pragma unroll
  for (int a = 0; a < RUN; ++a) {
    if (j3_0 + a >= P) continue;
    const float2 Ah = upk(accA[a].h), Al = upk(accA[a].l);
    const float2 Bh = upk(accB[a].h), Bl2 = upk(accB[a].l);
    const double re = ((double)Ah.x + (double)Al.x) - ((double)Bh.y + (double)Bl2.y);
    const double im = ((double)Ah.y + (double)Al.y) + ((double)Bh.x + (double)Bl2.x);
    partial[(long long)chunk * p.KC + kcol + a] = make_double2(re, im);
  }
}

struct C64fPlan {
  int J2T, tiles, threads, LC, nch;
  size_t smem;
};

// l-lines of the longest visited plane list
int c64f_lines(const QParams &p) {
  int m = 0;
  for (int k1 = 0; k1 < p.N; ++k1) m = std::max(m, k1 / 2 + 1 + std::max(0, (k1 + p.N) / 2 - k1));
  return m * p.N;
}

C64fPlan c64f_plan(const QParams &p) {
  C64fPlan pl;
  const int R4 = (p.P + RUN - 1) / RUN;
  int J2T = THREADS / R4;
  if (J2T > p.P) J2T = p.P;
  const int tiles = (p.P + J2T - 1) / J2T;
  J2T = (p.P + tiles - 1) / tiles;
  pl.J2T = J2T;
  pl.tiles = tiles;
  pl.threads = J2T * R4;
  pl.smem = 2 * sizeof(float4) * (size_t)p.N * p.N;
  // enough CTAs for about four per SM, in whole line chunks
  const long long per_chunk = (long long)p.P * tiles;
  const int NL = c64f_lines(p);
  long long want = (4LL * device_sm_count() + per_chunk - 1) / per_chunk;
  if (want < 1) want = 1;
  if (want > NL) want = NL;
  pl.LC = (int)((NL + want - 1) / want);
  pl.nch = (NL + pl.LC - 1) / pl.LC;
  return pl;
}

}  // namespace

int calq64f_nchunk(const QParams &p) { return c64f_plan(p).nch; }

int calq64f_row_len(int amax) { return amax / 4 + 1; }

edb_status launch_calq64f_tables(int N, int filter, double rval, const double *d_T, int amax,
                                 const double *d_sigma, const double *d_Bmm, float2 *d_tc,
                                 float4 *d_bs, cudaStream_t st) {
  const int rl = calq64f_row_len(amax);
  const long long nt = (long long)(amax + 1) * rl;
  const long long blocks = std::min<long long>((nt + 255) / 256, 32LL * device_sm_count());
  tc_kernel<<<(unsigned)blocks, 256, 0, st>>>(amax, rl, rval, d_T, d_tc);
  EDB_LAUNCHED();
  const long long NQ = (long long)N * N * N;
  bs_kernel<<<(unsigned)((NQ + 255) / 256), 256, 0, st>>>(N, filter, d_sigma, d_Bmm, d_bs);
  EDB_LAUNCHED();
  return EDB_OK;
}

edb_status launch_calq64f(const QParams &p, int filter, int amax, const float2 *d_tc,
                          const float4 *d_bs, const float4 *d_fdf, double2 *d_partial,
                          double2 *d_Q, cudaStream_t st) {
  if (p.P != p.N || (p.sM % p.N) != 0 || (p.sL % p.N) != p.N - p.n)
    return fail(EDB_EINVAL, "calq64f: the on-the-fly table needs the aliased index shifts");
  const C64fPlan pl = c64f_plan(p);
  const void *fn = filter ? (const void *)calq64f_kernel<true> : (const void *)calq64f_kernel<false>;
  static std::mutex mu;
  {
    // the planes need more than the default 48 KB above N = 38
    std::lock_guard<std::mutex> lock(mu);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)std::max<size_t>(pl.smem, 48 * 1024));
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(calq64f)");
  }
  dim3 grid((unsigned)p.P, (unsigned)pl.tiles, (unsigned)pl.nch);
  const int rl = calq64f_row_len(amax);
  if (filter)
    calq64f_kernel<true><<<grid, pl.threads, pl.smem, st>>>(p, pl.J2T, pl.LC, rl, d_tc, d_bs,
                                                            d_fdf, d_partial);
  else
    calq64f_kernel<false><<<grid, pl.threads, pl.smem, st>>>(p, pl.J2T, pl.LC, rl, d_tc, d_bs,
                                                             d_fdf, d_partial);
  EDB_LAUNCHED();
  return launch_calq64_reduce(p, pl.nch, d_partial, d_Q, st);
}

}  // namespace edb
