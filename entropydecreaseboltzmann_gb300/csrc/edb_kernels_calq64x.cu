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
// Tiling: CTA = (output plane j1, a tile of j2, all j3) x (a chunk of row
// planes i1).  Thread = (j2, run of 4 consecutive j3).  For each i1 the f-hat
// m1-plane (m1 = j1 - i1 + sM mod N) is staged in shared memory; along i3 the
// needed f_m slide down by one (a ring of 4).  B rows are streamed from HBM
// with 16-byte loads, two rows ahead in registers.  Each CTA writes FP64
// partial sums per row chunk; calq64_reduce_kernel adds the chunks in order.
#include "edb_internal.cuh"

namespace edb {

namespace {
typedef unsigned long long u64;
constexpr int RUN = 4;  // outputs per thread along j3

__device__ __forceinline__ u64 pk(float a, float b) {
  u64 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
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
__device__ __forceinline__ u64 fma2(u64 a, u64 b, u64 c) {
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

struct DF2 {  // packed double-float pair: lanes (re, im)
  u64 h, l;
};

// acc += s * u for a real double-float scalar s (given as the pairs (s_h, s_h),
// (-s_h, -s_h), (-s_l, -s_l)) and u = -nu_h + uc.
__device__ __forceinline__ void df_axpy(DF2 &acc, u64 sh2, u64 nsh2, u64 nsl2, u64 nu_h, u64 uc) {
  // leading product s_h * u_h = s_h * (-nu_h): nph = -(s_h u_h) rounded, pe exact error
  const u64 nph = mul2(sh2, nu_h);       // = -rn(s_h u_h)
  const u64 pe = fma2(nsh2, nu_h, nph);  // = s_h u_h - rn(s_h u_h)
  // cross terms s_h * uc + s_l * u_h  (u_h = -nu_h, so s_l u_h = (-s_l) nu_h)
  const u64 pl = fma2(sh2, uc, fma2(nsl2, nu_h, pe));
  // two-sum of acc.h and p_h = -nph
  const u64 s = sub2(acc.h, nph);
  const u64 bb = sub2(s, acc.h);  // ~ p_h
  const u64 e = sub2(sub2(acc.h, sub2(s, bb)), add2(nph, bb));  // (acc.h - (s - bb)) + (p_h - bb)
  acc.h = s;
  acc.l = add2(acc.l, add2(e, pl));
}
}  // namespace

__global__ void fdf_split_kernel(long long n, const double2 *__restrict__ f, float4 *__restrict__ out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 v = f[i];
  const float rh = (float)v.x, ih = (float)v.y;
  const float rl = (float)(v.x - (double)rh), il = (float)(v.y - (double)ih);
  out[i] = make_float4(rh, ih, rl, il);
}

__global__ void b2_split_kernel(long long n, const double *__restrict__ B, float2 *__restrict__ B2) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = B[i];
  const float h = (float)v;
  B2[i] = make_float2(h, (float)(v - (double)h));
}

template <int MAXT>
__global__ void __launch_bounds__(MAXT, 2)
    calq64x_kernel(QParams p, int J2T, int L1C, const float2 *__restrict__ B2,
                   const float4 *__restrict__ fdf, double2 *__restrict__ partial) {
  extern __shared__ __align__(16) float4 plane[];  // [N][N] of the current m1
  const int N = p.N, P = p.P;
  const int R4 = (P + RUN - 1) / RUN;
  const int tid = threadIdx.x;
  const int r = tid % R4;
  const int j2l = tid / R4;
  const int j1 = blockIdx.x;
  const int j2 = blockIdx.y * J2T + j2l;
  const bool ok = (j2l < J2T) && (j2 < P);
  const int j2c = ok ? j2 : 0;
  const int j3_0 = r * RUN;
  const int chunk = blockIdx.z;
  const int i1_0 = chunk * L1C, i1_1 = min(N, i1_0 + L1C);
  const long long NN = (long long)N * N;
  const long long kcol = ((long long)j1 * P + j2c) * P + j3_0;
  // columns past P (ragged last run) read a clamped, in-row column and are
  // masked out of the output
  int colc[RUN];
#pragma unroll
  for (int a = 0; a < RUN; ++a) colc[a] = (j3_0 + a < P) ? a : 0;

  DF2 accA[RUN], accB[RUN];
#pragma unroll
  for (int a = 0; a < RUN; ++a) {
    accA[a].h = accA[a].l = 0ull;
    accB[a].h = accB[a].l = 0ull;
  }

  for (int i1 = i1_0; i1 < i1_1; ++i1) {
    const int m1 = ((j1 - i1 + p.sM) % N + N) % N;
    __syncthreads();
    for (long long e = tid; e < NN; e += blockDim.x) plane[e] = fdf[(long long)m1 * NN + e];
    __syncthreads();
    const int a1 = (i1 + p.sL) % N;
    for (int i2 = 0; i2 < N; ++i2) {
      const int m2 = ((j2c - i2 + p.sM) % N + N) % N;
      const int a2 = (i2 + p.sL) % N;
      const float4 *prow = plane + (long long)m2 * N;
      const float4 *flrow = fdf + ((long long)a1 * N + a2) * N;
      const long long lrow0 = ((long long)i1 * N + i2) * N;
      // ring of f_m along i3: slot(a, i3) = (a - i3) mod 4
      u64 rh[RUN], rl[RUN];
#pragma unroll
      for (int a = 0; a < RUN; ++a) {
        const int m3 = (j3_0 + a + p.sM) % N;
        const float4 v = prow[m3];
        rh[a] = pk(v.x, v.y);
        rl[a] = pk(v.z, v.w);
      }
      // B rows: two in flight
      const float2 *brow = B2 + lrow0 * p.KC + kcol;
      float2 bcur[RUN], bnext[RUN];
#pragma unroll
      for (int a = 0; a < RUN; ++a) bcur[a] = __ldg(brow + colc[a]);
      for (int g = 0; g < N; g += RUN) {
#pragma unroll
        for (int t = 0; t < RUN; ++t) {
          const int i3 = g + t;
          if (i3 >= N) break;
          if (i3 + 1 < N) {
            const float2 *bn = brow + (long long)(i3 + 1) * p.KC;
#pragma unroll
            for (int a = 0; a < RUN; ++a) bnext[a] = __ldg(bn + colc[a]);
          }
          if (i3 > 0) {  // new ring value enters at a = 0
            int m3 = (j3_0 - i3 + p.sM) % N;
            if (m3 < 0) m3 += N;
            const float4 v = prow[m3];
            const int slot = (RUN - t) % RUN;
            rh[slot] = pk(v.x, v.y);
            rl[slot] = pk(v.z, v.w);
          }
          const float4 fl = __ldg(flrow + (i3 + p.sL) % N);
          // broadcast pairs of f_l.re and f_l.im (hi; and negated hi, lo)
          const u64 xr = pk(fl.x, fl.x), nxr = pk(-fl.x, -fl.x), nlr = pk(-fl.z, -fl.z);
          const u64 xi = pk(fl.y, fl.y), nxi = pk(-fl.y, -fl.y), nli = pk(-fl.w, -fl.w);
#pragma unroll
          for (int a = 0; a < RUN; ++a) {
            const int slot = (a - t + RUN) % RUN;
            const float bh = bcur[a].x, bl = bcur[a].y;
            const u64 nbh2 = pk(-bh, -bh), bh2 = pk(bh, bh), bl2 = pk(bl, bl);
            // u = b * f_m:  nu_h = -(b_h f_m,h), uc = exact error + cross terms
            const u64 nu_h = mul2(nbh2, rh[slot]);
            const u64 ue = fma2(bh2, rh[slot], nu_h);
            const u64 uc = fma2(bh2, rl[slot], fma2(bl2, rh[slot], ue));
            df_axpy(accA[a], xr, nxr, nlr, nu_h, uc);
            df_axpy(accB[a], xi, nxi, nli, nu_h, uc);
          }
#pragma unroll
          for (int a = 0; a < RUN; ++a) bcur[a] = bnext[a];
        }
      }
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

// Chunks over i1 so that the grid covers the SMs a few times over.
int calq64x_nchunk(const QParams &p, int *J2T_out) {
  const int R4 = (p.P + RUN - 1) / RUN;
  int J2T = 256 / R4;
  if (J2T > p.P) J2T = p.P;
  const int tiles = (p.P + J2T - 1) / J2T;
  J2T = (p.P + tiles - 1) / tiles;
  if (J2T_out) *J2T_out = J2T;
  long long ctas = (long long)p.P * tiles;
  int nchunk = (int)((4LL * 152 + ctas - 1) / ctas);
  if (nchunk > p.N) nchunk = p.N;
  if (nchunk < 1) nchunk = 1;
  return nchunk;
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

edb_status launch_calq64x(const QParams &p, const float2 *d_B2, const float4 *d_fdf,
                          double2 *d_partial, double2 *d_Q, cudaStream_t st) {
  int J2T = 0;
  const int nchunk = calq64x_nchunk(p, &J2T);
  const int L1C = (p.N + nchunk - 1) / nchunk;
  const int nch = (p.N + L1C - 1) / L1C;
  const int R4 = (p.P + RUN - 1) / RUN;
  const int threads = J2T * R4;
  const int tiles = (p.P + J2T - 1) / J2T;
  const size_t smem = sizeof(float4) * (size_t)p.N * p.N;
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(calq64x_kernel<256>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(calq64x)");
    configured = true;
  }
  dim3 grid((unsigned)p.P, (unsigned)tiles, (unsigned)nch);
  calq64x_kernel<256><<<grid, threads, smem, st>>>(p, J2T, L1C, d_B2, d_fdf, d_partial);
  EDB_LAUNCHED();
  return launch_calq64_reduce(p, nch, d_partial, d_Q, st);
}

}  // namespace edb
