// Batched cubic 3-D DFT with the conventions of the reference's fft3d
// (CalQ/fft3d.h:25-48): forward = FFTW_FORWARD (exp(-2 pi i jk/N)),
// unnormalised; inverse = FFTW_BACKWARD then every element times 1./N^3.
//
// Three passes (axis 2, 1, 0) make the 3-D transform.  A pass loads one N x N
// tile of a cube (N lines of the transform axis) into shared memory, line by
// line, and runs a mixed-radix Stockham FFT on every line: N = r_1 r_2 ... r_m
// with radix-4 and radix-2 stages first (butterflies of additions and +-i
// swaps), then the odd prime factors in ascending order: radix 3 as a
// butterfly, any other odd radix R as one sum of R terms per output against
// the twiddle table exp(sign 2 pi i m/N) (the stage's input twiddle and its
// R-point DFT folded into one table index), so a prime N is the direct DFT.  Stockham's
// self-sorting form ping-pongs between two line buffers and leaves the result
// in natural order.  The per-point cost is sum(r_i) complex operations instead
// of N, e.g. 4 + 2 + 3 against 24 at N = 24.
//
// Three arithmetic types: double2 (FP64), float2 (FP32) and dfc, FP64 data
// in memory with double-float arithmetic in the passes (each part an
// unevaluated hi + lo float pair, edb_df.cuh): GB300 runs native FP64 at a
// small fraction of its FP32 rate, and the FP64 passes of the batch's step
// were bound by it (2.7 ms per pass at 4096 x N = 24).  Double-float keeps
// about 2^-47 relative per operation.
#include <type_traits>

#include "edb_df.cuh"
#include "edb_internal.cuh"

namespace edb {

// complex double-float value: re = rh + rl, im = ih + il
struct __align__(16) dfc {
  float rh, rl, ih, il;
};

namespace {
using df::fast_two_sum;
using df::sdf_add;
using df::sdf_mul;
using df::sdf_neg;

__device__ __forceinline__ float2 dsplit(double x) {
  const float h = (float)x;
  return make_float2(h, (float)(x - (double)h));
}
__device__ __forceinline__ dfc mk_dfc(float2 re, float2 im) { return dfc{re.x, re.y, im.x, im.y}; }
__device__ __forceinline__ float2 dre(const dfc &a) { return make_float2(a.rh, a.rl); }
__device__ __forceinline__ float2 dim(const dfc &a) { return make_float2(a.ih, a.il); }
constexpr int FFT_MAX_STAGES = 16;
constexpr int FFT_THREADS = 256;

struct FftPlan {
  int nst;
  int radix[FFT_MAX_STAGES];
};

// 4s, then 2s, then odd prime factors in ascending order.
FftPlan fft_plan(int N) {
  FftPlan p;
  p.nst = 0;
  int n = N;
  while (n % 4 == 0 && p.nst < FFT_MAX_STAGES) {
    p.radix[p.nst++] = 4;
    n /= 4;
  }
  while (n % 2 == 0 && p.nst < FFT_MAX_STAGES) {
    p.radix[p.nst++] = 2;
    n /= 2;
  }
  for (int f = 3; n > 1 && p.nst < FFT_MAX_STAGES; f += 2)
    while (n % f == 0 && p.nst < FFT_MAX_STAGES) {
      p.radix[p.nst++] = f;
      n /= f;
    }
  return p;
}

template <typename R2>
__device__ __forceinline__ R2 c_add(R2 a, R2 b) {
  R2 r;
  r.x = a.x + b.x;
  r.y = a.y + b.y;
  return r;
}
template <typename R2>
__device__ __forceinline__ R2 c_sub(R2 a, R2 b) {
  R2 r;
  r.x = a.x - b.x;
  r.y = a.y - b.y;
  return r;
}
template <typename R2>
__device__ __forceinline__ R2 c_mul(R2 a, R2 w) {
  R2 r;
  r.x = a.x * w.x - a.y * w.y;
  r.y = a.x * w.y + a.y * w.x;
  return r;
}
template <>
__device__ __forceinline__ dfc c_add<dfc>(dfc a, dfc b) {
  return mk_dfc(sdf_add(dre(a), dre(b)), sdf_add(dim(a), dim(b)));
}
template <>
__device__ __forceinline__ dfc c_sub<dfc>(dfc a, dfc b) {
  return mk_dfc(sdf_add(dre(a), sdf_neg(dre(b))), sdf_add(dim(a), sdf_neg(dim(b))));
}
template <>
__device__ __forceinline__ dfc c_mul<dfc>(dfc a, dfc w) {
  return mk_dfc(sdf_add(sdf_mul(dre(a), dre(w)), sdf_neg(sdf_mul(dim(a), dim(w)))),
                sdf_add(sdf_mul(dre(a), dim(w)), sdf_mul(dim(a), dre(w))));
}
// sign i t (sign = +-1): exact
template <typename R2>
__device__ __forceinline__ R2 c_rot(R2 t, int sign) {
  R2 d;
  d.x = -sign * t.y;
  d.y = sign * t.x;
  return d;
}
template <>
__device__ __forceinline__ dfc c_rot<dfc>(dfc t, int sign) {
  return sign > 0 ? dfc{-t.ih, -t.il, t.rh, t.rl} : dfc{t.ih, t.il, -t.rh, -t.rl};
}
// radix-3 parts: t = v0 - s / 2, u = i h d (h real)
template <typename R2>
__device__ __forceinline__ void r3_parts(R2 v0, R2 sm, R2 df, R2 hw, R2 &t, R2 &u) {
  const auto h = hw.y;
  t.x = v0.x - 0.5f * sm.x;
  t.y = v0.y - 0.5f * sm.y;
  u.x = -h * df.y;
  u.y = h * df.x;
}
template <>
__device__ __forceinline__ void r3_parts<dfc>(dfc v0, dfc sm, dfc df, dfc hw, dfc &t, dfc &u) {
  const float2 h = dim(hw);
  // halving is exact in both parts
  t = mk_dfc(sdf_add(dre(v0), make_float2(-0.5f * sm.rh, -0.5f * sm.rl)),
             sdf_add(dim(v0), make_float2(-0.5f * sm.ih, -0.5f * sm.il)));
  u = mk_dfc(sdf_neg(sdf_mul(h, dim(df))), sdf_mul(h, dre(df)));
}
// memory element <-> working value
template <typename R2, typename G>
__device__ __forceinline__ R2 to_work(G g) {
  return g;
}
template <>
__device__ __forceinline__ dfc to_work<dfc, double2>(double2 g) {
  return mk_dfc(dsplit(g.x), dsplit(g.y));
}
// times a real scale (1 or 1/N^3), then to memory
template <typename R2, typename R, typename G>
__device__ __forceinline__ G from_work(R2 x, R scale) {
  x.x *= scale;
  x.y *= scale;
  return x;
}
template <>
__device__ __forceinline__ double2 from_work<dfc, double, double2>(dfc x, double scale) {
  if (scale != 1.0) {
    const float2 sc = dsplit(scale);
    x = mk_dfc(sdf_mul(dre(x), sc), sdf_mul(dim(x), sc));
  }
  return make_double2((double)x.rh + (double)x.rl, (double)x.ih + (double)x.il);
}
template <typename R2>
__device__ __forceinline__ R2 make_tw(double c, double s) {
  R2 w;
  w.x = (decltype(w.x))c;
  w.y = (decltype(w.y))s;
  return w;
}
template <>
__device__ __forceinline__ dfc make_tw<dfc>(double c, double s) {
  return mk_dfc(dsplit(c), dsplit(s));
}

// One Stockham stage of radix R (2, 3 or 4) on every line of the tile:
// butterfly j of a line reads src[j + i M] (M = N / R), applies the input
// twiddles w^(i tstep), does the R-point DFT and writes dst[expand(j) + q Ns].
template <int R, typename R2>
__device__ __forceinline__ void fft_stage_pow2(int N, int LS, int Ns, int sign, const R2 *src,
                                               R2 *dst, const R2 *tw) {
  const int M = N / R;
  for (int e = threadIdx.x; e < N * M; e += blockDim.x) {
    const int line = e / M, j = e - line * M;
    const R2 *sl = src + (size_t)line * LS;
    R2 *dl = dst + (size_t)line * LS;
    const int k = j % Ns;
    const int tstep = (N / (Ns * R)) * k;
    R2 v[R];
    v[0] = sl[j];
#pragma unroll
    for (int i = 1; i < R; ++i) v[i] = c_mul(sl[j + i * M], tw[(i * tstep) % N]);
    const int d0 = (j / Ns) * Ns * R + k;
    if (R == 2) {
      dl[d0] = c_add(v[0], v[1]);
      dl[d0 + Ns] = c_sub(v[0], v[1]);
    } else if (R == 3) {
      // w3 = exp(sign 2 pi i / 3) = (-1/2, h), h = tw[N / 3].y = sign sqrt(3)/2:
      // o0 = v0 + s, o1,2 = v0 - s/2 +- i h d  (s = v1 + v2, d = v1 - v2)
      const R2 sm = c_add(v[1], v[2]), df = c_sub(v[1], v[2]);
      R2 t, u;
      r3_parts(v[0], sm, df, tw[N / 3], t, u);
      dl[d0] = c_add(v[0], sm);
      dl[d0 + Ns] = c_add(t, u);
      dl[d0 + 2 * Ns] = c_sub(t, u);
    } else {
      // w4 = exp(sign 2 pi i / 4) = sign i; (v1 - v3) w4
      const R2 a = c_add(v[0], v[2]), b = c_sub(v[0], v[2]), c = c_add(v[1], v[3]);
      const R2 d = c_rot(c_sub(v[1], v[3]), sign);
      dl[d0] = c_add(a, c);
      dl[d0 + Ns] = c_add(b, d);
      dl[d0 + 2 * Ns] = c_sub(a, c);
      dl[d0 + 3 * Ns] = c_sub(b, d);
    }
  }
}

// One Stockham stage of any radix R, one output per thread: output q of
// butterfly j is sum_i src[j + i M] w^(i (tstep + q N / R)), i ascending.
template <typename R2, typename R>
__device__ __forceinline__ void fft_stage_direct(int N, int LS, int Rd, int Ns, const R2 *src,
                                                 R2 *dst, const R2 *tw) {
  const int M = N / Rd;
  for (int e = threadIdx.x; e < N * N; e += blockDim.x) {
    const int line = e / N, p = e - line * N;
    const R2 *sl = src + (size_t)line * LS;
    // p = (j / Ns) Ns R + q Ns + k with k = j mod Ns
    const int k = p % Ns, rest = p / Ns;
    const int q = rest % Rd, j = (rest / Rd) * Ns + k;
    const int step = (N / (Ns * Rd)) * k + q * M;
    R2 o;
    if constexpr (std::is_same<R2, dfc>::value) {
      o = dfc{0.f, 0.f, 0.f, 0.f};
      int m = 0;
      for (int i = 0; i < Rd; ++i) {
        o = c_add(o, c_mul(sl[j + i * M], tw[m]));
        m += step;
        if (m >= N) m %= N;
      }
    } else {
      R sr = 0, si = 0;
      int m = 0;
      for (int i = 0; i < Rd; ++i) {
        const R2 x = sl[j + i * M];
        const R2 w = tw[m];
        sr += x.x * w.x - x.y * w.y;
        si += x.x * w.y + x.y * w.x;
        m += step;
        if (m >= N) m %= N;
      }
      o.x = sr;
      o.y = si;
    }
    dst[(size_t)line * LS + p] = o;
  }
}
}  // namespace

// One pass: the tile's N lines along `axis` of cube blockIdx.y.
//   axis 2: tile = plane i (t); lines are rows (contiguous k), u = j.
//   axis 1: tile = plane i (t); lines are columns (fixed k), along j.
//   axis 0: tile = rows i of fixed j (t); lines are columns (fixed k), along i.
// Shared memory holds the tile twice (line stride N + 1, so that loading
// columns does not hit one bank) and the twiddle table.  in may alias out
// (passes 2 and 3 run in place): every global read happens before the first
// barrier and every write after the last.
template <typename R2, typename R, typename G>
__global__ void fft_pass_kernel(int N, int axis, int sign, R scale, FftPlan plan, const G *in,
                                G *out) {
  extern __shared__ unsigned char smem_raw[];
  const int LS = N + 1;
  R2 *buf0 = reinterpret_cast<R2 *>(smem_raw);  // [N][LS]
  R2 *buf1 = buf0 + (size_t)N * LS;              // [N][LS]
  R2 *tw = buf1 + (size_t)N * LS;                // [N]
  const long long NQ = (long long)N * N * N;
  const long long NN = (long long)N * N;
  const int cube = blockIdx.y;
  const int t = blockIdx.x;
  long long base, row_stride;
  if (axis == 0) {
    base = (long long)cube * NQ + (long long)t * N;
    row_stride = NN;
  } else {
    base = (long long)cube * NQ + (long long)t * NN;
    row_stride = N;
  }
  // tile element (u, v): u = row, v = column (contiguous in memory)
  for (int e = threadIdx.x; e < N * N; e += blockDim.x) {
    const int u = e / N, v = e - u * N;
    const R2 x = to_work<R2, G>(in[base + (long long)u * row_stride + v]);
    if (axis == 2)
      buf0[(size_t)u * LS + v] = x;
    else
      buf0[(size_t)v * LS + u] = x;
  }
  for (int r = threadIdx.x; r < N; r += blockDim.x) {
    const double ang = 8.0 * atan(1.0) * r / N;
    tw[r] = make_tw<R2>(cos(ang), sign * sin(ang));
  }
  __syncthreads();
  R2 *src = buf0, *dst = buf1;
  int Ns = 1;
  for (int s = 0; s < plan.nst; ++s) {
    const int Rd = plan.radix[s];
    if (Rd == 4)
      fft_stage_pow2<4>(N, LS, Ns, sign, src, dst, tw);
    else if (Rd == 2)
      fft_stage_pow2<2>(N, LS, Ns, sign, src, dst, tw);
    else if (Rd == 3)
      fft_stage_pow2<3>(N, LS, Ns, sign, src, dst, tw);
    else
      fft_stage_direct<R2, R>(N, LS, Rd, Ns, src, dst, tw);
    __syncthreads();
    R2 *x = src;
    src = dst;
    dst = x;
    Ns *= Rd;
  }
  for (int e = threadIdx.x; e < N * N; e += blockDim.x) {
    const int u = e / N, v = e - u * N;
    const R2 x = (axis == 2) ? src[(size_t)u * LS + v] : src[(size_t)v * LS + u];
    out[base + (long long)u * row_stride + v] = from_work<R2, R, G>(x, scale);
  }
}

template <typename R2, typename R, typename G>
static edb_status dft3d_t(int N, int batch, const G *in, G *out, int inverse, cudaStream_t st) {
  if (N < 1 || N > 64) return fail(EDB_EINVAL, "dft3d: N out of range [1,64]");
  const int sign = inverse ? +1 : -1;
  const int threads = N * N < FFT_THREADS ? ((N * N + 31) / 32) * 32 : FFT_THREADS;
  const size_t smem = sizeof(R2) * (2 * (size_t)N * (N + 1) + N);
  // once per instantiation, thread-safe (N = 64 in FP64 needs 131 KB)
  static const cudaError_t configured = cudaFuncSetAttribute(
      fft_pass_kernel<R2, R, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  if (configured != cudaSuccess) return cuda_fail(configured, "cudaFuncSetAttribute(fft_pass)");
  const FftPlan plan = fft_plan(N);
  dim3 grid((unsigned)N, (unsigned)batch);
  const R one = (R)1;
  const R scale = inverse ? (R)(1. / ((double)N * N * N)) : one;
  fft_pass_kernel<R2, R, G><<<grid, threads, smem, st>>>(N, 2, sign, one, plan, in, out);
  EDB_LAUNCHED();
  fft_pass_kernel<R2, R, G><<<grid, threads, smem, st>>>(N, 1, sign, one, plan, out, out);
  EDB_LAUNCHED();
  fft_pass_kernel<R2, R, G><<<grid, threads, smem, st>>>(N, 0, sign, scale, plan, out, out);
  EDB_LAUNCHED();
  return EDB_OK;
}

edb_status launch_dft3d(int N, int batch, const void *d_in, void *d_out, void *d_tmp, int inverse,
                        int fp32, cudaStream_t st) {
  (void)d_tmp;
  if (fp32 == EDB_DFT_DOUBLE_FLOAT)
    return dft3d_t<dfc, double, double2>(N, batch, (const double2 *)d_in, (double2 *)d_out,
                                         inverse, st);
  if (fp32)
    return dft3d_t<float2, float, float2>(N, batch, (const float2 *)d_in, (float2 *)d_out,
                                          inverse, st);
  return dft3d_t<double2, double, double2>(N, batch, (const double2 *)d_in, (double2 *)d_out,
                                           inverse, st);
}

}  // namespace edb
