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
#include "edb_internal.cuh"

namespace edb {

namespace {
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
      const auto h = tw[N / 3].y;
      R2 t, u;
      t.x = v[0].x - 0.5f * sm.x;
      t.y = v[0].y - 0.5f * sm.y;
      u.x = -h * df.y;
      u.y = h * df.x;
      dl[d0] = c_add(v[0], sm);
      dl[d0 + Ns] = c_add(t, u);
      dl[d0 + 2 * Ns] = c_sub(t, u);
    } else {
      // w4 = exp(sign 2 pi i / 4) = sign i; (v1 - v3) w4
      const R2 a = c_add(v[0], v[2]), b = c_sub(v[0], v[2]), c = c_add(v[1], v[3]);
      const R2 t = c_sub(v[1], v[3]);
      R2 d;
      d.x = -sign * t.y;
      d.y = sign * t.x;
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
    R2 o;
    o.x = sr;
    o.y = si;
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
template <typename R2, typename R>
__global__ void fft_pass_kernel(int N, int axis, int sign, R scale, FftPlan plan, const R2 *in,
                                R2 *out) {
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
    const R2 x = in[base + (long long)u * row_stride + v];
    if (axis == 2)
      buf0[(size_t)u * LS + v] = x;
    else
      buf0[(size_t)v * LS + u] = x;
  }
  for (int r = threadIdx.x; r < N; r += blockDim.x) {
    const double ang = 8.0 * atan(1.0) * r / N;
    R2 w;
    w.x = (R)cos(ang);
    w.y = (R)(sign * sin(ang));
    tw[r] = w;
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
    R2 x = (axis == 2) ? src[(size_t)u * LS + v] : src[(size_t)v * LS + u];
    x.x *= scale;
    x.y *= scale;
    out[base + (long long)u * row_stride + v] = x;
  }
}

template <typename R2, typename R>
static edb_status dft3d_t(int N, int batch, const R2 *in, R2 *out, int inverse, cudaStream_t st) {
  if (N < 1 || N > 64) return fail(EDB_EINVAL, "dft3d: N out of range [1,64]");
  const int sign = inverse ? +1 : -1;
  const int threads = N * N < FFT_THREADS ? ((N * N + 31) / 32) * 32 : FFT_THREADS;
  const size_t smem = sizeof(R2) * (2 * (size_t)N * (N + 1) + N);
  // once per instantiation, thread-safe (N = 64 in FP64 needs 131 KB)
  static const cudaError_t configured = cudaFuncSetAttribute(
      fft_pass_kernel<R2, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  if (configured != cudaSuccess) return cuda_fail(configured, "cudaFuncSetAttribute(fft_pass)");
  const FftPlan plan = fft_plan(N);
  dim3 grid((unsigned)N, (unsigned)batch);
  const R one = (R)1;
  const R scale = inverse ? (R)(1. / ((double)N * N * N)) : one;
  fft_pass_kernel<R2, R><<<grid, threads, smem, st>>>(N, 2, sign, one, plan, in, out);
  EDB_LAUNCHED();
  fft_pass_kernel<R2, R><<<grid, threads, smem, st>>>(N, 1, sign, one, plan, out, out);
  EDB_LAUNCHED();
  fft_pass_kernel<R2, R><<<grid, threads, smem, st>>>(N, 0, sign, scale, plan, out, out);
  EDB_LAUNCHED();
  return EDB_OK;
}

edb_status launch_dft3d(int N, int batch, const void *d_in, void *d_out, void *d_tmp, int inverse,
                        int fp32, cudaStream_t st) {
  (void)d_tmp;
  if (fp32)
    return dft3d_t<float2, float>(N, batch, (const float2 *)d_in, (float2 *)d_out, inverse, st);
  return dft3d_t<double2, double>(N, batch, (const double2 *)d_in, (double2 *)d_out, inverse, st);
}

}  // namespace edb
