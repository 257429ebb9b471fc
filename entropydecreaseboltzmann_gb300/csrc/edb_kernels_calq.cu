// Collision sum Q-hat (QCalculator::calQ, CalQ/QCalculator.h:231-257).
//
// FP64 drop-in path (one solve, the reference's B table streamed from HBM):
//   Q_c[kflat] = sum_l f_l f_m B[lflat * KC + kflat]
// with the per-dimension index maps of QParams (both index modes).  The grid
// is (k tiles) x (l chunks); every l chunk writes its partial sums and a
// second kernel adds the chunks in a fixed order (deterministic) and applies
// the output permutation of convertQ (:144-155).
//
// Batched FP32 path (many solves sharing one B table, ALIASED mode): a CTA
// owns a group of solves and a k-tile (one k1, a run of k2, all k3) and walks
// every l; see calq32_kernel below.
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
  long long want = (4LL * 152 + tiles - 1) / tiles;
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

// ---------------------------------------------------------------------------
// Batched FP32 kernel.
//
// Work: Q^s_K = sum_L B[L][K] f^s_L f^s_(K-L mod N) for S solves, all indices
// in FFTW order, B32 row-major [L][K].
//
// CTA = (group of SG = SC*WS solves) x (k1, a tile of K2T k2 values, all k3).
// Thread = (k2, run of A consecutive k3, SC solves).  The WS threads that
// share a (k2, k3-run) are adjacent lanes, so their B loads coalesce into one
// transaction.  For each L the thread needs
//   B[L][k1,k2,k3..k3+A)   A floats, shared by its SC solves,
//   f^s_L                  one complex per solve (same for the whole CTA),
//   f^s_(K-L)              A complex per solve; along l3 these form a sliding
//                          window over m3 = k3 + a - l3, so one new value per
//                          l3 step is loaded into a ring of A registers.
// The m1-plane f^s[m1][:][:] (m1 = k1 - l1) of the CTA's solves is staged in
// shared memory while l1 is fixed.  Sums: plain FP32 FMA along one l3 line
// (N terms), then a two-sum fold into (hi, lo) per accumulator — blocked
// compensated summation (fast inner sum, error-free outer sum).
// ---------------------------------------------------------------------------
namespace {
constexpr int A = 8;   // k3 outputs per thread
constexpr int SC = 2;  // solves per thread
constexpr int WS = 8;  // solve subgroups per CTA
constexpr int SG = SC * WS;
constexpr int MAX_THREADS = 384;

__device__ __forceinline__ void two_sum_fold(float &hi, float &lo, float x) {
  float s = hi + x;
  float bb = s - hi;
  float e = (hi - (s - bb)) + (x - bb);
  hi = s;
  lo += e;
}
}  // namespace

__global__ void __launch_bounds__(MAX_THREADS, 1)
    calq32_kernel(int N, int S, int K2T, const float *__restrict__ B32,
                  const float2 *__restrict__ fin, float2 *__restrict__ Q) {
  extern __shared__ float4 smem_f4[];
  float2 *fplane = reinterpret_cast<float2 *>(smem_f4);  // [m2][m3][SG]
  const long long NQ = (long long)N * N * N;
  const int NN = N * N;
  const int R = (N + A - 1) / A;
  const int tid = threadIdx.x;
  const int w = tid % WS;
  const int rest = tid / WS;
  const int r = rest % R;
  const int k2l = rest / R;
  const int k1 = blockIdx.y;
  const int k2 = blockIdx.z * K2T + k2l;
  const bool k_ok = (k2l < K2T) && (k2 < N);
  const int k2c = k2 < N ? k2 : N - 1;
  const int k3_0 = r * A;
  const int s0 = blockIdx.x * SG;
  const int sA = s0 + w * SC;  // first solve of this thread

  float2 hi[A][SC], lo[A][SC];
#pragma unroll
  for (int a = 0; a < A; ++a)
#pragma unroll
    for (int c = 0; c < SC; ++c) {
      hi[a][c] = make_float2(0.f, 0.f);
      lo[a][c] = make_float2(0.f, 0.f);
    }

  const bool vec = (N % 4) == 0;
  const int NL3 = R * A;

  for (int l1 = 0; l1 < N; ++l1) {
    const int m1 = (k1 - l1 + N) % N;
    __syncthreads();
    for (int idx = tid; idx < NN * SG; idx += blockDim.x) {
      int sl = idx / NN, pos = idx % NN;
      int s = s0 + sl;
      float2 v = make_float2(0.f, 0.f);
      if (s < S) v = __ldg(&fin[(long long)s * NQ + (long long)m1 * NN + pos]);
      fplane[(long long)pos * SG + sl] = v;
    }
    __syncthreads();
    for (int l2 = 0; l2 < N; ++l2) {
      const int m2 = (k2c - l2 + N) % N;
      const float2 *fp = fplane + (long long)m2 * N * SG + w * SC;
      const float *Brow = B32 + (long long)((l1 * N + l2) * N) * NQ + (long long)k1 * NN +
                          (long long)k2c * N + k3_0;
      const float2 *fL[SC];
#pragma unroll
      for (int c = 0; c < SC; ++c) {
        int s = sA + c < S ? sA + c : S - 1;
        fL[c] = fin + (long long)s * NQ + (long long)(l1 * N + l2) * N;
      }
      float2 acc[A][SC];
#pragma unroll
      for (int a = 0; a < A; ++a)
#pragma unroll
        for (int c = 0; c < SC; ++c) acc[a][c] = make_float2(0.f, 0.f);
      float2 ring[A][SC];
#pragma unroll
      for (int a = 0; a < A; ++a) {
        int idx = (k3_0 + a) % N;
#pragma unroll
        for (int c = 0; c < SC; ++c) ring[a][c] = fp[idx * SG + c];
      }
      for (int g = 0; g < NL3; g += A) {
        int base = (k3_0 - g) % N;
        if (base < 0) base += N;
#pragma unroll
        for (int t = 0; t < A; ++t) {
          const int l3 = g + t;
          if (l3 > 0) {
            int idx = base - t;
            while (idx < 0) idx += N;
            const int slot = (A - t) % A;
#pragma unroll
            for (int c = 0; c < SC; ++c) ring[slot][c] = fp[idx * SG + c];
          }
          const bool valid = l3 < N;
          float bv[A];
          const float *bp = Brow + (long long)(valid ? l3 : 0) * NQ;
          if (vec) {
            float4 b0 = __ldg(reinterpret_cast<const float4 *>(bp));
            float4 b1 = __ldg(reinterpret_cast<const float4 *>(bp) + 1);
            bv[0] = b0.x; bv[1] = b0.y; bv[2] = b0.z; bv[3] = b0.w;
            bv[4] = b1.x; bv[5] = b1.y; bv[6] = b1.z; bv[7] = b1.w;
          } else {
#pragma unroll
            for (int a = 0; a < A; ++a) bv[a] = __ldg(bp + a);
          }
          float2 fl[SC];
#pragma unroll
          for (int c = 0; c < SC; ++c)
            fl[c] = valid ? __ldg(fL[c] + l3) : make_float2(0.f, 0.f);
#pragma unroll
          for (int a = 0; a < A; ++a) {
            const int slot = (a - t + A) % A;
#pragma unroll
            for (int c = 0; c < SC; ++c) {
              const float2 fm = ring[slot][c];
              const float pr = fl[c].x * fm.x - fl[c].y * fm.y;
              const float pi = fl[c].x * fm.y + fl[c].y * fm.x;
              acc[a][c].x = fmaf(bv[a], pr, acc[a][c].x);
              acc[a][c].y = fmaf(bv[a], pi, acc[a][c].y);
            }
          }
        }
      }
#pragma unroll
      for (int a = 0; a < A; ++a)
#pragma unroll
        for (int c = 0; c < SC; ++c) {
          two_sum_fold(hi[a][c].x, lo[a][c].x, acc[a][c].x);
          two_sum_fold(hi[a][c].y, lo[a][c].y, acc[a][c].y);
        }
    }
  }
  if (!k_ok) return;
#pragma unroll
  for (int c = 0; c < SC; ++c) {
    const int s = sA + c;
    if (s >= S) continue;
    float2 *qp = Q + (long long)s * NQ + (long long)k1 * NN + (long long)k2 * N;
#pragma unroll
    for (int a = 0; a < A; ++a) {
      const int k3 = k3_0 + a;
      if (k3 < N) qp[k3] = make_float2(hi[a][c].x + lo[a][c].x, hi[a][c].y + lo[a][c].y);
    }
  }
}

edb_status launch_calq32_batch(int N, int S, const float *d_B32, const float2 *d_fin, float2 *d_Q,
                               cudaStream_t st) {
  const int R = (N + A - 1) / A;
  int K2T = MAX_THREADS / (R * WS);
  if (K2T > N) K2T = N;
  if (K2T < 1) return fail(EDB_EINVAL, "calq32: N too large for the thread tile");
  // balance the k2 tiles
  int tiles = (N + K2T - 1) / K2T;
  K2T = (N + tiles - 1) / tiles;
  const int threads = K2T * R * WS;
  size_t smem = (size_t)N * N * SG * sizeof(float2);
  static int configured = 0;
  if (!configured) {
    EDB_CUDA(cudaFuncSetAttribute(calq32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  227 * 1024));
    configured = 1;
  }
  if (smem > 227 * 1024) return fail(EDB_EINVAL, "calq32: N too large for shared memory");
  dim3 grid((unsigned)((S + SG - 1) / SG), (unsigned)N, (unsigned)tiles);
  calq32_kernel<<<grid, threads, smem, st>>>(N, S, K2T, d_B32, d_fin, d_Q);
  EDB_LAUNCHED();
  return EDB_OK;
}

}  // namespace edb
