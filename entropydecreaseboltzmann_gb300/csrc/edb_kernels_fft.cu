// Batched cubic 3-D DFT with the conventions of the reference's fft3d
// (CalQ/fft3d.h:25-48): forward = FFTW_FORWARD (exp(-2 pi i jk/N)),
// unnormalised; inverse = FFTW_BACKWARD then every element times 1./N^3.
//
// N is small (<= 64) and the transform is O(N^4) per cube against the
// O(N^6) collision sum, so each axis is a direct DFT: a pass loads an N x N
// tile (N rows of N contiguous elements) into shared memory, transforms it
// along one tile axis with a twiddle table exp(sign 2 pi i r/N), r = jk mod N,
// summing j in increasing order, and writes it back in place.  Three passes
// (axis 2, 1, 0) make the 3-D transform.
#include "edb_internal.cuh"

namespace edb {

template <typename R2, typename R>
__global__ void dft_pass_kernel(int N, int axis, int sign, R scale, const R2 *in, R2 *out) {
  // in may alias out (passes 2 and 3 run in place): every read of the tile
  // happens before the barrier, every write after it.
  extern __shared__ unsigned char smem_raw[];
  R2 *tile = reinterpret_cast<R2 *>(smem_raw);  // [N][N]
  R2 *tw = tile + N * N;                         // [N]
  const long long NQ = (long long)N * N * N;
  const long long NN = (long long)N * N;
  const int cube = blockIdx.y;
  const int t = blockIdx.x;  // tile index within the cube
  // tile element (u, v), u = row, v = column (contiguous in memory)
  // axis 2: tile = plane i (t); transform along v (k), rows u = j.
  // axis 1: tile = plane i (t); transform along u (j), columns v = k.
  // axis 0: tile = rows i (u) of fixed j (t), columns k (v); transform along u.
  long long base;
  long long row_stride;
  if (axis == 0) {
    base = (long long)cube * NQ + (long long)t * N;
    row_stride = NN;
  } else {
    base = (long long)cube * NQ + (long long)t * NN;
    row_stride = N;
  }
  for (int e = threadIdx.x; e < N * N; e += blockDim.x) {
    int u = e / N, v = e % N;
    tile[e] = in[base + (long long)u * row_stride + v];
  }
  for (int r = threadIdx.x; r < N; r += blockDim.x) {
    double ang = 8.0 * atan(1.0) * r / N;
    R2 w;
    w.x = (R)cos(ang);
    w.y = (R)(sign * sin(ang));
    tw[r] = w;
  }
  __syncthreads();
  R2 res[4];
  int cnt = 0;
  for (int e = threadIdx.x; e < N * N; e += blockDim.x, ++cnt) {
    int u = e / N, v = e % N;
    R sr = 0, si = 0;
    if (axis == 2) {
      for (int j = 0; j < N; ++j) {
        R2 x = tile[u * N + j];
        R2 w = tw[(j * v) % N];
        sr += x.x * w.x - x.y * w.y;
        si += x.x * w.y + x.y * w.x;
      }
    } else {
      for (int j = 0; j < N; ++j) {
        R2 x = tile[j * N + v];
        R2 w = tw[(j * u) % N];
        sr += x.x * w.x - x.y * w.y;
        si += x.x * w.y + x.y * w.x;
      }
    }
    res[cnt].x = sr * scale;
    res[cnt].y = si * scale;
  }
  __syncthreads();
  cnt = 0;
  for (int e = threadIdx.x; e < N * N; e += blockDim.x, ++cnt) {
    int u = e / N, v = e % N;
    out[base + (long long)u * row_stride + v] = res[cnt];
  }
}

template <typename R2, typename R>
static edb_status dft3d_t(int N, int batch, const R2 *in, R2 *out, int inverse, cudaStream_t st) {
  if (N < 1 || N > 64) return fail(EDB_EINVAL, "dft3d: N out of range [1,64]");
  const int sign = inverse ? +1 : -1;
  int threads = N * N < 1024 ? ((N * N + 31) / 32) * 32 : 1024;
  // each thread keeps up to 4 results: N*N <= 4 * threads
  if (N * N > 4 * threads) return fail(EDB_EINVAL, "dft3d: tile too large");
  size_t smem = sizeof(R2) * ((size_t)N * N + N);
  dim3 grid((unsigned)N, (unsigned)batch);
  const R one = (R)1;
  const R scale = inverse ? (R)(1. / ((double)N * N * N)) : one;
  dft_pass_kernel<R2, R><<<grid, threads, smem, st>>>(N, 2, sign, one, in, out);
  EDB_LAUNCHED();
  dft_pass_kernel<R2, R><<<grid, threads, smem, st>>>(N, 1, sign, one, out, out);
  EDB_LAUNCHED();
  dft_pass_kernel<R2, R><<<grid, threads, smem, st>>>(N, 0, sign, scale, out, out);
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
