// Kernel-table construction (genB) on the device, FP64.
//
// Restates QCalculator::genB (CalQ/QCalculator.h:158-229) for the GPU:
//   beta(l,k) = F(|l+m| lp, |l-m| lp) sigma(l) sigma(m) rval - Bmm[m],
//   Bmm[m]    = F(2|m| lp, 0) sigma(m)^2 rval,   m = k - l wrapped,
// with lp = lambda*pi = 2 pi/(3+sqrt 2) (:163) and rval = 4 pi (2 lambda/pi *
// L/N)^(3+gamma) (:176).  F depends on l, m only through the integer squared
// norms a = |l+m|^2 and b = |l-m|^2 (calXi takes sqrt of an int, :165-167),
// so it is tabulated once over (a, b) — a and b are always congruent mod 4
// (a - b = 4 l.m), so only those entries are filled — and the N^6 table is a
// gather from that small table.  This translation unit is compiled with
// -fmad=false: products and sums are rounded in the reference's order.
#include <math.h>

#include "edb_internal.cuh"

namespace edb {

// F_0 / F_1 closed forms, QCalculator.h:76-106 (ReadMe.md:55-68).
__device__ double funF_closed(int alpha, double xi, double eta) {
  double p = xi + eta, q = xi - eta;
  double res = 0.0;
  if (alpha == 0) {
    if (eta < 1.0e-10) {
      if (xi < 1.0e-10)
        res = 1. / 3.;
      else
        res = (-xi * cos(xi) + sin(xi)) / (xi * xi * xi);
    } else {
      if (xi < 1.0e-10)
        res = (-eta * cos(eta) + sin(eta)) / (eta * eta * eta);
      else if (fabs(xi - eta) < 1.0e-10)
        res = (xi - cos(xi) * sin(xi)) / (2. * xi * xi * xi);
      else
        res = (p * sin(q) - q * sin(p)) / (2. * xi * eta * p * q);
    }
  } else if (alpha == 1) {
    if (eta < 1.0e-10) {
      if (xi < 1.0e-10)
        res = 1. / 4.;
      else
        res = (-2. - (-2. + xi * xi) * cos(xi) + 2. * xi * sin(xi)) / (xi * xi * xi * xi);
    } else {
      if (xi < 1.0e-10)
        res = (-2. - (-2. + eta * eta) * cos(eta) + 2. * eta * sin(eta)) /
              (eta * eta * eta * eta);
      else if (fabs(xi - eta) < 1.0e-10)
        res = -(-1. - 2. * xi * xi + cos(2. * xi) + 2. * xi * sin(2. * xi)) /
              (8. * xi * xi * xi * xi);
      else
        res = (q * sin(q) + cos(q)) / (2. * xi * eta * q * q) -
              (p * sin(p) + cos(p)) / (2. * xi * eta * p * p) - 2. / (p * p * q * q);
    }
  }
  return res;
}

__global__ void ftable_closed_kernel(int amax, int alpha, double lp, double *__restrict__ T) {
  long long W = amax + 1;
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= W * W) return;
  int a = (int)(idx / W), b = (int)(idx % W);
  if ((a - b) & 3) {
    T[idx] = 0.0;
    return;
  }
  double xi = sqrt((double)a) * lp;
  double eta = sqrt((double)b) * lp;
  T[idx] = funF_closed(alpha, xi, eta);
}

// General gamma: F(xi, eta) = int_0^1 r^(2+gamma) sinc(xi r) sinc(eta r) dr,
// with r = u^2 and composite Gauss-Legendre nodes u_j, weights W_j (which
// include 2 u_j^(5+2 gamma)).  S[a][j] = sinc(sqrt(a) lp u_j^2).
__global__ void sinc_table_kernel(int amax, int nodes, double lp, const double *__restrict__ u,
                                  double *__restrict__ S) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)(amax + 1) * nodes) return;
  int a = (int)(idx / nodes), j = (int)(idx % nodes);
  double x = sqrt((double)a) * lp * (u[j] * u[j]);
  S[idx] = (x == 0.0) ? 1.0 : sin(x) / x;
}

__global__ void ftable_quad_kernel(int amax, int nodes, const double *__restrict__ S,
                                   const double *__restrict__ W, double *__restrict__ T) {
  long long Wd = amax + 1;
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= Wd * Wd) return;
  int a = (int)(idx / Wd), b = (int)(idx % Wd);
  if ((a - b) & 3) {
    T[idx] = 0.0;
    return;
  }
  const double *sa = S + (long long)a * nodes;
  const double *sb = S + (long long)b * nodes;
  double sum = 0.0;
  for (int j = 0; j < nodes; ++j) sum += W[j] * sa[j] * sb[j];
  T[idx] = sum;
}

// Gauss-Legendre nodes on [-1,1] by Newton iteration on the three-term
// recurrence (host; setup constants of the quadrature rule).
static void gauss_legendre(int G, double *x, double *w) {
  for (int i = 0; i < G; ++i) {
    double z = cos(M_PI * (i + 0.75) / (G + 0.5));
    double dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= G; ++k) {
        double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = pk;
      }
      dp = G * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) break;
    }
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= G; ++k) {
      double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = pk;
    }
    dp = G * (z * p1 - p0) / (z * z - 1.0);
    x[i] = z;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

static double lambda_pi() { return 2. / (3. + sqrt(2.)) * M_PI; }

// rval of QCalculator::genB (QCalculator.h:176) with the box half-width L.
double genb_rval(int N, double gamma, double L) {
  return (4. * M_PI) * pow(2. * lambda_pi() / M_PI * L / N, 3 + gamma);
}

edb_status launch_ftable(int N, double gamma, double *d_T, int amax, cudaStream_t st) {
  (void)N;
  const double lp = lambda_pi();
  long long total = (long long)(amax + 1) * (amax + 1);
  int threads = 256;
  long long blocks = (total + threads - 1) / threads;
  if (gamma == 0.0 || gamma == 1.0) {
    ftable_closed_kernel<<<(unsigned)blocks, threads, 0, st>>>(amax, (int)gamma, lp, d_T);
    EDB_LAUNCHED();
    return EDB_OK;
  }
  // composite Gauss-Legendre in u = sqrt(r): 32 panels x 16 nodes
  const int G = 16, P = 32, nodes = G * P;
  double gx[16], gw[16];
  gauss_legendre(G, gx, gw);
  double hu[512], hw[512];
  const double h = 1.0 / P;
  for (int p = 0; p < P; ++p)
    for (int i = 0; i < G; ++i) {
      double u = p * h + 0.5 * h * (gx[i] + 1.0);
      hu[p * G + i] = u;
      hw[p * G + i] = 0.5 * h * gw[i] * 2.0 * pow(u, 5.0 + 2.0 * gamma);
    }
  double *d_u = nullptr, *d_S = nullptr;
  EDB_CUDA(cudaMallocAsync(&d_u, sizeof(double) * 2 * nodes, st));
  EDB_CUDA(cudaMallocAsync(&d_S, sizeof(double) * (amax + 1) * nodes, st));
  EDB_CUDA(cudaMemcpyAsync(d_u, hu, sizeof(double) * nodes, cudaMemcpyHostToDevice, st));
  EDB_CUDA(cudaMemcpyAsync(d_u + nodes, hw, sizeof(double) * nodes, cudaMemcpyHostToDevice, st));
  long long ns = (long long)(amax + 1) * nodes;
  sinc_table_kernel<<<(unsigned)((ns + 255) / 256), 256, 0, st>>>(amax, nodes, lp, d_u, d_S);
  EDB_LAUNCHED();
  ftable_quad_kernel<<<(unsigned)blocks, threads, 0, st>>>(amax, nodes, d_S, d_u + nodes, d_T);
  EDB_LAUNCHED();
  // the host arrays above must outlive the async copies
  EDB_CUDA(cudaStreamSynchronize(st));
  EDB_CUDA(cudaFreeAsync(d_S, st));
  EDB_CUDA(cudaFreeAsync(d_u, st));
  return EDB_OK;
}

// sigma(beta) of QCalculator::filtering (:67-74) for centred indices c - n.
__global__ void sigma_kernel(int N, double PI, double *__restrict__ sigma) {
  int c = threadIdx.x;
  if (c >= N) return;
  int n = (N - 1) / 2;
  double tmp = (double)(n + 1);
  double b = fabs((double)(c - n));
  sigma[c] = ((tmp - b) * cos(PI * b / tmp) + sin(PI * b / tmp) / tan(PI / tmp)) / tmp;
}

// Bmm (QCalculator.h:181-192).  REFERENCE: (2n+1)^3 entries filled in the
// (2n+1)-extent loop order, the rest zero (the vector is N^3 long, :179).
// ALIASED: all N^3 centred modes.  fil = sigma(k1) sigma(k2) sigma(k3).
__global__ void bmm_kernel(int N, int mode, int filter, double rval, const double *__restrict__ T,
                           int amax, const double *__restrict__ sigma, double *__restrict__ Bmm) {
  long long NQ = (long long)N * N * N;
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= NQ) return;
  int n = (N - 1) / 2;
  int P = (mode == EDB_INDEX_REFERENCE) ? 2 * n + 1 : N;
  long long PQ = (long long)P * P * P;
  if (q >= PQ) {
    Bmm[q] = 0.0;
    return;
  }
  int c1 = (int)(q / ((long long)P * P)), c2 = (int)((q / P) % P), c3 = (int)(q % P);
  int k1 = c1 - n, k2 = c2 - n, k3 = c3 - n;
  int a = (2 * k1) * (2 * k1) + (2 * k2) * (2 * k2) + (2 * k3) * (2 * k3);
  double fil = filter ? sigma[c1] * sigma[c2] * sigma[c3] : 1.0;
  Bmm[q] = T[(long long)a * (amax + 1)] * fil * fil * rval;
}

edb_status launch_bmm(int N, double gamma, double L, int filter, int mode, const double *d_T,
                      int amax, double *d_sigma, double *d_Bmm, cudaStream_t st) {
  const double PI = 4. * atan(1.);
  sigma_kernel<<<1, 64, 0, st>>>(N, PI, d_sigma);
  EDB_LAUNCHED();
  const double lam = lambda_pi();
  const double rval = (4. * M_PI) * pow(2. * lam / M_PI * L / N, 3 + gamma);
  long long NQ = (long long)N * N * N;
  bmm_kernel<<<(unsigned)((NQ + 255) / 256), 256, 0, st>>>(N, mode, filter, rval, d_T, amax,
                                                          d_sigma, d_Bmm);
  EDB_LAUNCHED();
  return EDB_OK;
}

// One CTA per row l (centred); columns k over all N^3 centred modes.
// Writes B64[l][k] (when given) and, when B32 is given, the symmetric pair
// table of the batched kernel in FFTW order (lf = (l - n) mod N per
// dimension), for the visited planes only (c32_plane_pos): the terms l and
// m = k - l of a Q-hat sum carry the same product f_l f_m, so the batched
// kernel visits only the l1 planes with l1 <= m1 and weights them by
// B[l][k] + B[m][k], computed here in
// FP64 and rounded once; on the planes l1 = m1 (both terms inside the plane)
// the entry stays B[l][k].  The partner's value needs no second table lookup:
// l + m and |l - m| are the same for both, so B[m][k] differs from B[l][k]
// only in its self-interaction term, Bmm[l] instead of Bmm[m].
__global__ void genB_kernel(int N, int filter, double rval, const double *__restrict__ T, int amax,
                            const double *__restrict__ sigma, const double *__restrict__ Bmm,
                            double *__restrict__ B64, float *__restrict__ B32) {
  const int n = (N - 1) / 2;
  const long long NQ = (long long)N * N * N;
  const long long lc = blockIdx.x;
  const int l1 = (int)(lc / (N * N)), l2 = (int)((lc / N) % N), l3 = (int)(lc % N);
  const double sigmal = filter ? sigma[l1] * sigma[l2] * sigma[l3] : 1.0;
  const long long W = amax + 1;
  const long long lf = ((long long)((l1 - n + N) % N) * N + (l2 - n + N) % N) * N + (l3 - n + N) % N;
  for (long long kc = threadIdx.x; kc < NQ; kc += blockDim.x) {
    int k1 = (int)(kc / (N * N)), k2 = (int)((kc / N) % N), k3 = (int)(kc % N);
    int m1 = k1 - l1 + n;
    if (m1 < 0) m1 += N;
    else if (m1 > N - 1) m1 -= N;
    int m2 = k2 - l2 + n;
    if (m2 < 0) m2 += N;
    else if (m2 > N - 1) m2 -= N;
    int m3 = k3 - l3 + n;
    if (m3 < 0) m3 += N;
    else if (m3 > N - 1) m3 -= N;
    int x1 = l1 - n + m1 - n, x2 = l2 - n + m2 - n, x3 = l3 - n + m3 - n;
    int e1 = l1 - m1, e2 = l2 - m2, e3 = l3 - m3;
    int a = x1 * x1 + x2 * x2 + x3 * x3;
    int b = e1 * e1 + e2 * e2 + e3 * e3;
    double sigmam = filter ? sigma[m1] * sigma[m2] * sigma[m3] : 1.0;
    long long m = ((long long)m1 * N + m2) * N + m3;
    const double t = T[(long long)a * W + b];
    double v = t * sigmal * sigmam * rval - Bmm[m];
    if (B64) B64[lc * NQ + kc] = v;
    const int k1f = (k1 - n + N) % N;
    const int pos = B32 ? c32_plane_pos(N, k1f, (int)(lf / (N * N))) : -1;
    if (pos >= 0) {
      // [k1][p][l2][l3][k2][k3] (FFTW order; p = position of l1 in k1's
      // visited list): the batched kernel's tile for one line and k1 lies
      // within N^3 floats, and planes it never visits are not stored
      const long long k23 = (long long)((k2 - n + N) % N) * N + (k3 - n + N) % N;
      const long long l2f = (lf / N) % N, l3f = lf % N;
      double w = v;
      if (l1 != m1) w += t * sigmam * sigmal * rval - Bmm[lc];  // B[m][k], as its row writes it
      B32[((((long long)k1f * c32_maxlist(N) + pos) * N + l2f) * N + l3f) * (N * N) + k23] =
          (float)w;
    }
  }
}

edb_status launch_genB(int N, double gamma, double L, int filter, int mode, const double *d_T,
                       int amax, const double *d_sigma, const double *d_Bmm, double *d_B64,
                       float *d_B32, cudaStream_t st) {
  (void)mode;
  const double lam = lambda_pi();
  const double rval = (4. * M_PI) * pow(2. * lam / M_PI * L / N, 3 + gamma);
  long long NQ = (long long)N * N * N;
  genB_kernel<<<(unsigned)NQ, 256, 0, st>>>(N, filter, rval, d_T, amax, d_sigma, d_Bmm, d_B64,
                                            d_B32);
  EDB_LAUNCHED();
  return EDB_OK;
}

// ---- pointwise evaluation (QCalculator::funF, ::filtering as public methods)
__global__ void funF_points_kernel(int alpha, long long n, const double *__restrict__ xi,
                                   const double *__restrict__ eta, double *__restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = funF_closed(alpha, xi[i], eta[i]);
}

__global__ void filtering_points_kernel(int N, double PI, long long n, const int *__restrict__ beta,
                                        double *__restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int nn = (N - 1) / 2;
  const double tmp = (double)(nn + 1);
  const double b = fabs((double)beta[i]);
  out[i] = ((tmp - b) * cos(PI * b / tmp) + sin(PI * b / tmp) / tan(PI / tmp)) / tmp;
}

edb_status launch_funF_points(int alpha, long long n, const double *d_xi, const double *d_eta,
                              double *d_out, cudaStream_t st) {
  funF_points_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(alpha, n, d_xi, d_eta, d_out);
  EDB_LAUNCHED();
  return EDB_OK;
}

edb_status launch_filtering_points(int N, long long n, const int *d_beta, double *d_out,
                                   cudaStream_t st) {
  const double PI = 4. * atan(1.);
  filtering_points_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(N, PI, n, d_beta, d_out);
  EDB_LAUNCHED();
  return EDB_OK;
}

}  // namespace edb
