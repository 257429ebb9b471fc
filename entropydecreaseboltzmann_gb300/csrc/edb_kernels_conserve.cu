// Moment conservation and the moment-preserving entropy fix (FP64).
//
// Conservation.  The Fourier-spectral collision operator keeps mass, momentum
// and energy only to spectral accuracy.  In conservative mode a solve is
// projected after every step back onto its initial moments with the
// minimum-norm Lagrange-multiplier correction of Gamba & Tharkabhushanam
// (J. Comput. Phys. 228, 2009).  With C the 5 x N^3 matrix of the grid moment
// functionals h^3 {1, v1, v2, v3, |v|^2} and G = C C^T:
//     F <- F - C^T G^-1 (C F - m0).
// Given C F_n = m0 this equals F_n + P(F_{n+1} - F_n) with P the orthogonal
// projector onto null(C), i.e. every Q-hat stage of the step's final
// combination projected.  The functionals and the correction are separable,
// so in Fourier space both touch only the three axis lines (k,0,0), (0,k,0),
// (0,0,k) of F-hat:
//     sum_j v_j1 F_j = sum_k Fhat(k,0,0) W1(k),  W1(k) = (1/N) sum_j v_j e^{+2 pi i jk/N}
//     DFT(v_j1)(k)   = N^3 conj(W1(k1)) on the first axis line, 0 elsewhere
// (W2 the same with v_j^2).  One warp per solve; O(N) work.
//
// Entropy fix.  The reference's FixSol (EntropyFix.h:211-253) blends f toward
// its mean, which keeps mass only.  The moment-preserving fix blends f toward
// the discrete Maxwellian M = exp(a + b.v + c|v|^2) whose grid moments equal
// f's.  (a, b, c) are the Lagrange multipliers of the discrete entropy
// minimisation under those five constraints, found by damped Newton on the
// convex dual  Phi(theta) = h^3 sum_j exp(theta.phi_j) - theta.m.  Every blend
// (1 - beta) f + beta M keeps the five moments, and the same bisection on beta
// as the reference's FixSol brings the entropy under the integrator's target.
#include <math.h>

#include "edb_internal.cuh"

namespace edb {

namespace {
constexpr int CT = 512;          // threads of a per-solve fix CTA
constexpr int CW = CT / 32;      // its warps
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

// Block sum of K values in a fixed order; results valid in every thread.
// red holds (CW + 1) * K doubles.
template <int K>
__device__ void block_sum_k(double (&v)[K], double *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < K; ++q) v[q] = warp_sum(v[q]);
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < K; ++q) red[warp * K + q] = v[q];
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double s = 0.0;
    for (int w = 0; w < CW; ++w) s += red[w * K + threadIdx.x];
    red[CW * K + threadIdx.x] = s;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < K; ++q) v[q] = red[CW * K + q];
  __syncthreads();
}

// flogf (BKW.h:153-161), the integrator's entropy density.
__device__ __forceinline__ double flogf_c(double f) {
  if (fabs(f) < 1.0e-6) return 0.;
  return f * log(f) - f;
}

// 5x5 solve A x = b by Gaussian elimination with partial pivoting (one thread).
__device__ bool solve5(double A[5][5], double b[5], double x[5]) {
  for (int c = 0; c < 5; ++c) {
    int p = c;
    for (int r = c + 1; r < 5; ++r)
      if (fabs(A[r][c]) > fabs(A[p][c])) p = r;
    if (!(fabs(A[p][c]) > 0.0)) return false;
    if (p != c) {
      for (int k = 0; k < 5; ++k) {
        double t = A[c][k];
        A[c][k] = A[p][k];
        A[p][k] = t;
      }
      double t = b[c];
      b[c] = b[p];
      b[p] = t;
    }
    for (int r = c + 1; r < 5; ++r) {
      const double f = A[r][c] / A[c][c];
      for (int k = c; k < 5; ++k) A[r][k] -= f * A[c][k];
      b[r] -= f * b[c];
    }
  }
  for (int r = 4; r >= 0; --r) {
    double s = b[r];
    for (int k = r + 1; k < 5; ++k) s -= A[r][k] * x[k];
    x[r] = s / A[r][r];
  }
  return true;
}

// Grid moments h^3 sum F_j {1, v1, v2, v3, |v|^2} from the axis lines of F-hat
// (one warp; result in every lane).
__device__ void hat_moments_warp(int N, const double *tab, const double2 *Fh, double m[5]) {
  const int lane = threadIdx.x & 31;
  const long long NN = (long long)N * N;
  double s1 = 0, s2 = 0, s3 = 0, s4 = 0;
  for (int k = lane; k < N; k += 32) {
    const double w1r = tab[2 * k], w1i = tab[2 * k + 1];
    const double w2r = tab[2 * N + 2 * k], w2i = tab[2 * N + 2 * k + 1];
    const double2 a = Fh[k * NN], b = Fh[(long long)k * N], c = Fh[k];
    s1 += a.x * w1r - a.y * w1i;
    s2 += b.x * w1r - b.y * w1i;
    s3 += c.x * w1r - c.y * w1i;
    s4 += (a.x + b.x + c.x) * w2r - (a.y + b.y + c.y) * w2i;
  }
  const double h3 = tab[4 * N + 25];
  m[0] = h3 * Fh[0].x;
  m[1] = h3 * warp_sum(s1);
  m[2] = h3 * warp_sum(s2);
  m[3] = h3 * warp_sum(s3);
  m[4] = h3 * warp_sum(s4);
}
}  // namespace

__global__ void hat_moments_kernel(int N, int S, const double *__restrict__ tab,
                                   const double2 *__restrict__ Fhat, double *__restrict__ out) {
  const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (s >= S) return;
  double m[5];
  hat_moments_warp(N, tab, Fhat + (long long)s * N * N * N, m);
  if ((threadIdx.x & 31) == 0)
    for (int q = 0; q < 5; ++q) out[(long long)s * 5 + q] = m[q];
}

__global__ void project_moments_kernel(int N, int S, const double *__restrict__ tab,
                                       double2 *__restrict__ Fhat, const double *__restrict__ m0) {
  const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (s >= S) return;
  const int lane = threadIdx.x & 31;
  const long long NN = (long long)N * N;
  double2 *Fh = Fhat + (long long)s * NN * N;
  double m[5];
  hat_moments_warp(N, tab, Fh, m);  // every lane has read its axis values
  double d[5], mu[5];
  for (int q = 0; q < 5; ++q) d[q] = m[q] - m0[(long long)s * 5 + q];
  const double *Gi = tab + 4 * N;
  for (int r = 0; r < 5; ++r) {
    double acc = 0.0;
    for (int q = 0; q < 5; ++q) acc += Gi[r * 5 + q] * d[q];
    mu[r] = acc;
  }
  const double c = -tab[4 * N + 25] * (double)N * (double)NN;  // -h^3 N^3
  for (int k = lane; k < N; k += 32) {
    const double w1r = tab[2 * k], w1i = -tab[2 * k + 1];  // conj(W1)
    const double w2r = tab[2 * N + 2 * k], w2i = -tab[2 * N + 2 * k + 1];
    if (k == 0) {  // the origin lies on all three lines and carries the mass term
      const double sb = mu[1] + mu[2] + mu[3];
      Fh[0].x += c * (mu[0] + sb * w1r + 3.0 * mu[4] * w2r);
      Fh[0].y += c * (sb * w1i + 3.0 * mu[4] * w2i);
      continue;
    }
    double2 *pa = Fh + k * NN, *pb = Fh + (long long)k * N, *pc = Fh + k;
    pa->x += c * (mu[1] * w1r + mu[4] * w2r);
    pa->y += c * (mu[1] * w1i + mu[4] * w2i);
    pb->x += c * (mu[2] * w1r + mu[4] * w2r);
    pb->y += c * (mu[2] * w1i + mu[4] * w2i);
    pc->x += c * (mu[3] * w1r + mu[4] * w2r);
    pc->y += c * (mu[3] * w1i + mu[4] * w2i);
  }
}

namespace {
// Discrete Maxwellian of Re F (one CTA): writes M_j into F[j].y and returns
// true, or returns false (F untouched) when f has no positive temperature or
// Newton fails.  theta_out (shared) receives (a, b1, b2, b3, c).
__device__ bool discrete_maxwellian(int N, double R, double2 *F, double *red, double *theta_out,
                                    int *iters_out) {
  __shared__ double sh_th[5], sh_dl[5], sh_best[5];
  __shared__ double sh_phi_best;
  __shared__ int sh_flag;
  const long long NQ = (long long)N * N * N, NN = (long long)N * N;
  const double h = 2 * R / N, h3 = h * h * h;
  // target moments of f
  double m[5] = {0, 0, 0, 0, 0};
  for (long long l = threadIdx.x; l < NQ; l += blockDim.x) {
    const double x = -R + (double)(l / NN) * h, y = -R + (double)((l / N) % N) * h,
                 z = -R + (double)(l % N) * h;
    const double f = F[l].x;
    m[0] += f;
    m[1] += f * x;
    m[2] += f * y;
    m[3] += f * z;
    m[4] += f * (x * x + y * y + z * z);
  }
  block_sum_k<5>(m, red);
  for (int q = 0; q < 5; ++q) m[q] *= h3;
  const double rho = m[0];
  if (!(rho > 0.0)) return false;
  const double u1 = m[1] / rho, u2 = m[2] / rho, u3 = m[3] / rho;
  const double u2s = u1 * u1 + u2 * u2 + u3 * u3;
  const double T = (m[4] / rho - u2s) / 3.0;
  if (!(T > 0.0)) return false;
  if (threadIdx.x == 0) {
    sh_th[0] = log(rho / pow(2.0 * M_PI * T, 1.5)) - u2s / (2.0 * T);
    sh_th[1] = u1 / T;
    sh_th[2] = u2 / T;
    sh_th[3] = u3 / T;
    sh_th[4] = -0.5 / T;
    sh_phi_best = INFINITY;
    sh_flag = 0;
  }
  __syncthreads();
  double step = 1.0;
  int it = 0;
  const int MAX_IT = 60;
  bool converged = false;
  for (; it < MAX_IT; ++it) {
    const double a = sh_th[0], b1 = sh_th[1], b2 = sh_th[2], b3 = sh_th[3], c = sh_th[4];
    // moments of M(theta) and the Jacobian (15 distinct sums)
    double g[15];
#pragma unroll
    for (int q = 0; q < 15; ++q) g[q] = 0.0;
    for (long long l = threadIdx.x; l < NQ; l += blockDim.x) {
      const double x = -R + (double)(l / NN) * h, y = -R + (double)((l / N) % N) * h,
                   z = -R + (double)(l % N) * h;
      const double r2 = x * x + y * y + z * z;
      const double M = exp(a + b1 * x + b2 * y + b3 * z + c * r2);
      g[0] += M;
      g[1] += M * x;
      g[2] += M * y;
      g[3] += M * z;
      g[4] += M * r2;
      g[5] += M * x * x;
      g[6] += M * x * y;
      g[7] += M * x * z;
      g[8] += M * y * y;
      g[9] += M * y * z;
      g[10] += M * z * z;
      g[11] += M * x * r2;
      g[12] += M * y * r2;
      g[13] += M * z * r2;
      g[14] += M * r2 * r2;
    }
    block_sum_k<15>(g, red);
    if (threadIdx.x == 0) {
      for (int q = 0; q < 15; ++q) g[q] *= h3;
      const double phi = g[0] - (a * m[0] + b1 * m[1] + b2 * m[2] + b3 * m[3] + c * m[4]);
      int flag = 0;  // 0 continue, 1 converged, 2 failed
      if (!(phi <= sh_phi_best + 1e-15 * fabs(sh_phi_best)) || !isfinite(phi)) {
        // no descent: backtrack from the best point
        step *= 0.5;
        if (step < 1e-6) flag = 2;
        for (int q = 0; q < 5; ++q) sh_th[q] = sh_best[q] + step * sh_dl[q];
      } else {
        sh_phi_best = phi;
        for (int q = 0; q < 5; ++q) sh_best[q] = sh_th[q];
        double J[5][5] = {{g[0], g[1], g[2], g[3], g[4]},
                          {g[1], g[5], g[6], g[7], g[11]},
                          {g[2], g[6], g[8], g[9], g[12]},
                          {g[3], g[7], g[9], g[10], g[13]},
                          {g[4], g[11], g[12], g[13], g[14]}};
        double res[5] = {m[0] - g[0], m[1] - g[1], m[2] - g[2], m[3] - g[3], m[4] - g[4]};
        const double scale[5] = {fabs(m[0]), sqrt(fabs(m[0] * m[4])), sqrt(fabs(m[0] * m[4])),
                                 sqrt(fabs(m[0] * m[4])), fabs(m[4])};
        bool small = true;
        for (int q = 0; q < 5; ++q) small = small && fabs(res[q]) <= 1e-13 * scale[q];
        double dl[5];
        if (small) {
          flag = 1;
        } else if (!solve5(J, res, dl)) {
          flag = 2;
        } else {
          step = 1.0;
          for (int q = 0; q < 5; ++q) {
            sh_dl[q] = dl[q];
            sh_th[q] = sh_best[q] + dl[q];
          }
          if (!(sh_th[4] < 0.0)) {  // keep M decaying: shorten toward the best point
            double t = 1.0;
            while (!(sh_best[4] + t * dl[4] < 0.0) && t > 1e-6) t *= 0.5;
            step = t;
            for (int q = 0; q < 5; ++q) sh_th[q] = sh_best[q] + t * dl[q];
          }
        }
      }
      sh_flag = flag;
    }
    __syncthreads();
    const int flag = sh_flag;
    __syncthreads();
    if (flag == 1) {
      converged = true;
      break;
    }
    if (flag == 2) break;
  }
  if (iters_out && threadIdx.x == 0) *iters_out = it;
  if (!converged) return false;
  const double a = sh_best[0], b1 = sh_best[1], b2 = sh_best[2], b3 = sh_best[3],
               c = sh_best[4];
  for (long long l = threadIdx.x; l < NQ; l += blockDim.x) {
    const double x = -R + (double)(l / NN) * h, y = -R + (double)((l / N) % N) * h,
                 z = -R + (double)(l % N) * h;
    F[l].y = exp(a + b1 * x + b2 * y + b3 * z + c * (x * x + y * y + z * z));
  }
  if (theta_out && threadIdx.x < 5) theta_out[threadIdx.x] = sh_best[threadIdx.x];
  __syncthreads();
  return true;
}

// Moment-preserving FixSol: bisection on beta for y = (1-beta) f + beta M
// with f = Re F and M = Im F (from discrete_maxwellian), the same loop rule as
// the reference's FixSol (EntropyFix.h:211-253) on the integrator's entropy
// density; writes (y, 0) into F.
__device__ void fixsol_moment(double2 *F, long long NQ, double eps, double aim, double *red) {
  const int MAX_BISECT = 400;
  double betaL = 0.0, betaR = 1.0;
  for (int it = 0; it < MAX_BISECT && (betaR - betaL) > eps; ++it) {
    const double mid = 0.5 * (betaL + betaR);
    double acc[1] = {0.0};
    for (long long i = threadIdx.x; i < NQ; i += blockDim.x) {
      const double2 v = F[i];
      acc[0] += flogf_c((1.0 - mid) * v.x + mid * v.y);
    }
    block_sum_k<1>(acc, red);
    const double ent = acc[0] / (double)NQ;
    if (ent < aim && (aim - ent) < eps) {
      betaR = mid;
      break;
    }
    if (ent < aim)
      betaR = mid;
    else
      betaL = mid;
  }
  for (long long i = threadIdx.x; i < NQ; i += blockDim.x) {
    const double2 v = F[i];
    F[i] = make_double2((1.0 - betaR) * v.x + betaR * v.y, 0.0);
  }
  __syncthreads();
}
}  // namespace

// Post-step rule in conservative mode (one CTA per solve): H = calEntropy(F);
// if the scheme allows a fix and H - H_prev > 1e-10, blend Re F toward its
// discrete Maxwellian until H <= H_prev, and flag the solve so the caller
// transforms the fixed F back into F-hat.  Same trace / H_prev / step
// bookkeeping as the reference rule.
__global__ void __launch_bounds__(CT)
    step_entropy_conserve_kernel(int N, double R, double vol, double R3, double2 *__restrict__ F,
                                 EfixState *__restrict__ state, double eps, int fix_mode,
                                 double *__restrict__ trace_raw, double *__restrict__ trace_fixed,
                                 int trace_cap, int keep_last) {
  __shared__ double red[(CW + 1) * 15];
  __shared__ double H_prev;
  __shared__ int step, rec;
  const long long NQ = (long long)N * N * N;
  double2 *Fs = F + (long long)blockIdx.x * NQ;
  EfixState *st = state + blockIdx.x;
  if (threadIdx.x == 0) {
    H_prev = st->H_prev;
    step = st->step;
    rec = st->rec;
  }
  __syncthreads();
  double acc[1] = {0.0};
  for (long long i = threadIdx.x; i < NQ; i += blockDim.x) acc[0] += flogf_c(Fs[i].x);
  block_sum_k<1>(acc, red);
  double H = acc[0] * vol;
  const double raw = H;
  bool allowed = false;
  if (fix_mode == 1) allowed = step > 1;
  else if (fix_mode == 2) allowed = step != 0;
  int fixed = 0;
  if (allowed && H - H_prev > 1.0e-10) {
    if (discrete_maxwellian(N, R, Fs, red, nullptr, nullptr)) {
      fixsol_moment(Fs, NQ, eps, H_prev / R3, red);
      double acc2[1] = {0.0};
      for (long long i = threadIdx.x; i < NQ; i += blockDim.x) acc2[0] += flogf_c(Fs[i].x);
      block_sum_k<1>(acc2, red);
      H = acc2[0] * vol;
      fixed = 1;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int slot = keep_last ? rec % trace_cap : rec;  // as in step_entropy_kernel
    if (slot < trace_cap) {
      trace_raw[(long long)blockIdx.x * trace_cap + slot] = raw;
      trace_fixed[(long long)blockIdx.x * trace_cap + slot] = H;
    }
    st->fixed = fixed;
    st->rec = rec + 1;
    st->H_prev = H;
    st->step = step + 1;
  }
}

// Discrete Maxwellian fit of S real arrays (test and host-API entry):
// M (S x N^3), theta (S x 5: a, b1, b2, b3, c), status (S: Newton iterations,
// or -1 on failure).
__global__ void __launch_bounds__(CT)
    maxwellian_fit_kernel(int N, double R, double2 *__restrict__ F, double *__restrict__ theta,
                          int *__restrict__ status) {
  __shared__ double red[(CW + 1) * 15];
  __shared__ double th[5];
  __shared__ int iters;
  const long long NQ = (long long)N * N * N;
  double2 *Fs = F + (long long)blockIdx.x * NQ;
  const bool ok = discrete_maxwellian(N, R, Fs, red, th, &iters);
  if (threadIdx.x == 0) status[blockIdx.x] = ok ? iters : -1;
  if (ok && threadIdx.x < 5) theta[(long long)blockIdx.x * 5 + threadIdx.x] = th[threadIdx.x];
}

// Copies solve s of src into dst where state[s].fixed is set.
__global__ void masked_copy_kernel(long long NQ, int S, const EfixState *__restrict__ state,
                                   const double2 *__restrict__ src, double2 *__restrict__ dst) {
  const int s = blockIdx.y;
  if (s >= S || !state[s].fixed) return;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < NQ;
       i += (long long)gridDim.x * blockDim.x)
    dst[(long long)s * NQ + i] = src[(long long)s * NQ + i];
}

// Conservative mode starts the entropy rule from the initial data's entropy
// (the reference starts from entropy0 = 1 and skips the fix on step 0).
__global__ void state_from_entropy_kernel(int S, const double *__restrict__ H,
                                          EfixState *__restrict__ state) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  state[s].H_prev = H[s];
  state[s].step = 1;
}

// ------------------------------------------------------------------ host

void build_conserve_table(int N, double R, std::vector<double> &tab) {
  tab.assign((size_t)conserve_table_len(N), 0.0);
  const long double h = 2.0L * R / N;
  const long double PI = 3.141592653589793238462643383279502884L;
  long double S1 = 0, S2 = 0, S3 = 0, S4 = 0;
  for (int j = 0; j < N; ++j) {
    const long double v = -R + j * h;
    S1 += v;
    S2 += v * v;
    S3 += v * v * v;
    S4 += v * v * v * v;
  }
  for (int k = 0; k < N; ++k) {
    long double w1r = 0, w1i = 0, w2r = 0, w2i = 0;
    for (int j = 0; j < N; ++j) {
      const long double v = -R + j * h;
      const long double ang = 2.0L * PI * (long double)((long long)j * k % N) / N;
      const long double cr = cosl(ang), ci = sinl(ang);
      w1r += v * cr;
      w1i += v * ci;
      w2r += v * v * cr;
      w2i += v * v * ci;
    }
    tab[2 * k] = (double)(w1r / N);
    tab[2 * k + 1] = (double)(w1i / N);
    tab[2 * N + 2 * k] = (double)(w2r / N);
    tab[2 * N + 2 * k + 1] = (double)(w2i / N);
  }
  // Gram matrix of the functionals h^3 {1, x, y, z, |v|^2} over the N^3 grid
  const long double n = N, h6 = h * h * h * h * h * h;
  long double G[5][10];
  for (auto &r : G)
    for (auto &x : r) x = 0;
  G[0][0] = n * n * n;
  for (int a = 1; a <= 3; ++a) {
    G[0][a] = G[a][0] = n * n * S1;
    G[a][a] = n * n * S2;
    for (int b = 1; b <= 3; ++b)
      if (b != a) G[a][b] = n * S1 * S1;
    G[a][4] = G[4][a] = n * n * S3 + 2 * n * S1 * S2;
  }
  G[0][4] = G[4][0] = 3 * n * n * S2;
  G[4][4] = 3 * n * n * S4 + 6 * n * S2 * S2;
  for (int r = 0; r < 5; ++r) {
    for (int c = 0; c < 5; ++c) G[r][c] *= h6;
    for (int c = 0; c < 5; ++c) G[r][5 + c] = (r == c) ? 1 : 0;
  }
  // Gauss-Jordan with partial pivoting (long double)
  for (int c = 0; c < 5; ++c) {
    int p = c;
    for (int r = c + 1; r < 5; ++r)
      if (fabsl(G[r][c]) > fabsl(G[p][c])) p = r;
    for (int k = 0; k < 10; ++k) {
      long double t = G[c][k];
      G[c][k] = G[p][k];
      G[p][k] = t;
    }
    const long double piv = G[c][c];
    for (int k = 0; k < 10; ++k) G[c][k] /= piv;
    for (int r = 0; r < 5; ++r) {
      if (r == c) continue;
      const long double f = G[r][c];
      for (int k = 0; k < 10; ++k) G[r][k] -= f * G[c][k];
    }
  }
  for (int r = 0; r < 5; ++r)
    for (int c = 0; c < 5; ++c) tab[4 * N + r * 5 + c] = (double)G[r][5 + c];
  tab[4 * N + 25] = (double)(h * h * h);
}

edb_status launch_hat_moments(int N, int S, const double *d_tab, const double2 *d_Fhat,
                              double *d_out, cudaStream_t st) {
  const int wpb = 4;
  hat_moments_kernel<<<(S + wpb - 1) / wpb, 32 * wpb, 0, st>>>(N, S, d_tab, d_Fhat, d_out);
  EDB_LAUNCHED();
  return EDB_OK;
}

edb_status launch_project_moments(int N, int S, const double *d_tab, double2 *d_Fhat,
                                  const double *d_m0, cudaStream_t st) {
  const int wpb = 4;
  project_moments_kernel<<<(S + wpb - 1) / wpb, 32 * wpb, 0, st>>>(N, S, d_tab, d_Fhat, d_m0);
  EDB_LAUNCHED();
  return EDB_OK;
}

edb_status launch_step_entropy_conserve(int N, int batch, double R, double2 *d_F,
                                        EfixState *d_state, double eps, int fix_mode,
                                        double *d_trace_raw, double *d_trace_fixed,
                                        int trace_cap, cudaStream_t st, bool keep_last) {
  const long long NQ = (long long)N * N * N;
  const double vol = pow(2 * R, 3.) / (double)NQ, R3 = pow(2 * R, 3);
  if (keep_last && trace_cap < 1) return fail(EDB_EINVAL, "step entropy: empty trace");
  step_entropy_conserve_kernel<<<batch, CT, 0, st>>>(N, R, vol, R3, d_F, d_state, eps, fix_mode,
                                                     d_trace_raw, d_trace_fixed, trace_cap,
                                                     keep_last ? 1 : 0);
  EDB_LAUNCHED();
  return EDB_OK;
}

edb_status launch_maxwellian_fit(int N, int S, double R, double2 *d_F, double *d_theta,
                                 int *d_status, cudaStream_t st) {
  maxwellian_fit_kernel<<<S, CT, 0, st>>>(N, R, d_F, d_theta, d_status);
  EDB_LAUNCHED();
  return EDB_OK;
}

edb_status launch_state_from_entropy(int S, const double *d_H, EfixState *d_state,
                                     cudaStream_t st) {
  state_from_entropy_kernel<<<(S + 127) / 128, 128, 0, st>>>(S, d_H, d_state);
  EDB_LAUNCHED();
  return EDB_OK;
}

edb_status launch_masked_copy(long long NQ, int S, const EfixState *d_state,
                              const double2 *d_src, double2 *d_dst, cudaStream_t st) {
  dim3 grid((unsigned)((NQ + 255) / 256 < 64 ? (NQ + 255) / 256 : 64), (unsigned)S);
  masked_copy_kernel<<<grid, 256, 0, st>>>(NQ, S, d_state, d_src, d_dst);
  EDB_LAUNCHED();
  return EDB_OK;
}

}  // namespace edb
