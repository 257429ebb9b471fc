// Entropy, EntropyFix, moments, stage updates and conversions (FP64).
//
// Compiled with -fmad=false: every product and sum is rounded where the
// reference rounds it, so stage updates reproduce BKW.h's expressions
// operation by operation.  Reductions run one CTA per solve with a fixed
// tree order (deterministic run to run; the reference sums sequentially, so
// sums agree to round-off only).
#include <math.h>

#include "edb_internal.cuh"

namespace edb {

namespace {
constexpr int RT = 1024;  // threads of a per-solve reduction CTA

// Block-wide sum in a fixed order; result valid in every thread.
__device__ double block_sum(double v, double *red) {
  const int tid = threadIdx.x;
  red[tid] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (tid < s) red[tid] += red[tid + s];
    __syncthreads();
  }
  double r = red[0];
  __syncthreads();
  return r;
}

// flogf (BKW.h:153-161)
__device__ __forceinline__ double flogf_dev(double f) {
  if (fabs(f) < 1.0e-6) return 0.;
  return f * log(f) - f;
}

// sum over f_i > eps of f_i log f_i (EntropyFix.h:139-143) of
// fMid_i = beta*avg + (1-beta) f_i (FixSol's trial state, :226-231), or of
// f_i itself when beta_bar < 0.
__device__ double efix_sum(const double2 *F, const double *f, long long Nf, double betaFbar,
                           double omb, bool trial, double eps, double *red) {
  double acc = 0.0;
  for (long long i = threadIdx.x; i < Nf; i += blockDim.x) {
    double x = F ? F[i].x : f[i];
    if (trial) {
      double y = betaFbar;
      y += omb * x;
      x = y;
    }
    if (x > eps) acc += x * log(x);
  }
  return block_sum(acc, red);
}

__device__ double mean_re(const double2 *F, const double *f, long long Nf, double *red) {
  double acc = 0.0;
  for (long long i = threadIdx.x; i < Nf; i += blockDim.x) acc += F ? F[i].x : f[i];
  return block_sum(acc, red) / (double)Nf;
}

// Block-uniform copy of the latched average (EntropyFix.h:20-22).  Thread 0
// loads it from the per-solve state before a barrier and stores it back after
// one, so no thread ever reads the state while another writes it.
struct AvgSnap {
  double avg;
  int flag;
};

// FixSol (EntropyFix.h:211-253) on Re F (F != null, imaginary parts zeroed as
// BKW.h:232 does) or on a real array f.  `snap` lives in shared memory and is
// block-uniform on entry and exit.  The bisection halves [betaL, betaR] until
// its width is <= eps (about 34 halvings from [0,1] at eps = 1e-10), so the
// loop is bounded; MAX_BISECT is a hard guard on top.  Every branch below
// depends only on block-reduced values, so all threads take it together.
__device__ void fixsol_dev(double2 *F, double *f, long long Nf, AvgSnap *snap, double eps,
                           double aim, double *red) {
  const int MAX_BISECT = 400;
  double betaL = 0.0, betaR = 1.0;
  for (int it = 0; it < MAX_BISECT && (betaR - betaL) > eps; ++it) {
    double betaMid = 0.5 * (betaL + betaR);
    if (!snap->flag) {
      double avg = mean_re(F, f, Nf, red);  // ends with a barrier
      if (threadIdx.x == 0) {
        snap->avg = avg;
        snap->flag = 1;
      }
      __syncthreads();
    }
    const double avg = snap->avg;
    const double betaFbar = betaMid * avg;
    const double omb = 1. - betaMid;
    double s = efix_sum(F, f, Nf, betaFbar, omb, true, eps, red);
    double entMid = s / (double)Nf - avg;
    if ((entMid < aim) && ((aim - entMid) < eps)) {
      for (long long i = threadIdx.x; i < Nf; i += blockDim.x) {
        double x = F ? F[i].x : f[i];
        double y = betaFbar;
        y += omb * x;
        if (F)
          F[i] = make_double2(y, 0.0);
        else
          f[i] = y;
      }
      __syncthreads();
      return;
    }
    if (entMid < aim)
      betaR = betaMid;
    else
      betaL = betaMid;
  }
  const double betaFbar = betaR * snap->avg;
  for (long long i = threadIdx.x; i < Nf; i += blockDim.x) {
    double x = F ? F[i].x : f[i];
    x *= (1.0 - betaR);
    x += betaFbar;
    if (F)
      F[i] = make_double2(x, 0.0);
    else
      f[i] = x;
  }
  __syncthreads();
}
}  // namespace

// calEntropy (BKW.h:140-152): (sum flogf(Re F_i)) * ((2R)^3 / N^3).
__global__ void __launch_bounds__(RT) calentropy_kernel(long long NQ, double vol,
                                                        const double2 *__restrict__ F,
                                                        double *__restrict__ H) {
  __shared__ double red[RT];
  const double2 *Fs = F + (long long)blockIdx.x * NQ;
  double acc = 0.0;
  for (long long i = threadIdx.x; i < NQ; i += blockDim.x) acc += flogf_dev(Fs[i].x);
  double s = block_sum(acc, red);
  if (threadIdx.x == 0) H[blockIdx.x] = s * vol;
}

edb_status launch_calentropy(int N, int batch, double R, const double2 *d_F, double *d_H,
                             cudaStream_t st) {
  long long NQ = (long long)N * N * N;
  double vol = pow(2 * R, 3.) / (double)NQ;
  calentropy_kernel<<<batch, RT, 0, st>>>(NQ, vol, d_F, d_H);
  EDB_LAUNCHED();
  return EDB_OK;
}

// Post-step rule of the integrators, one CTA per solve (BKW.h:225-242,
// 286-310, 427-445, 497-515): H = calEntropy(F); if the scheme allows a fix
// this step and H - H_prev > 1e-10 then FixSol(Re F, H_prev/(2R)^3) and
// recompute H; record (raw, fixed); H_prev = H; step++.
__global__ void __launch_bounds__(RT)
    step_entropy_kernel(long long NQ, double vol, double R3, double2 *__restrict__ F,
                        EfixState *__restrict__ state, double eps, int fix_mode,
                        double *__restrict__ trace_raw, double *__restrict__ trace_fixed,
                        int trace_cap, int keep_last) {
  __shared__ double red[RT];
  __shared__ AvgSnap snap;
  __shared__ double H_prev;
  __shared__ int step, rec;
  double2 *Fs = F + (long long)blockIdx.x * NQ;
  EfixState *st = state + blockIdx.x;
  if (threadIdx.x == 0) {
    snap.avg = st->avg;
    snap.flag = st->avg_flag;
    H_prev = st->H_prev;
    step = st->step;
    rec = st->rec;
  }
  __syncthreads();
  double acc = 0.0;
  for (long long i = threadIdx.x; i < NQ; i += blockDim.x) acc += flogf_dev(Fs[i].x);
  double H = block_sum(acc, red) * vol;
  const double raw = H;
  bool allowed = false;
  if (fix_mode == 1) allowed = step > 1;
  else if (fix_mode == 2) allowed = step != 0;
  if (allowed && H - H_prev > 1.0e-10) {
    fixsol_dev(Fs, nullptr, NQ, &snap, eps, H_prev / R3, red);
    double acc2 = 0.0;
    for (long long i = threadIdx.x; i < NQ; i += blockDim.x) acc2 += flogf_dev(Fs[i].x);
    H = block_sum(acc2, red) * vol;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // keep_last: the trace keeps the last trace_cap steps (slot rec mod cap)
    const int slot = keep_last ? rec % trace_cap : rec;
    if (slot < trace_cap) {
      trace_raw[(long long)blockIdx.x * trace_cap + slot] = raw;
      trace_fixed[(long long)blockIdx.x * trace_cap + slot] = H;
    }
    st->avg = snap.avg;
    st->avg_flag = snap.flag;
    st->rec = rec + 1;
    st->H_prev = H;
    st->step = step + 1;
  }
}

edb_status launch_step_entropy(int N, int batch, double R, double2 *d_F, EfixState *d_state,
                               double eps, int fix_mode, double *d_trace_raw,
                               double *d_trace_fixed, int trace_cap, cudaStream_t st,
                               bool keep_last) {
  long long NQ = (long long)N * N * N;
  double vol = pow(2 * R, 3.) / (double)NQ;
  double R3 = pow(2 * R, 3);
  if (keep_last && trace_cap < 1) return fail(EDB_EINVAL, "step entropy: empty trace");
  step_entropy_kernel<<<batch, RT, 0, st>>>(NQ, vol, R3, d_F, d_state, eps, fix_mode,
                                            d_trace_raw, d_trace_fixed, trace_cap,
                                            keep_last ? 1 : 0);
  EDB_LAUNCHED();
  return EDB_OK;
}

// ---- EntropyFix primitives on a real array (host-API wrappers)
__global__ void __launch_bounds__(RT) efix_average_kernel(long long Nf, const double *f,
                                                          EfixState *st) {
  __shared__ double red[RT];
  double avg = mean_re(nullptr, f, Nf, red);
  if (threadIdx.x == 0) {
    st->avg = avg;
    st->avg_flag = 1;
  }
}

__global__ void __launch_bounds__(RT) efix_entropy_kernel(long long Nf, const double *f,
                                                          EfixState *st, double eps,
                                                          double *H) {
  __shared__ double red[RT];
  __shared__ AvgSnap snap;
  if (threadIdx.x == 0) {
    snap.avg = st->avg;
    snap.flag = st->avg_flag;
  }
  __syncthreads();
  if (!snap.flag) {
    double avg = mean_re(nullptr, f, Nf, red);  // ends with a barrier
    if (threadIdx.x == 0) {
      snap.avg = avg;
      snap.flag = 1;
    }
    __syncthreads();
  }
  double s = efix_sum(nullptr, f, Nf, 0.0, 1.0, false, eps, red);
  if (threadIdx.x == 0) {
    *H = s / (double)Nf - snap.avg;
    st->avg = snap.avg;
    st->avg_flag = snap.flag;
  }
}

__global__ void __launch_bounds__(RT) efix_fixsol_kernel(long long Nf, double *f, EfixState *st,
                                                         double eps, double aim) {
  __shared__ double red[RT];
  __shared__ AvgSnap snap;
  if (threadIdx.x == 0) {
    snap.avg = st->avg;
    snap.flag = st->avg_flag;
  }
  __syncthreads();
  fixsol_dev(nullptr, f, Nf, &snap, eps, aim, red);
  if (threadIdx.x == 0) {
    st->avg = snap.avg;
    st->avg_flag = snap.flag;
  }
}

edb_status launch_efix_average(int Nf, const double *d_f, EfixState *d_state, cudaStream_t st) {
  efix_average_kernel<<<1, RT, 0, st>>>(Nf, d_f, d_state);
  EDB_LAUNCHED();
  return EDB_OK;
}
edb_status launch_efix_entropy(int Nf, const double *d_f, EfixState *d_state, double eps,
                               double *d_H, cudaStream_t st) {
  efix_entropy_kernel<<<1, RT, 0, st>>>(Nf, d_f, d_state, eps, d_H);
  EDB_LAUNCHED();
  return EDB_OK;
}
edb_status launch_efix_fixsol(int Nf, double *d_f, EfixState *d_state, double eps, double aim,
                              cudaStream_t st) {
  efix_fixsol_kernel<<<1, RT, 0, st>>>(Nf, d_f, d_state, eps, aim);
  EDB_LAUNCHED();
  return EDB_OK;
}

// ---- stage updates
// Each op reproduces one BKW.h expression operation by operation (this unit
// has no multiply-add contraction); the scalars are computed on the host
// exactly as BKW.h writes them (0.5*dt, 0.25*dt, 2./3.*dt, dt/6., ...).
//   STAGE_AXPY    y = x + c1*q0                      FE :221-222, CFE :282-283,
//                                                    RK2 :342-346, SSP3 :417-418,
//                                                    RK4 :483-490
//   STAGE_SSP3_2  y = 0.75*x + 0.25*z + c1*q0        SSP3 :420-421
//   STAGE_SSP3_3  y = x/3. + 2.*z/3. + c1*q0         SSP3 :423-424
//   STAGE_RK4     y = x + c1*(q0 + 2.*q1 + 2.*q2 + q3)   RK4 :493-494
//   STAGE_DUFORT  y = c0*(z + c1*q0 + c2*(z - w))    DUFORT :597-598
// Q-hat inputs are double2 (FP64 path) or float2 (batched FP32 path, widened
// exactly).  y32, when given, receives the result rounded to float.
template <typename TQ>
__device__ __forceinline__ double2 ld(const TQ *p, long long i) {
  return make_double2((double)p[i].x, (double)p[i].y);
}

template <typename TQ>
__global__ void stage_kernel(long long n, int op, double c0, double c1, double c2, double2 *y,
                             const double2 *x, const double2 *z, const double2 *w, const TQ *q0,
                             const TQ *q1, const TQ *q2, const TQ *q3, float2 *y32) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double rx, ry;
  if (op == STAGE_AXPY) {
    double2 a = x[i], q = ld(q0, i);
    rx = a.x + c1 * q.x;
    ry = a.y + c1 * q.y;
  } else if (op == STAGE_SSP3_2) {
    double2 a = x[i], b = z[i], q = ld(q0, i);
    rx = 0.75 * a.x + 0.25 * b.x + c1 * q.x;
    ry = 0.75 * a.y + 0.25 * b.y + c1 * q.y;
  } else if (op == STAGE_SSP3_3) {
    double2 a = x[i], b = z[i], q = ld(q0, i);
    rx = a.x / 3. + 2. * b.x / 3. + c1 * q.x;
    ry = a.y / 3. + 2. * b.y / 3. + c1 * q.y;
  } else if (op == STAGE_RK4) {
    double2 a = x[i], p0 = ld(q0, i), p1 = ld(q1, i), p2 = ld(q2, i), p3 = ld(q3, i);
    rx = a.x + c1 * (p0.x + 2. * p1.x + 2. * p2.x + p3.x);
    ry = a.y + c1 * (p0.y + 2. * p1.y + 2. * p2.y + p3.y);
  } else {  // STAGE_DUFORT
    double2 b = z[i], o = w[i], q = ld(q0, i);
    rx = c0 * (b.x + c1 * q.x + c2 * (b.x - o.x));
    ry = c0 * (b.y + c1 * q.y + c2 * (b.y - o.y));
  }
  if (y) y[i] = make_double2(rx, ry);
  if (y32) y32[i] = make_float2((float)rx, (float)ry);
}

template <typename TQ>
static edb_status stage_t(long long n, int op, double c0, double c1, double c2, double2 *y,
                          const double2 *x, const double2 *z, const double2 *w, const TQ *q0,
                          const TQ *q1, const TQ *q2, const TQ *q3, float2 *y32,
                          cudaStream_t st) {
  stage_kernel<TQ><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, op, c0, c1, c2, y, x, z, w,
                                                                 q0, q1, q2, q3, y32);
  EDB_LAUNCHED();
  return EDB_OK;
}

edb_status launch_stage(long long n, int op, double c0, double c1, double c2, double2 *y,
                        const double2 *x, const double2 *z, const double2 *w, const double2 *q0,
                        const double2 *q1, const double2 *q2, const double2 *q3, float2 *y32,
                        cudaStream_t st) {
  return stage_t<double2>(n, op, c0, c1, c2, y, x, z, w, q0, q1, q2, q3, y32, st);
}

edb_status launch_stage_f32q(long long n, int op, double c0, double c1, double c2, double2 *y,
                             const double2 *x, const double2 *z, const double2 *w,
                             const float2 *q0, const float2 *q1, const float2 *q2,
                             const float2 *q3, float2 *y32, cudaStream_t st) {
  return stage_t<float2>(n, op, c0, c1, c2, y, x, z, w, q0, q1, q2, q3, y32, st);
}

__global__ void d2f_kernel(long long n, const double2 *x, float2 *y) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = make_float2((float)x[i].x, (float)x[i].y);
}
__global__ void f2d_kernel(long long n, const float2 *x, double2 *y) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = make_double2((double)x[i].x, (double)x[i].y);
}
__global__ void r2c_kernel(long long n, const double *x, double2 *y) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = make_double2(x[i], 0.0);
}

edb_status launch_d2f(long long n, const double2 *x, float2 *y, cudaStream_t st) {
  d2f_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, x, y);
  EDB_LAUNCHED();
  return EDB_OK;
}
edb_status launch_f2d(long long n, const float2 *x, double2 *y, cudaStream_t st) {
  f2d_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, x, y);
  EDB_LAUNCHED();
  return EDB_OK;
}
// Re y -> x (the inverse of r2c for real data).
__global__ void c2r_kernel(long long n, const double2 *__restrict__ y, double *__restrict__ x) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = y[i].x;
}

edb_status launch_complex_to_real(long long n, const double2 *y, double *x, cudaStream_t st) {
  const long long cap = 32LL * device_sm_count();
  const long long blocks = (n + 255) / 256 < cap ? (n + 255) / 256 : cap;
  c2r_kernel<<<(unsigned)blocks, 256, 0, st>>>(n, y, x);
  EDB_LAUNCHED();
  return EDB_OK;
}

edb_status launch_real_to_complex(long long n, const double *x, double2 *y, cudaStream_t st) {
  r2c_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, x, y);
  EDB_LAUNCHED();
  return EDB_OK;
}

// setInitialValue with the live funExact branch (BKW.h:96-138).
// BKW3D::funExact, the live branch (BKW.h:96-112): the synthetic sinusoid.
__device__ double funexact_dev(double R, double PI, double x, double y, double z) {
  double r1 = (x + R) / (2. * R);
  double r2 = (y + R) / (2. * R);
  double r3 = (z + R) / (2. * R);
  double val = 3.2;
  for (int jj = 0; jj < 11; ++jj)
    val += fabs((double)jj) / 55 * sin(jj * (r1 - 0.5) * PI) +
           fabs((double)jj) / 55. * sin(jj * (r2 - 0.5) * PI) +
           fabs((double)jj) / 55. * sin(jj * (r3 - 0.5) * PI);
  return val;
}

__global__ void sinusoid_kernel(int N, double R, double PI, double2 *F) {
  long long NQ = (long long)N * N * N;
  long long l = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= NQ) return;
  int i = (int)(l / ((long long)N * N)), j = (int)((l / N) % N), k = (int)(l % N);
  double h = 2 * R / (double)N;
  double x = -R + i * h, y = -R + j * h, z = -R + k * h;
  F[l] = make_double2(funexact_dev(R, PI, x, y, z), 0.0);
}

edb_status launch_sinusoid_init(int N, double R, double2 *d_F, cudaStream_t st) {
  long long NQ = (long long)N * N * N;
  sinusoid_kernel<<<(unsigned)((NQ + 255) / 256), 256, 0, st>>>(N, R, M_PI, d_F);
  EDB_LAUNCHED();
  return EDB_OK;
}

// funExact at n points (x[i], y, z) (outV1Direction's reference column).
__global__ void funexact_points_kernel(double R, double PI, int n, const double *__restrict__ x,
                                       double y, double z, double *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = funexact_dev(R, PI, x[i], y, z);
}

edb_status launch_funexact_points(double R, int n, const double *d_x, double y, double z,
                                  double *d_out, cudaStream_t st) {
  funexact_points_kernel<<<(n + 127) / 128, 128, 0, st>>>(R, M_PI, n, d_x, y, z, d_out);
  EDB_LAUNCHED();
  return EDB_OK;
}

// Copies Re F into record (rec - 1) of the history: the record the step's
// entropy rule has just written (the index lives on the device, so a replayed
// graph fills successive rows).
__global__ void record_re_kernel(long long NQ, const double2 *__restrict__ F,
                                 const EfixState *__restrict__ state, double *__restrict__ hist,
                                 int cap) {
  const int rec = state->rec - 1;
  if (rec < 0 || rec >= cap) return;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < NQ;
       i += (long long)gridDim.x * blockDim.x)
    hist[(long long)rec * NQ + i] = F[i].x;
}

edb_status launch_record_re(long long NQ, const double2 *d_F, const EfixState *d_state,
                            double *d_hist, int cap, cudaStream_t st) {
  const long long blocks = (NQ + 255) / 256 < 1024 ? (NQ + 255) / 256 : 1024;
  record_re_kernel<<<(unsigned)blocks, 256, 0, st>>>(NQ, d_F, d_state, d_hist, cap);
  EDB_LAUNCHED();
  return EDB_OK;
}

// mass, momentum, energy of Re F on the grid x_i = -R + i h (FP64).
__global__ void __launch_bounds__(RT) moments_kernel(int N, double R, const double2 *F,
                                                     double *out) {
  __shared__ double red[RT];
  long long NQ = (long long)N * N * N;
  const double2 *Fs = F + (long long)blockIdx.x * NQ;
  double h = 2 * R / (double)N;
  double m = 0, p1 = 0, p2 = 0, p3 = 0, e = 0;
  for (long long l = threadIdx.x; l < NQ; l += blockDim.x) {
    int i = (int)(l / ((long long)N * N)), j = (int)((l / N) % N), k = (int)(l % N);
    double x = -R + i * h, y = -R + j * h, z = -R + k * h;
    double f = Fs[l].x;
    m += f;
    p1 += f * x;
    p2 += f * y;
    p3 += f * z;
    e += 0.5 * f * (x * x + y * y + z * z);
  }
  double h3 = h * h * h;
  double vals[5] = {m, p1, p2, p3, e};
  for (int q = 0; q < 5; ++q) {
    double s = block_sum(vals[q], red);
    if (threadIdx.x == 0) out[(long long)blockIdx.x * 5 + q] = s * h3;
  }
}

edb_status launch_moments(int N, int batch, double R, const double2 *d_F, double *d_out,
                          cudaStream_t st) {
  moments_kernel<<<batch, RT, 0, st>>>(N, R, d_F, d_out);
  EDB_LAUNCHED();
  return EDB_OK;
}

}  // namespace edb
