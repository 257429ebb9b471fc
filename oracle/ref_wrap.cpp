// C entry points over the UNMODIFIED reference headers — ORACLE TEST INFRASTRUCTURE ONLY.
//
// Compiled by oracle/Makefile (target `ref`) directly from the reference
// sources where they lie (CalQ/QCalculator.h, CalQ/EntropyFix.h, CalQ/fft3d.h,
// CalQ/BKW.h, CalQ/TimeWatch.h), into oracle/_ref/libedbref.so.  The FFTW3
// calls inside CalQ/fft3d.h resolve to the in-repo shim oracle/fftw_shim/fftw3.h.
// Nothing here re-implements reference arithmetic: every function forwards to
// the reference class methods.  Private members are opened with
// `#define private public` only to read the B table (QCalculator.h:29) and the
// BKW3D state arrays (BKW.h:31-33).
//
// This library exists only where the reference sources exist; tests that use
// it skip when it is absent.
#include <assert.h>
#include <sys/time.h>

#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

#define private public
#include "BKW.h"
#undef private

typedef std::complex<double> c_t;
typedef QCalculator<c_t, double> QC;
typedef EntropyFix<int, double> EF;
typedef BKW3D<c_t, double> BK;

namespace {
// Captures std::cout for the lifetime of the object (the reference prints its
// entropy history and timers there; BKW.h:212-241, TimeWatch.h:24-34).
struct CoutCapture {
  std::ostringstream buf;
  std::streambuf *old;
  CoutCapture() : old(std::cout.rdbuf(buf.rdbuf())) {}
  ~CoutCapture() { std::cout.rdbuf(old); }
  void copy_to(char *dst, int cap) {
    if (!dst || cap <= 0) return;
    std::string s = buf.str();
    int n = (int)s.size() < cap - 1 ? (int)s.size() : cap - 1;
    std::memcpy(dst, s.data(), n);
    dst[n] = 0;
  }
};
}  // namespace

extern "C" {

// QCalculator(N, alpha) (QCalculator.h:39), optional closeFilter (:54), genB (:158).
void *edbref_qcalc_new(int N, int alpha, int filter) {
  QC *q = new QC(N, alpha);
  if (!filter) q->closeFilter();
  q->genB();
  return q;
}

// QCalculator::calQ (QCalculator.h:231-257); fin / qout are N^3 interleaved complex.
void edbref_qcalc_calQ(void *h, const double *fin, double *qout) {
  QC *q = (QC *)h;
  int nq = q->NQ;
  std::vector<c_t> in(nq), out(nq);
  for (int i = 0; i < nq; ++i) in[i] = c_t(fin[2 * i], fin[2 * i + 1]);
  q->calQ(out.data(), in.data());
  for (int i = 0; i < nq; ++i) {
    qout[2 * i] = out[i].real();
    qout[2 * i + 1] = out[i].imag();
  }
}

// Copy of the private B table (QCalculator.h:29, filled by genB :158-229).
void edbref_qcalc_copyB(void *h, double *out) {
  QC *q = (QC *)h;
  long nb = (long)q->NQ * q->NQ;
  std::memcpy(out, q->B, sizeof(double) * nb);
}

void edbref_qcalc_free(void *h) { delete (QC *)h; }

// funF / filtering (QCalculator.h:67-106) on an object without tables.
static QC *bare(int N, int alpha) {
  QC *q = new QC();
  q->N = N;
  q->n = (N - 1) / 2;
  q->alpha = alpha;
  q->Q = nullptr;
  q->f = nullptr;
  q->B = nullptr;
  return q;
}
double edbref_funF(int alpha, double xi, double eta) {
  QC *q = bare(3, alpha);
  double r = q->funF(xi, eta);
  delete q;
  return r;
}
double edbref_filtering(int N, int beta) {
  QC *q = bare(N, 0);
  double r = q->filtering(beta);
  delete q;
  return r;
}

// EntropyFix (EntropyFix.h:29-253).
void *edbref_efix_new(int Nt, double eps) { return new EF(Nt, eps); }
void edbref_efix_free(void *h) { delete (EF *)h; }
double edbref_efix_entropy(void *h, int Nf, double *f) {
  CoutCapture cap;
  return ((EF *)h)->EntropyCal(Nf, f);
}
void edbref_efix_setaverage(void *h, int Nf, double *f) {
  CoutCapture cap;
  ((EF *)h)->setAverage(Nf, f);
}
void edbref_efix_fixsol(void *h, int Nf, double *f, double aim) {
  CoutCapture cap;
  ((EF *)h)->FixSol(Nf, f, aim);
}
double edbref_efix_average(void *h) { return ((EF *)h)->Averagef; }
int edbref_efix_average_flag(void *h) { return ((EF *)h)->Average_flag ? 1 : 0; }

// fft3d::fft / ifft (fft3d.h:25-48).
void edbref_fft(int nx, int ny, int nz, double *re, double *fre) {
  fft3d f;
  f.fft(nx, ny, nz, (fftw_complex *)re, (fftw_complex *)fre);
}
void edbref_ifft(int nx, int ny, int nz, double *re, double *fre) {
  fft3d f;
  f.ifft(nx, ny, nz, (fftw_complex *)re, (fftw_complex *)fre);
}

// BKW3D::setInitialValue (BKW.h:121-138) -> F (N^3 complex).
void edbref_bkw_initial(int N, double R, double t, double *F_out) {
  BK b(N, R);
  b.setInitialValue(t);
  std::memcpy(F_out, (double *)b.F, sizeof(double) * 2 * b.N3d);
}

// BKW3D::calEntropy (BKW.h:140-152) of a given F.
double edbref_bkw_entropy(int N, double R, const double *F) {
  BK b(N, R);
  std::memcpy((double *)b.F, F, sizeof(double) * 2 * b.N3d);
  return b.calEntropy();
}

// Runs one reference integrator end to end and returns the final F and Fhat
// plus everything it printed.  scheme: 0 FEuler (BKW.h:191), 1 CFE (:254),
// 2 RK2 (:314), 3 SSP3 (:387), 4 RK4 (:452), 5 DUFORT (:522).
// FEuler writes F.dat into the current directory (BKW.h:217).
int edbref_bkw_run(int N, double R, int scheme, double T0, double TEnd, double dt,
                   double beta, int fix_entropy, double *Fhat_out, double *F_out,
                   char *log_out, int log_cap) {
  BK b(N, R);
  b.setFixEntropy(fix_entropy != 0);
  CoutCapture cap;
  switch (scheme) {
    case 0: b.FEuler(T0, TEnd, dt); break;
    case 1: b.CFE(T0, TEnd, dt, beta); break;
    case 2: b.RK2(T0, TEnd, dt); break;
    case 3: b.SSP3(T0, TEnd, dt); break;
    case 4: b.RK4(T0, TEnd, dt); break;
    case 5: b.DUFORT(T0, TEnd, dt, beta); break;
    default: return -1;
  }
  std::memcpy(Fhat_out, (double *)b.Fhat, sizeof(double) * 2 * b.N3d);
  std::memcpy(F_out, (double *)b.F, sizeof(double) * 2 * b.N3d);
  cap.copy_to(log_out, log_cap);
  return 0;
}

// BKW3D::FEuler (BKW.h:191-251), which writes F.dat into the current
// directory, then outV1Direction(slice) as testBKW3D.cpp:43-45 does; stdout is
// captured and dropped.
int edbref_bkw_fe_files(int N, double R, double T0, double TEnd, double dt, int fix_entropy,
                        const char *slice) {
  BK b(N, R);
  b.setFixEntropy(fix_entropy != 0);
  CoutCapture cap;
  b.FEuler(T0, TEnd, dt);
  b.outV1Direction(slice);
  return 0;
}

// Times the reference calQ: `reps` calls on the same input; returns seconds
// per call (steady_clock).  Used only as a CPU baseline where the reference
// sources exist.
double edbref_time_calQ(void *h, const double *fin, double *qout, int reps) {
  auto t0 = std::chrono::steady_clock::now();
  for (int r = 0; r < reps; ++r) edbref_qcalc_calQ(h, fin, qout);
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count() / (reps > 0 ? reps : 1);
}

}  // extern "C"
