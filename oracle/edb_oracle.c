/*
 * edb_oracle.c — CPU restatement of the reference spectral collision step.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline; see
 * edb_oracle.h).  Compiled with -ffp-contract=off so that the arithmetic is
 * the plain IEEE double sequence of the reference's C++ on every host.
 * Every function cites the reference lines (path within the reference
 * project) whose algorithm it restates.
 */
#include "edb_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ kernel */

/* Jackson-type filter sigma(beta), QCalculator.h:67-74, with n = (N-1)/2 (:44). */
double edbo_filtering(int N, int beta) {
  int n = (N - 1) / 2;
  double tmp = (double)(n + 1);
  double PI = 4. * atan(1.);
  double b = fabs((double)beta);
  return ((tmp - b) * cos(PI * b / tmp) + sin(PI * b / tmp) / tan(PI / tmp)) / tmp;
}

/* Closed forms F_0 (Maxwell) and F_1 (hard sphere), QCalculator.h:76-106
 * (ReadMe.md:55-68).  Any other alpha returns 0, as the reference does (:104). */
double edbo_funF(int alpha, double xi, double eta) {
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
  } else {
    res = 0.0;
  }
  return res;
}

/* ---- general VHS exponent: F_gamma(xi, eta) = int_0^1 r^(2+gamma) sinc(xi r) sinc(eta r) dr
 * (ReadMe.md:51; the reference has no code for gamma outside {0,1}).  Computed
 * with the substitution r = u^2, which makes the integrand 2 u^(5+2 gamma)
 * sinc(xi u^2) sinc(eta u^2) smooth on [0,1], and composite Gauss-Legendre
 * quadrature (EDBO_GL_PANELS panels of EDBO_GL_ORDER nodes; nodes by Newton
 * iteration on the Legendre three-term recurrence). */
#define EDBO_GL_ORDER 16
#define EDBO_GL_PANELS 32
static double gl_x[EDBO_GL_ORDER], gl_w[EDBO_GL_ORDER];
static int gl_ready = 0;
static pthread_mutex_t gl_mu = PTHREAD_MUTEX_INITIALIZER;

static void gl_init(void) {
  pthread_mutex_lock(&gl_mu);
  if (!gl_ready) {
    const int G = EDBO_GL_ORDER;
    for (int i = 0; i < G; ++i) {
      double x = cos(M_PI * (i + 0.75) / (G + 0.5));
      double dp = 0.0;
      for (int it = 0; it < 100; ++it) {
        double p0 = 1.0, p1 = x;
        for (int k = 2; k <= G; ++k) {
          double pk = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
          p0 = p1;
          p1 = pk;
        }
        dp = G * (x * p1 - p0) / (x * x - 1.0);
        double dx = p1 / dp;
        x -= dx;
        if (fabs(dx) < 1e-16) break;
      }
      {
        double p0 = 1.0, p1 = x;
        for (int k = 2; k <= G; ++k) {
          double pk = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
          p0 = p1;
          p1 = pk;
        }
        dp = G * (x * p1 - p0) / (x * x - 1.0);
      }
      gl_x[i] = x;
      gl_w[i] = 2.0 / ((1.0 - x * x) * dp * dp);
    }
    gl_ready = 1;
  }
  pthread_mutex_unlock(&gl_mu);
}

static double sinc(double x) { return x == 0.0 ? 1.0 : sin(x) / x; }

double edbo_funF_quad(double gamma, double xi, double eta) {
  if (!gl_ready) gl_init();
  double sum = 0.0;
  const double h = 1.0 / EDBO_GL_PANELS;
  for (int p = 0; p < EDBO_GL_PANELS; ++p) {
    double a = p * h;
    for (int i = 0; i < EDBO_GL_ORDER; ++i) {
      double u = a + 0.5 * h * (gl_x[i] + 1.0);
      double r = u * u;
      double wt = 0.5 * h * gl_w[i] * 2.0 * pow(u, 5.0 + 2.0 * gamma);
      sum += wt * sinc(xi * r) * sinc(eta * r);
    }
  }
  return sum;
}

/* lambda*pi of the reference (QCalculator.h:163): lambda = 2/(3+sqrt 2). */
double edbo_lambda(void) { return 2. / (3. + sqrt(2.)) * M_PI; }

/* rval = 4 pi (2 lambda / pi * R / N)^(3+gamma), QCalculator.h:176, with the
 * reference's hard-coded R = 6.62132 generalised to the box half-width R. */
double edbo_rval(int N, double gamma, double R) {
  double lambda = edbo_lambda();
  return (4. * M_PI) * pow(2. * lambda / M_PI * R / N, 3 + gamma);
}

/* Largest |l+m|^2 or |l-m|^2 over the modes of either index mode. */
int edbo_amax(int N) {
  int n = (N - 1) / 2;
  int hi = 2 * (N - 1 - n); /* |l_i + m_i| <= 2 max(n, N-1-n) */
  if (N - 1 > hi) hi = N - 1;
  return 3 * hi * hi;
}

/* F(sqrt(a) lambda pi, sqrt(b) lambda pi) for integer squared norms a, b,
 * memoised; identical values to evaluating funF on xi = calXi(...) because
 * calXi is r_type(sqrt(int)) * lambda (QCalculator.h:165-167). */
typedef struct {
  int amax;
  double gamma;
  double *tab;
} ftab_t;

static int is_closed(double gamma) { return gamma == 0.0 || gamma == 1.0; }

static double ftab_get(ftab_t *t, int a, int b) {
  double *slot = &t->tab[(long)a * (t->amax + 1) + b];
  if (isnan(*slot)) {
    double lambda = edbo_lambda();
    double xi = (double)sqrt((double)a) * lambda;
    double eta = (double)sqrt((double)b) * lambda;
    *slot = is_closed(t->gamma) ? edbo_funF((int)t->gamma, xi, eta)
                                : edbo_funF_quad(t->gamma, xi, eta);
  }
  return *slot;
}

static int ftab_init(ftab_t *t, int N, double gamma) {
  t->amax = edbo_amax(N);
  t->gamma = gamma;
  long sz = (long)(t->amax + 1) * (t->amax + 1);
  t->tab = (double *)malloc(sizeof(double) * sz);
  if (!t->tab) return -1;
  for (long i = 0; i < sz; ++i) t->tab[i] = NAN;
  return 0;
}

static double calfil(int N, int x1, int x2, int x3) {
  return edbo_filtering(N, x1) * edbo_filtering(N, x2) * edbo_filtering(N, x3);
}

/* genB, QCalculator.h:158-229.
 * mode REFERENCE: the literal loops, including the (2n+1)^3 extent of the Bmm
 *   loop (:181-183) against the N^3 row stride used at :219 — identical to the
 *   aliased table for odd N, scrambled for even N exactly as the reference is.
 * mode ALIASED: modes c - n, c in [0,N), m = k - l wrapped once into
 *   [-n, N-1-n]; Bmm over all N^3 modes.
 * B is row-major [l][k] over centred indices, N^3 x N^3 doubles. */
int edbo_genB(int N, double gamma, double R, int filter, int mode, double *B) {
  const int n = (N - 1) / 2;
  const long NQ = (long)N * N * N;
  const double rval = edbo_rval(N, gamma, R);
  ftab_t ft;
  if (ftab_init(&ft, N, gamma)) return -1;
  double *Bmm = (double *)calloc(NQ, sizeof(double));
  if (!Bmm) {
    free(ft.tab);
    return -1;
  }
  double fil_val = 1.0;
  if (mode == EDBO_INDEX_REFERENCE) {
    long ibm = 0;
    for (int k1 = -n; k1 < n + 1; ++k1)
      for (int k2 = -n; k2 < n + 1; ++k2)
        for (int k3 = -n; k3 < n + 1; ++k3) {
          int a = (2 * k1) * (2 * k1) + (2 * k2) * (2 * k2) + (2 * k3) * (2 * k3);
          if (filter) fil_val = calfil(N, k1, k2, k3);
          Bmm[ibm++] = ftab_get(&ft, a, 0) * fil_val * fil_val * rval;
        }
  } else {
    long ibm = 0;
    for (int k1 = -n; k1 < N - n; ++k1)
      for (int k2 = -n; k2 < N - n; ++k2)
        for (int k3 = -n; k3 < N - n; ++k3) {
          int a = (2 * k1) * (2 * k1) + (2 * k2) * (2 * k2) + (2 * k3) * (2 * k3);
          if (filter) fil_val = calfil(N, k1, k2, k3);
          Bmm[ibm++] = ftab_get(&ft, a, 0) * fil_val * fil_val * rval;
        }
  }
  /* The main loop is the same for both modes: with centred indices c in [0,N)
   * the reference's m_i = k_i - l_i + n wrapped into [0, N) (:204-218) is the
   * centred index of m = k - l wrapped into [-n, N-1-n]. */
  double *sig = (double *)malloc(sizeof(double) * N);
  for (int c = 0; c < N; ++c) sig[c] = edbo_filtering(N, c - n);
  double sigmal = 1.0, sigmam = 1.0;
  long ib = 0;
  for (int l1 = 0; l1 < N; ++l1)
    for (int l2 = 0; l2 < N; ++l2)
      for (int l3 = 0; l3 < N; ++l3) {
        if (filter) sigmal = sig[l1] * sig[l2] * sig[l3];
        for (int k1 = 0; k1 < N; ++k1) {
          int m1 = k1 - l1 + n;
          if (m1 < 0)
            m1 += N;
          else if (m1 > N - 1)
            m1 -= N;
          int xi1 = l1 - n + m1 - n, eta1 = l1 - m1;
          for (int k2 = 0; k2 < N; ++k2) {
            int m2 = k2 - l2 + n;
            if (m2 < 0)
              m2 += N;
            else if (m2 > N - 1)
              m2 -= N;
            int xi2 = l2 - n + m2 - n, eta2 = l2 - m2;
            for (int k3 = 0; k3 < N; ++k3) {
              int m3 = k3 - l3 + n;
              if (m3 < 0)
                m3 += N;
              else if (m3 > N - 1)
                m3 -= N;
              long m = ((long)m1 * N + m2) * N + m3;
              int xi3 = l3 - n + m3 - n, eta3 = l3 - m3;
              int a = xi1 * xi1 + xi2 * xi2 + xi3 * xi3;
              int b = eta1 * eta1 + eta2 * eta2 + eta3 * eta3;
              if (filter) sigmam = sig[m1] * sig[m2] * sig[m3];
              B[ib++] = ftab_get(&ft, a, b) * sigmal * sigmam * rval - Bmm[m];
            }
          }
        }
      }
  free(sig);
  free(Bmm);
  free(ft.tab);
  return 0;
}

/* number of terms one calQ evaluates: N^3 (2n+1)^3 (reference), N^6 (aliased) */
long edbo_terms(int N, int mode) {
  long NQ = (long)N * N * N;
  if (mode == EDBO_INDEX_ALIASED) return NQ * NQ;
  long P = 2 * ((N - 1) / 2) + 1;
  return NQ * P * P * P;
}

/* calQ, QCalculator.h:231-257 with transf (:108-123) and convertQ (:144-155).
 * mode REFERENCE: the literal loops — f doubled to (2N)^3, l over [n+1, N+n]^3,
 *   k over (2n+1)^3 starting at 3n+2-l, B consumed sequentially (m++), Q of
 *   N^3 entries filled over its first (2n+1)^3, then convertQ.
 * mode ALIASED: Q_k = sum_l f_l f_((k-l) wrapped) B[l][k] over all N^3 x N^3
 *   pairs with centred indices; identical operation sequence to REFERENCE for
 *   odd N. */
int edbo_calQ(int N, int mode, const double *B, const double *fin, double *Qout) {
  const int n = (N - 1) / 2;
  const long NQ = (long)N * N * N;
  double *Q = (double *)calloc(2 * NQ, sizeof(double));
  if (!Q) return -1;
  if (mode == EDBO_INDEX_REFERENCE) {
    const int N2 = 2 * N;
    double *f = (double *)malloc(sizeof(double) * 2 * 8 * NQ);
    if (!f) {
      free(Q);
      return -1;
    }
    long k = 0;
    for (int k1 = 0; k1 < N2; ++k1) {
      int kin1 = (k1 < N) ? k1 : k1 - N;
      for (int k2 = 0; k2 < N2; ++k2) {
        int kin2 = (k2 < N) ? k2 : k2 - N;
        for (int k3 = 0; k3 < N2; ++k3) {
          int kin3 = (k3 < N) ? k3 : k3 - N;
          long kin = ((long)kin1 * N + kin2) * N + kin3;
          f[2 * k] = fin[2 * kin];
          f[2 * k + 1] = fin[2 * kin + 1];
          ++k;
        }
      }
    }
    long m = 0;
    for (int l1 = n + 1; l1 < N + n + 1; ++l1)
      for (int l2 = n + 1; l2 < N + n + 1; ++l2)
        for (int l3 = n + 1; l3 < N + n + 1; ++l3) {
          long kq = 0;
          long l = ((long)l1 * N2 + l2) * N2 + l3;
          const double fr = f[2 * l], fi = f[2 * l + 1];
          for (int k1 = 3 * n + 2 - l1; k1 < 5 * n + 3 - l1; ++k1)
            for (int k2 = 3 * n + 2 - l2; k2 < 5 * n + 3 - l2; ++k2)
              for (int k3 = 3 * n + 2 - l3; k3 < 5 * n + 3 - l3; ++k3) {
                long kl = ((long)k1 * N2 + k2) * N2 + k3;
                const double gr = f[2 * kl], gi = f[2 * kl + 1];
                const double pr = fr * gr - fi * gi;
                const double pi = fr * gi + fi * gr;
                const double bb = B[m++];
                Q[2 * kq] += pr * bb;
                Q[2 * kq + 1] += pi * bb;
                ++kq;
              }
        }
    free(f);
  } else {
    int *cidx = (int *)malloc(sizeof(int) * N); /* centred index -> FFTW index */
    for (int c = 0; c < N; ++c) {
      int fr = c - n;
      cidx[c] = fr >= 0 ? fr : fr + N;
    }
    long m = 0;
    for (int l1 = 0; l1 < N; ++l1)
      for (int l2 = 0; l2 < N; ++l2)
        for (int l3 = 0; l3 < N; ++l3) {
          long li = ((long)cidx[l1] * N + cidx[l2]) * N + cidx[l3];
          const double fr = fin[2 * li], fi = fin[2 * li + 1];
          long kq = 0;
          for (int k1 = 0; k1 < N; ++k1) {
            int m1 = k1 - l1 + n;
            if (m1 < 0) m1 += N;
            else if (m1 > N - 1) m1 -= N;
            for (int k2 = 0; k2 < N; ++k2) {
              int m2 = k2 - l2 + n;
              if (m2 < 0) m2 += N;
              else if (m2 > N - 1) m2 -= N;
              for (int k3 = 0; k3 < N; ++k3) {
                int m3 = k3 - l3 + n;
                if (m3 < 0) m3 += N;
                else if (m3 > N - 1) m3 -= N;
                long mi = ((long)cidx[m1] * N + cidx[m2]) * N + cidx[m3];
                const double gr = fin[2 * mi], gi = fin[2 * mi + 1];
                const double pr = fr * gr - fi * gi;
                const double pi = fr * gi + fi * gr;
                const double bb = B[m++];
                Q[2 * kq] += pr * bb;
                Q[2 * kq + 1] += pi * bb;
                ++kq;
              }
            }
          }
        }
    /* centred -> FFTW order with the same mode convention as the input */
    long kq = 0;
    for (int k1 = 0; k1 < N; ++k1)
      for (int k2 = 0; k2 < N; ++k2)
        for (int k3 = 0; k3 < N; ++k3) {
          long ko = ((long)cidx[k1] * N + cidx[k2]) * N + cidx[k3];
          Qout[2 * ko] = Q[2 * kq];
          Qout[2 * ko + 1] = Q[2 * kq + 1];
          ++kq;
        }
    free(cidx);
    free(Q);
    return 0;
  }
  /* convertQ (:144-155): centred (stride-N) index -> FFTW order */
  long k = 0;
  for (int k1 = 0; k1 < N; ++k1) {
    int kq1 = (k1 < n + 1) ? k1 + n : k1 - (n + 1);
    for (int k2 = 0; k2 < N; ++k2) {
      int kq2 = (k2 < n + 1) ? k2 + n : k2 - (n + 1);
      for (int k3 = 0; k3 < N; ++k3) {
        int kq3 = (k3 < n + 1) ? k3 + n : (k3 - n - 1);
        long kq = ((long)kq1 * N + kq2) * N + kq3;
        Qout[2 * k] = Q[2 * kq];
        Qout[2 * k + 1] = Q[2 * kq + 1];
        ++k;
      }
    }
  }
  free(Q);
  return 0;
}

/* Direct O(N^6) aliased evaluation with the kernel computed in frequency
 * space per term, without any B table: Q_k = sum_l f_l f_m [F(l+m, l-m)
 * sigma(l) sigma(m) - F(2m, 0) sigma(m)^2] rval, m = k - l wrapped into
 * [-n, N-1-n].  The idea of an independent direct evaluator follows
 * oldTest/calBBox.h:332-371; the kernel is that of QCalculator.h:181-224.
 * Accumulation order differs from calQ (it runs over k outer, l inner). */
/* One output mode K (modes in [-n, N-1-n]) of the direct evaluation. */
static void direct_one(int N, int n, double rval, ftab_t *ft, const double *sig, const double *fin,
                       int K1, int K2, int K3, double *qr_out, double *qi_out) {
  double qr = 0.0, qi = 0.0;
  for (int L1 = -n; L1 < N - n; ++L1)
    for (int L2 = -n; L2 < N - n; ++L2)
      for (int L3 = -n; L3 < N - n; ++L3) {
        int M[3] = {K1 - L1, K2 - L2, K3 - L3};
        int L[3] = {L1, L2, L3};
        for (int d = 0; d < 3; ++d) {
          if (M[d] < -n) M[d] += N;
          else if (M[d] > N - 1 - n) M[d] -= N;
        }
        int a = 0, b = 0, a2 = 0;
        double sl = 1.0, sm = 1.0;
        long li = 0, mi = 0;
        for (int d = 0; d < 3; ++d) {
          a += (L[d] + M[d]) * (L[d] + M[d]);
          b += (L[d] - M[d]) * (L[d] - M[d]);
          a2 += 4 * M[d] * M[d];
          sl *= sig[L[d] + n];
          sm *= sig[M[d] + n];
          li = li * N + (L[d] >= 0 ? L[d] : L[d] + N);
          mi = mi * N + (M[d] >= 0 ? M[d] : M[d] + N);
        }
        double beta = ftab_get(ft, a, b) * sl * sm * rval - ftab_get(ft, a2, 0) * sm * sm * rval;
        double fr = fin[2 * li], fi = fin[2 * li + 1];
        double gr = fin[2 * mi], gi = fin[2 * mi + 1];
        qr += (fr * gr - fi * gi) * beta;
        qi += (fr * gi + fi * gr) * beta;
      }
  *qr_out = qr;
  *qi_out = qi;
}

int edbo_direct(int N, double gamma, double R, int filter, const double *fin, double *Qout) {
  const int n = (N - 1) / 2;
  const double rval = edbo_rval(N, gamma, R);
  ftab_t ft;
  if (ftab_init(&ft, N, gamma)) return -1;
  double *sig = (double *)malloc(sizeof(double) * N);
  for (int c = 0; c < N; ++c) sig[c] = filter ? edbo_filtering(N, c - n) : 1.0;
  for (int K1 = -n; K1 < N - n; ++K1)
    for (int K2 = -n; K2 < N - n; ++K2)
      for (int K3 = -n; K3 < N - n; ++K3) {
        long ko = ((long)(K1 >= 0 ? K1 : K1 + N) * N + (K2 >= 0 ? K2 : K2 + N)) * N +
                  (K3 >= 0 ? K3 : K3 + N);
        direct_one(N, n, rval, &ft, sig, fin, K1, K2, K3, &Qout[2 * ko], &Qout[2 * ko + 1]);
      }
  free(sig);
  free(ft.tab);
  return 0;
}

/* The direct evaluation at nk chosen output modes, given by FFTW flat index
 * (kidx), so large N can be checked without the N^6 table: O(nk N^3). */
int edbo_direct_modes(int N, double gamma, double R, int filter, const double *fin, int nk,
                      const long *kidx, double *Qout) {
  const int n = (N - 1) / 2;
  const double rval = edbo_rval(N, gamma, R);
  ftab_t ft;
  if (ftab_init(&ft, N, gamma)) return -1;
  double *sig = (double *)malloc(sizeof(double) * N);
  for (int c = 0; c < N; ++c) sig[c] = filter ? edbo_filtering(N, c - n) : 1.0;
  for (int j = 0; j < nk; ++j) {
    const long k = kidx[j];
    int kf[3] = {(int)(k / ((long)N * N)), (int)((k / N) % N), (int)(k % N)};
    int K[3];
    for (int d = 0; d < 3; ++d) K[d] = kf[d] > N - 1 - n ? kf[d] - N : kf[d];
    direct_one(N, n, rval, &ft, sig, fin, K[0], K[1], K[2], &Qout[2 * j], &Qout[2 * j + 1]);
  }
  free(sig);
  free(ft.tab);
  return 0;
}

/* Independent solves spread over host threads (the reference itself is
 * single-threaded; this is the all-cores CPU baseline). */
typedef struct {
  int N, mode, S, nthreads, tid, rc;
  const double *B, *fin;
  double *Qout;
} batch_arg_t;

static void *batch_worker(void *p) {
  batch_arg_t *a = (batch_arg_t *)p;
  long NQ = (long)a->N * a->N * a->N;
  a->rc = 0;
  for (int s = a->tid; s < a->S; s += a->nthreads)
    a->rc |= edbo_calQ(a->N, a->mode, a->B, a->fin + 2 * NQ * s, a->Qout + 2 * NQ * s);
  return NULL;
}

int edbo_calQ_batch_mt(int N, int mode, const double *B, int S, const double *fin,
                       double *Qout, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > S) nthreads = S;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
  batch_arg_t *args = (batch_arg_t *)malloc(sizeof(batch_arg_t) * nthreads);
  for (int t = 0; t < nthreads; ++t) {
    batch_arg_t a = {N, mode, S, nthreads, t, 0, B, fin, Qout};
    args[t] = a;
    pthread_create(&th[t], NULL, batch_worker, &args[t]);
  }
  int rc = 0;
  for (int t = 0; t < nthreads; ++t) {
    pthread_join(th[t], NULL);
    rc |= args[t].rc;
  }
  free(th);
  free(args);
  return rc;
}

/* -------------------------------------------------------------- transforms */

/* One axis of the unnormalised DFT, in place; the same summation as the
 * FFTW-API shim used to compile the reference (oracle/fftw_shim/fftw3.h). */
static void dft_axis(double *buf, const int *nn, int axis, int sign) {
  const int len = nn[axis];
  long stride = 1;
  for (int a = axis + 1; a < 3; ++a) stride *= nn[a];
  long total = (long)nn[0] * nn[1] * nn[2];
  double *tw = (double *)malloc(sizeof(double) * 2 * len);
  const double two_pi = 8.0 * atan(1.0);
  for (int r = 0; r < len; ++r) {
    tw[2 * r] = cos(two_pi * r / len);
    tw[2 * r + 1] = sign * sin(two_pi * r / len);
  }
  double *line = (double *)malloc(sizeof(double) * 2 * len);
  for (long base = 0; base < total; ++base) {
    if ((base / stride) % len != 0) continue;
    for (int j = 0; j < len; ++j) {
      line[2 * j] = buf[2 * (base + j * stride)];
      line[2 * j + 1] = buf[2 * (base + j * stride) + 1];
    }
    for (int k = 0; k < len; ++k) {
      double sr = 0.0, si = 0.0;
      for (int j = 0; j < len; ++j) {
        int r = (int)(((long)j * k) % len);
        double c = tw[2 * r], s = tw[2 * r + 1];
        sr += line[2 * j] * c - line[2 * j + 1] * s;
        si += line[2 * j] * s + line[2 * j + 1] * c;
      }
      buf[2 * (base + k * stride)] = sr;
      buf[2 * (base + k * stride) + 1] = si;
    }
  }
  free(line);
  free(tw);
}

/* fft3d::fft (fft3d.h:25-30): FFTW_FORWARD, unnormalised.
 * fft3d::ifft (fft3d.h:32-48): FFTW_BACKWARD then every element times 1./N
 * (the reference's loop bounds use Ny for the third axis, :43; cubes only). */
void edbo_fft3d(int nx, int ny, int nz, const double *in, double *out, int inverse) {
  int nn[3] = {nx, ny, nz};
  long total = (long)nx * ny * nz;
  memmove(out, in, sizeof(double) * 2 * total);
  for (int axis = 0; axis < 3; ++axis) dft_axis(out, nn, axis, inverse ? +1 : -1);
  if (inverse) {
    int Nn = nx * ny * nz;
    long k = 0;
    for (int i = 0; i < nx; ++i)
      for (int j = 0; j < ny; ++j)
        for (int l = 0; l < ny; ++l) {
          out[2 * k] *= 1. / Nn;
          out[2 * k + 1] *= 1. / Nn;
          ++k;
        }
  }
}

/* ------------------------------------------------------------- entropy fix */

/* EntropyFix(Nt, eps), EntropyFix.h:29-32 (Averagef = 1, flag false, :20-22). */
void edbo_efix_init(edbo_efix *e, int Nt, double eps) {
  e->Nt = Nt;
  e->eps = eps;
  e->avg = 1.0;
  e->avg_flag = 0;
}

/* setAverage(Nf, f), EntropyFix.h:65-78: sequential sum / Nf, latched. */
void edbo_efix_setaverage(edbo_efix *e, int Nf, const double *f) {
  e->avg_flag = 1;
  e->avg = 0.;
  for (int i = 0; i < Nf; ++i) e->avg += f[i];
  e->avg /= (double)Nf;
}

/* EntropyCal(Nf, f), EntropyFix.h:124-161 (the non-MKL branch):
 * (sum over f_i > eps of f_i log f_i) / Nf - Averagef. */
double edbo_efix_entropy(edbo_efix *e, int Nf, const double *f) {
  double res = 0.0;
  if (!e->avg_flag) edbo_efix_setaverage(e, Nf, f);
  for (int i = 0; i < Nf; i++)
    if (f[i] > e->eps) res += f[i] * log(f[i]);
  res = res / (double)Nf - e->avg;
  return res;
}

/* FixSol(Nf, f, aim), EntropyFix.h:211-253: bisection on beta in [0,1] for
 * f_beta = (1-beta) f + beta * Averagef, early exit when 0 < aim - H < eps,
 * otherwise f <- f_betaR. */
int edbo_efix_fixsol(edbo_efix *e, int Nf, double *f, double aim) {
  double *fMid = (double *)malloc(sizeof(double) * e->Nt);
  if (!fMid) return -1;
  double betaL = 0.0, betaR = 1.0, betaMid, entMid, betaFbar;
  double BiEps = e->eps;
  while ((betaR - betaL) > BiEps) {
    betaMid = 0.5 * (betaL + betaR);
    if (!e->avg_flag) edbo_efix_setaverage(e, Nf, f);
    betaFbar = betaMid * e->avg;
    for (int i = 0; i < e->Nt; i++) fMid[i] = betaFbar;
    for (int i = 0; i < Nf; ++i) fMid[i] += (1. - betaMid) * f[i];
    entMid = edbo_efix_entropy(e, e->Nt, fMid);
    if ((entMid < aim) && ((aim - entMid) < e->eps)) {
      for (int i = 0; i < Nf; ++i) f[i] = fMid[i];
      free(fMid);
      return 0;
    }
    if (entMid < aim)
      betaR = betaMid;
    else
      betaL = betaMid;
  }
  betaFbar = betaR * e->avg;
  for (int i = 0; i < Nf; ++i) f[i] *= (1.0 - betaR);
  for (int i = 0; i < Nf; i++) f[i] += betaFbar;
  free(fMid);
  return 0;
}

/* ------------------------------------------------------------ BKW3D pieces */

/* BKW3D::funExact live branch (BKW.h:96-112): a synthetic sinusoid. */
double edbo_funexact_sinusoid(double R, double x, double y, double z) {
  double r1 = (x + R) / (2. * R);
  double r2 = (y + R) / (2. * R);
  double r3 = (z + R) / (2. * R);
  double val = 3.2;
  for (int j = 0; j < 11; ++j)
    val += fabs((double)j) / 55 * sin(j * (r1 - 0.5) * M_PI) +
           fabs((double)j) / 55. * sin(j * (r2 - 0.5) * M_PI) +
           fabs((double)j) / 55. * sin(j * (r3 - 0.5) * M_PI);
  return val;
}

/* BKW3D::setInitialValue (BKW.h:121-138): grid x_i = -R + i h, h = 2R/N. */
void edbo_initial_sinusoid(int N, double R, double *F) {
  double h = 2 * R / (double)N;
  long l = 0;
  for (int i = 0; i < N; ++i) {
    double x = -R + i * h;
    for (int j = 0; j < N; ++j) {
      double y = -R + j * h;
      for (int k = 0; k < N; ++k) {
        double z = -R + k * h;
        F[2 * l] = edbo_funexact_sinusoid(R, x, y, z);
        F[2 * l + 1] = 0.0;
        ++l;
      }
    }
  }
}

/* BKW exact solution, BKW.h:114-116 / testfft.cpp:11-16, as a function of
 * s = K(t): f = (2 pi s)^(-3/2) exp(-v^2 / 2s) ((5s-3)/(2s) + (1-s) v^2 / (2 s^2)). */
double edbo_bkw_f(double s, double v2) {
  return 1. / pow(2. * M_PI * s, 1.5) * exp(-v2 / (2. * s)) *
         ((5. * s - 3.) / (2. * s) + (1. - s) / (2. * s * s) * v2);
}

/* d f / d s of the BKW solution (analytic derivative of edbo_bkw_f). */
double edbo_bkw_dfds(double s, double v2) {
  double P = 1. / pow(2. * M_PI * s, 1.5) * exp(-v2 / (2. * s));
  double G = (5. * s - 3.) / (2. * s) + (1. - s) / (2. * s * s) * v2;
  double dP = -1.5 / s + v2 / (2. * s * s);
  double dG = 1.5 / (s * s) - v2 / (s * s * s) + v2 / (2. * s * s);
  return P * (dP * G + dG);
}

/* Samples real values (N^3, row-major) into an interleaved complex array. */
void edbo_grid_real(int N, double R, const double *vals, double *F) {
  (void)R;
  long NQ = (long)N * N * N;
  for (long i = 0; i < NQ; ++i) {
    F[2 * i] = vals[i];
    F[2 * i + 1] = 0.0;
  }
}

/* BKW solution with s = K on the reference grid (BKW.h:124-133). */
void edbo_initial_bkw(int N, double R, double s, double *F) {
  double h = 2 * R / (double)N;
  long l = 0;
  for (int i = 0; i < N; ++i) {
    double x = -R + i * h;
    for (int j = 0; j < N; ++j) {
      double y = -R + j * h;
      for (int k = 0; k < N; ++k) {
        double z = -R + k * h;
        F[2 * l] = edbo_bkw_f(s, x * x + y * y + z * z);
        F[2 * l + 1] = 0.0;
        ++l;
      }
    }
  }
}

/* BKW3D::calEntropy / flogf (BKW.h:140-161). */
double edbo_calentropy(int N, double R, const double *F) {
  long N3d = (long)N * N * N;
  double entropy = 0;
  for (long i = 0; i < N3d; ++i) {
    double f = F[2 * i];
    double val;
    if (fabs(f) < 1.0e-6)
      val = 0.;
    else
      val = f * log(f) - f;
    entropy += val;
  }
  entropy *= pow(2 * R, 3.) / (double)N3d;
  return entropy;
}

/* mass, momentum (3), energy of Re F on the reference grid:
 * h^3 sum f, h^3 sum f v, h^3 sum f |v|^2 / 2.  (Not in the reference; used
 * for the conservation checks.) */
void edbo_moments(int N, double R, const double *F, double *out5) {
  double h = 2 * R / (double)N;
  double m = 0, p1 = 0, p2 = 0, p3 = 0, e = 0;
  long l = 0;
  for (int i = 0; i < N; ++i) {
    double x = -R + i * h;
    for (int j = 0; j < N; ++j) {
      double y = -R + j * h;
      for (int k = 0; k < N; ++k) {
        double z = -R + k * h;
        double f = F[2 * l];
        m += f;
        p1 += f * x;
        p2 += f * y;
        p3 += f * z;
        e += 0.5 * f * (x * x + y * y + z * z);
        ++l;
      }
    }
  }
  double h3 = h * h * h;
  out5[0] = m * h3;
  out5[1] = p1 * h3;
  out5[2] = p2 * h3;
  out5[3] = p3 * h3;
  out5[4] = e * h3;
}

/* ------------------------------------------------------------- integrators */

static void axpy_c(long n, double *y, const double *x, double a, const double *z) {
  /* y = x + a * z  (complex arrays, real a) */
  for (long i = 0; i < n; ++i) {
    y[2 * i] = x[2 * i] + a * z[2 * i];
    y[2 * i + 1] = x[2 * i + 1] + a * z[2 * i + 1];
  }
}

/* Fix step shared by FEuler/CFE/SSP3/RK4 (BKW.h:229-235, 294-305, 432-440,
 * 502-510): F <- FixSol(Re F, H_prev / (2R)^3) with zero imaginary part. */
static void apply_fix(int N, double R, edbo_efix *ef, double *F, double *Ftmp,
                      double entropy0) {
  long N3d = (long)N * N * N;
  for (long i = 0; i < N3d; ++i) Ftmp[i] = F[2 * i];
  edbo_efix_fixsol(ef, (int)N3d, Ftmp, entropy0 / (pow(2 * R, 3)));
  for (long i = 0; i < N3d; ++i) {
    F[2 * i] = Ftmp[i];
    F[2 * i + 1] = 0.0;
  }
}

/* One full reference run (BKW.h:191-633).  The initial real-space data is F0
 * (N^3 complex) or, when F0 is NULL, the sinusoid of setInitialValue(T0).  The
 * kernel table is genB(N, gamma, Rb, filter, mode); the reference itself always
 * uses gamma 0, Rb 6.62132, filter on (BKW.h:201,264,324,397,462,532).  The
 * entropy after each step (before and after the fix) is recorded. */
int edbo_run(int N, double R, int scheme, int mode, double gamma, double Rb, int filter,
             double T0, double TEnd, double dt, double beta, int fix_flag, const double *F0,
             double *Fhat_out, double *F_out, double *ent_raw, double *ent_fixed,
             int trace_cap, int *nsteps) {
  const long N3d = (long)N * N * N;
  double *F = (double *)malloc(sizeof(double) * 2 * N3d);
  double *Fhat = (double *)malloc(sizeof(double) * 2 * N3d);
  double *Q = (double *)malloc(sizeof(double) * 2 * N3d * 4);
  double *F1 = (double *)malloc(sizeof(double) * 2 * N3d * 3);
  double *Ftmp = (double *)malloc(sizeof(double) * N3d);
  double *B = (double *)malloc(sizeof(double) * N3d * N3d);
  if (!F || !Fhat || !Q || !F1 || !Ftmp || !B) return -1;
  double *Q1 = Q + 2 * N3d, *Q2 = Q + 4 * N3d, *Q3 = Q + 6 * N3d;
  double *F2 = F1 + 2 * N3d, *F3 = F1 + 4 * N3d;
  if (F0)
    memcpy(F, F0, sizeof(double) * 2 * N3d);
  else
    edbo_initial_sinusoid(N, R, F);
  edbo_fft3d(N, N, N, F, Fhat, 0);
  edbo_genB(N, gamma, Rb, filter, mode, B);
  edbo_efix ef;
  edbo_efix_init(&ef, (int)N3d, 1.0e-10);

  double t = T0, entropy, entropy0 = 1.;
  int step = 0, rec = 0;
  if (scheme == EDBO_FE) {
    entropy0 = edbo_calentropy(N, R, F);
    step = 1;
  }
  double *Fold = NULL;
  if (scheme == EDBO_DUFORT) {
    Fold = (double *)malloc(sizeof(double) * 2 * N3d);
    memcpy(Fold, Fhat, sizeof(double) * 2 * N3d);
  }
  int phase = (scheme == EDBO_DUFORT) ? 0 : 1;
  double dtRK2 = dt / 8;
  for (;;) {
    if (scheme == EDBO_DUFORT && phase == 0)
      t += dtRK2;
    else
      t += dt;
    switch (scheme) {
      case EDBO_FE: /* BKW.h:219-222 */
        edbo_calQ(N, mode, B, Fhat, Q);
        axpy_c(N3d, Fhat, Fhat, dt, Q);
        break;
      case EDBO_CFE: /* BKW.h:280-283 */
        edbo_calQ(N, mode, B, Fhat, Q);
        axpy_c(N3d, Fhat, Fhat, (1. - exp(-beta * dt)) / beta, Q);
        break;
      case EDBO_RK2: /* BKW.h:340-346 */
        edbo_calQ(N, mode, B, Fhat, Q);
        axpy_c(N3d, F1, Fhat, 0.5 * dt, Q);
        edbo_calQ(N, mode, B, F1, Q);
        axpy_c(N3d, Fhat, Fhat, dt, Q);
        break;
      case EDBO_SSP3: /* BKW.h:415-424 */
        edbo_calQ(N, mode, B, Fhat, Q);
        axpy_c(N3d, F1, Fhat, dt, Q);
        edbo_calQ(N, mode, B, F1, Q);
        for (long l = 0; l < 2 * N3d; ++l) F2[l] = 0.75 * Fhat[l] + 0.25 * F1[l] + 0.25 * dt * Q[l];
        edbo_calQ(N, mode, B, F2, Q);
        for (long l = 0; l < 2 * N3d; ++l)
          Fhat[l] = Fhat[l] / 3. + 2. * F2[l] / 3. + 2. / 3. * dt * Q[l];
        break;
      case EDBO_RK4: /* BKW.h:481-494 */
        edbo_calQ(N, mode, B, Fhat, Q);
        axpy_c(N3d, F1, Fhat, 0.5 * dt, Q);
        edbo_calQ(N, mode, B, F1, Q1);
        axpy_c(N3d, F2, Fhat, 0.5 * dt, Q1);
        edbo_calQ(N, mode, B, F2, Q2);
        axpy_c(N3d, F3, Fhat, dt, Q2);
        edbo_calQ(N, mode, B, F3, Q3);
        for (long l = 0; l < 2 * N3d; ++l)
          Fhat[l] = Fhat[l] + dt / 6. * (Q[l] + 2. * Q1[l] + 2. * Q2[l] + Q3[l]);
        break;
      case EDBO_DUFORT:
        if (phase == 0) { /* BKW.h:550-556 (RK2 start-up with dt, not dt/8) */
          edbo_calQ(N, mode, B, Fhat, Q);
          axpy_c(N3d, F1, Fhat, 0.5 * dt, Q);
          edbo_calQ(N, mode, B, F1, Q);
          axpy_c(N3d, Fhat, Fhat, dt, Q);
        } else { /* BKW.h:595-598 */
          edbo_calQ(N, mode, B, Fhat, Q);
          memcpy(F1, Fhat, sizeof(double) * 2 * N3d);
          for (long l = 0; l < 2 * N3d; ++l)
            Fhat[l] = 1. / (1. + beta * dt) * (F1[l] + dt * Q[l] + beta * dt * (F1[l] - Fold[l]));
        }
        break;
      default:
        return -2;
    }
    edbo_fft3d(N, N, N, Fhat, F, 1);
    entropy = edbo_calentropy(N, R, F);
    double raw = entropy;
    int fix_allowed = 0;
    if (scheme == EDBO_FE)
      fix_allowed = (step > 1) && fix_flag;
    else if (scheme == EDBO_CFE)
      fix_allowed = step && fix_flag;
    else if (scheme == EDBO_SSP3 || scheme == EDBO_RK4)
      fix_allowed = step != 0; /* the flag is not consulted (BKW.h:432, 502) */
    if (fix_allowed && entropy - entropy0 > 1.0e-10) {
      apply_fix(N, R, &ef, F, Ftmp, entropy0);
      entropy = edbo_calentropy(N, R, F);
    }
    if (rec < trace_cap) {
      if (ent_raw) ent_raw[rec] = raw;
      if (ent_fixed) ent_fixed[rec] = entropy;
    }
    ++rec;
    entropy0 = entropy;
    step++;
    if (scheme == EDBO_DUFORT) {
      if (phase == 0) {
        if (!(step < 8)) {
          phase = 1;
          step = 0;
        }
        continue;
      }
      memcpy(Fold, F1, sizeof(double) * 2 * N3d);
    }
    if (!(t < TEnd)) break;
  }
  memcpy(Fhat_out, Fhat, sizeof(double) * 2 * N3d);
  memcpy(F_out, F, sizeof(double) * 2 * N3d);
  if (nsteps) *nsteps = rec;
  free(F);
  free(Fhat);
  free(Q);
  free(F1);
  free(Ftmp);
  free(B);
  free(Fold);
  return 0;
}
