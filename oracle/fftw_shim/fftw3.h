/*
 * Minimal FFTW3-API-compatible 3-D complex DFT — ORACLE TEST INFRASTRUCTURE ONLY.
 *
 * FFTW3 is not installed on this machine, and the reference's transform
 * wrapper (CalQ/fft3d.h:15,25-48) includes <fftw3.h>.  This header supplies
 * the handful of documented FFTW3 entry points that wrapper calls, so the
 * reference headers can be compiled unmodified into the oracle library:
 *
 *   fftw_complex, fftw_plan, fftw_plan_dft_3d, fftw_execute,
 *   fftw_destroy_plan, FFTW_FORWARD, FFTW_BACKWARD, FFTW_ESTIMATE.
 *
 * Semantics follow the FFTW3 manual ("What FFTW Really Computes"): an
 * unnormalised multi-dimensional DFT over a row-major array,
 *     out[k] = sum_j in[j] * exp(sign * 2*pi*i * (j0 k0/n0 + j1 k1/n1 + j2 k2/n2)),
 * with sign = FFTW_FORWARD = -1 or FFTW_BACKWARD = +1.  In-place plans are
 * allowed.  The transform is computed axis by axis as a direct O(n) sum per
 * output element, with twiddles exp(2*pi*i*r/n) evaluated from the reduced
 * integer r = (j*k) mod n.  FFTW itself is not pinned by the reference (no
 * version anywhere), so agreement with FFTW is to round-off only.
 */
#ifndef EDB_ORACLE_FFTW3_SHIM_H
#define EDB_ORACLE_FFTW3_SHIM_H

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_MEASURE (0U)

typedef struct edb_shim_plan_s {
  int n[3];
  int sign;
  fftw_complex *in;
  fftw_complex *out;
} *fftw_plan;

static inline fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in,
                                         fftw_complex *out, int sign, unsigned flags) {
  (void)flags;
  fftw_plan p = (fftw_plan)malloc(sizeof(struct edb_shim_plan_s));
  p->n[0] = n0;
  p->n[1] = n1;
  p->n[2] = n2;
  p->sign = sign;
  p->in = in;
  p->out = out;
  return p;
}

/* One axis of the DFT, in place on buf (row-major dims n[0..2]). */
static inline void edb_shim_dft_axis(double *buf, const int *n, int axis, int sign) {
  const int len = n[axis];
  long stride = 1;
  for (int a = axis + 1; a < 3; ++a) stride *= n[a];
  long total = (long)n[0] * n[1] * n[2];
  double *tw = (double *)malloc(sizeof(double) * 2 * len);
  const double two_pi = 8.0 * atan(1.0);
  for (int r = 0; r < len; ++r) {
    tw[2 * r] = cos(two_pi * r / len);
    tw[2 * r + 1] = sign * sin(two_pi * r / len);
  }
  double *line = (double *)malloc(sizeof(double) * 2 * len);
  for (long base = 0; base < total; ++base) {
    /* base must be the first element of a line along `axis` */
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

static inline void fftw_execute(const fftw_plan p) {
  long total = (long)p->n[0] * p->n[1] * p->n[2];
  double *buf = (double *)malloc(sizeof(double) * 2 * total);
  memcpy(buf, p->in, sizeof(double) * 2 * total);
  for (int axis = 0; axis < 3; ++axis) edb_shim_dft_axis(buf, p->n, axis, p->sign);
  memcpy(p->out, buf, sizeof(double) * 2 * total);
  free(buf);
}

static inline void fftw_destroy_plan(fftw_plan p) { free(p); }

#ifdef __cplusplus
}
#endif

#endif /* EDB_ORACLE_FFTW3_SHIM_H */
