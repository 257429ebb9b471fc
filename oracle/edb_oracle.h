/*
 * edb_oracle — CPU restatement of the reference spectral collision step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path
 * and the timed CPU baseline; nothing in the product links or calls it.
 * It restates, in plain C with double precision, the algorithms of
 *   CalQ/QCalculator.h  (filtering, funF, genB, transf/calQ/convertQ)
 *   CalQ/fft3d.h        (3-D DFT conventions)
 *   CalQ/EntropyFix.h   (EntropyCal, setAverage, FixSol bisection)
 *   CalQ/BKW.h          (initial data, calEntropy, FE/CFE/RK2/SSP3/RK4/DUFORT)
 * of YK2015/EntropyDecreaseBoltzmann, each function citing the lines it follows.
 * It is pinned against the compiled reference (oracle/_ref, where the
 * reference sources exist) and against committed golden vectors
 * (tests/golden/) generated from it.
 *
 * Complex arrays are interleaved (re, im) doubles, row-major [i][j][k] with k
 * fastest, exactly like std::complex<double> / fftw_complex arrays.
 */
#ifndef EDB_ORACLE_H
#define EDB_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* index modes of the collision sum */
#define EDBO_INDEX_REFERENCE 0 /* literal reference loops (QCalculator.h:181-183, 239-253) */
#define EDBO_INDEX_ALIASED 1   /* aliased convolution over modes [-n, N-1-n]^3 */

/* default box half-width hard-coded in the reference's rval (QCalculator.h:176) */
#define EDBO_R_REFERENCE 6.62132

double edbo_filtering(int N, int beta);
double edbo_funF(int alpha, double xi, double eta);
double edbo_funF_quad(double gamma, double xi, double eta);
double edbo_lambda(void);
double edbo_rval(int N, double gamma, double R);
int edbo_amax(int N);
int edbo_genB(int N, double gamma, double R, int filter, int mode, double *B);
int edbo_calQ(int N, int mode, const double *B, const double *fin, double *Qout);
int edbo_direct(int N, double gamma, double R, int filter, const double *fin, double *Qout);
/* edbo_direct at nk output modes given by FFTW flat index; O(nk N^3). */
int edbo_direct_modes(int N, double gamma, double R, int filter, const double *fin, int nk,
                      const long *kidx, double *Qout);
int edbo_calQ_batch_mt(int N, int mode, const double *B, int S, const double *fin,
                       double *Qout, int nthreads);
long edbo_terms(int N, int mode);

void edbo_fft3d(int nx, int ny, int nz, const double *in, double *out, int inverse);

typedef struct {
  int Nt;
  double eps;
  double avg;
  int avg_flag;
} edbo_efix;
void edbo_efix_init(edbo_efix *e, int Nt, double eps);
void edbo_efix_setaverage(edbo_efix *e, int Nf, const double *f);
double edbo_efix_entropy(edbo_efix *e, int Nf, const double *f);
int edbo_efix_fixsol(edbo_efix *e, int Nf, double *f, double aim);

double edbo_funexact_sinusoid(double R, double x, double y, double z);
void edbo_initial_sinusoid(int N, double R, double *F);
double edbo_bkw_f(double s, double v2);
double edbo_bkw_dfds(double s, double v2);
void edbo_grid_real(int N, double R, const double *vals, double *F);
void edbo_initial_bkw(int N, double R, double s, double *F);
double edbo_calentropy(int N, double R, const double *F);
void edbo_moments(int N, double R, const double *F, double *out5);

/* schemes, same numbering as the C ABI */
#define EDBO_FE 0
#define EDBO_CFE 1
#define EDBO_RK2 2
#define EDBO_SSP3 3
#define EDBO_RK4 4
#define EDBO_DUFORT 5

int edbo_run(int N, double R, int scheme, int mode, double gamma, double Rb, int filter,
             double T0, double TEnd, double dt, double beta, int fix_flag, const double *F0,
             double *Fhat_out, double *F_out, double *ent_raw, double *ent_fixed,
             int trace_cap, int *nsteps);

#ifdef __cplusplus
}
#endif
#endif
