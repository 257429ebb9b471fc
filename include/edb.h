/*
 * edb.h — C ABI of libedb.so, the GB300 (sm_103a) spectral collision step.
 *
 * The reference (YK2015/EntropyDecreaseBoltzmann) is header-only C++ with no C
 * ABI; its call surface for this path is the class trio
 *   QCalculator<c_type,r_type>  (CalQ/QCalculator.h:17-62)
 *   fft3d                       (CalQ/fft3d.h:17-49)
 *   EntropyFix<i_type,r_type>   (CalQ/EntropyFix.h:13-46)
 * driven by BKW3D's integrators (CalQ/BKW.h:191-633).  Each entry point below
 * names the reference interface it replaces.  The drop-in C++ headers under
 * entropydecreaseboltzmann_gb300/cpp/ wrap these functions in classes with
 * the reference's names and signatures.
 *
 * Conventions
 *  - Complex arrays are interleaved (re, im) doubles (or floats for the
 *    batched FP32 path), N^3 entries, row-major [i][j][k], k fastest, in FFTW
 *    frequency order — the memory layout of std::complex<double>[N^3] and
 *    fftw_complex[N^3] used by the reference.
 *  - Functions taking host pointers are synchronous.  Functions with a
 *    `_device` suffix take device pointers and a cudaStream_t (passed as
 *    void*, NULL = default stream) and are stream-ordered.
 *  - Every function returns an edb_status; edb_last_error() gives text for
 *    the calling thread's last failure.  The reference has no error codes
 *    (it asserts, EntropyFix.h:127,214).
 *  - Handles are not thread-safe (the reference's classes are not either:
 *    QCalculator::calQ mutates member scratch, QCalculator.h:27-29); use one
 *    handle per host thread.
 *  - There is no CPU fallback: without a usable sm_103a GPU every compute
 *    entry point fails with EDB_ECUDA.
 */
#ifndef EDB_H
#define EDB_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  EDB_OK = 0,
  EDB_EINVAL = 1,     /* bad argument */
  EDB_ENOMEM = 2,     /* device or host allocation failed / over budget */
  EDB_ECUDA = 3,      /* CUDA runtime error, or no usable GPU */
  EDB_ETIMEDOUT = 4,  /* a bounded device wait ran out */
  EDB_ENOTREADY = 5,  /* state not initialised (e.g. calQ before genB) */
  EDB_EBUSY = 6,      /* resource in use (e.g. server slots full) */
  EDB_ENOTFOUND = 7,  /* unknown request id */
  EDB_ECANCELED = 8,  /* the request was cancelled (edb_server_cancel) */
  EDB_ENONFINITE = 9  /* a solve's state became non-finite (NaN or infinity) */
} edb_status;

/* Index modes of the collision sum.
 * REFERENCE: the reference's literal loops (QCalculator.h:181-183, 239-253).
 *   For even N these run (2n+1)^3 = (N-1)^3 columns against an N^3 row
 *   stride, exactly as the reference does.
 * ALIASED: Q_k = sum_l f_l f_((k-l) mod N) beta(l,k) over modes
 *   [-n, N-1-n]^3, n = (N-1)/2; identical to REFERENCE for odd N. */
#define EDB_INDEX_REFERENCE 0
#define EDB_INDEX_ALIASED 1

/* Box half-width hard-coded in the reference's kernel scale
 * (QCalculator.h:176: rval = 4 pi (2 lambda/pi * 6.62132/N)^(3+alpha)). */
#define EDB_R_REFERENCE 6.62132

/* Time integrators of BKW3D (BKW.h:54-59). */
#define EDB_SCHEME_FE 0     /* BKW3D::FEuler, BKW.h:191-251 */
#define EDB_SCHEME_CFE 1    /* BKW3D::CFE,    BKW.h:254-313 */
#define EDB_SCHEME_RK2 2    /* BKW3D::RK2,    BKW.h:314-384 */
#define EDB_SCHEME_SSP3 3   /* BKW3D::SSP3,   BKW.h:387-449 */
#define EDB_SCHEME_RK4 4    /* BKW3D::RK4,    BKW.h:452-519 */
#define EDB_SCHEME_DUFORT 5 /* BKW3D::DUFORT, BKW.h:522-633 */

const char *edb_last_error(void);
const char *edb_status_string(edb_status s);
int edb_version(void);
/* Number of kernels this library has launched since load (all devices). */
long long edb_kernel_launch_count(void);
/* Measured FP32 FMA throughput of the current device in TFLOP/s (a short
 * probe kernel); the denominator of the batched kernel's roofline fraction.
 * No reference counterpart (the reference has no GPU code). */
edb_status edb_measure_fp32_peak(double *tflops);
/* Same with packed fma.rn.f32x2 instructions (two FP32 FMAs each). */
edb_status edb_measure_fp32x2_peak(double *tflops);

/* ------------------------------------------------------------ QCalculator */

/* Constructor arguments of QCalculator(N, alpha) (QCalculator.h:39), plus the
 * generalisations the reference hard-codes: the VHS exponent as a real number
 * (alpha is an int 0/1 there, :31), the box half-width L in rval (:176), the
 * filter switch (closeFilter, :54) and the index mode. */
typedef struct {
  int N;           /* modes per dimension, 3 <= N <= 64 */
  double gamma;    /* VHS exponent; 0 = Maxwell molecules, 1 = hard spheres */
  double L;        /* box half-width used in rval; EDB_R_REFERENCE reproduces the reference */
  int filter;      /* 1 = the reference default (IS_FILTER = 1, :34); 0 = closeFilter() */
  int index_mode;  /* EDB_INDEX_REFERENCE or EDB_INDEX_ALIASED */
} edb_qcalc_desc;

typedef struct edb_qcalc edb_qcalc;

/* Fills the reference defaults for QCalculator(N, alpha): gamma = alpha,
 * L = 6.62132, filter on, REFERENCE index mode. */
edb_status edb_qcalc_desc_init(edb_qcalc_desc *d, int N, int alpha);

/* QCalculator(N, alpha) (QCalculator.h:39-52).  Allocates nothing on the
 * device until genB. */
edb_status edb_qcalc_create(const edb_qcalc_desc *d, edb_qcalc **out);
/* ~QCalculator (QCalculator.h:38). */
edb_status edb_qcalc_destroy(edb_qcalc *q);
/* closeFilter (QCalculator.h:54); call before genB. */
edb_status edb_qcalc_close_filter(edb_qcalc *q);

/* genB (QCalculator.h:158-229) on the device in FP64: the N^3 x N^3 table
 * beta(l, k) (what edb_qcalc_copy_B returns), plus the kernels' own forms:
 * in ALIASED mode (and for odd N) the symmetric pair table
 * beta(l, k) + beta(k - l, k) that lets each Q-hat kernel visit half the
 * l1 planes, as FP32 in FFTW order for the batched path and split into
 * (hi, lo) floats for the double-float FP64 kernel.  gamma outside {0,1}
 * uses Gauss-Legendre quadrature of
 * F_gamma = int_0^1 r^(2+gamma) sinc(xi r) sinc(eta r) dr (ReadMe.md:51). */
edb_status edb_qcalc_genB(edb_qcalc *q);

/* QCalculator::funF(xi, eta) (QCalculator.h:76-106) at n points, evaluated
 * on the device: the closed forms for alpha 0 and 1, 0 for any other alpha
 * (as the reference).  Host arrays, synchronous. */
edb_status edb_funF(int alpha, long long n, const double *xi, const double *eta, double *out);
/* QCalculator::filtering(beta) (QCalculator.h:67-74) of an N-mode
 * calculator at n integer points, on the device.  Host arrays. */
edb_status edb_filtering(int N, long long n, const int *beta, double *out);

/* genB for batched use only (ALIASED mode): builds just the FP32 FFTW-order
 * pair table (4 bytes per entry instead of 8 + 8 + 4), so many tables fit in one
 * HBM budget.  The FP64 calQ entry points then report EDB_ENOTREADY. */
edb_status edb_qcalc_genB_f32(edb_qcalc *q);

/* virtual calQ(Qout, fin) (QCalculator.h:59, 231-257): FP64, host buffers,
 * synchronous.  fin and Qout hold N^3 interleaved complex doubles. */
edb_status edb_qcalc_calQ(edb_qcalc *q, const double *fin, double *Qout);

/* Same as edb_qcalc_calQ on device buffers, stream-ordered. */
edb_status edb_qcalc_calQ_device(edb_qcalc *q, const double *d_fin, double *d_Qout,
                                 void *stream);

/* Batched Q-hat for S independent solves sharing this handle's B table
 * (ALIASED mode only): d_fin / d_Qout hold S x N^3 interleaved complex
 * floats (FFTW order), solve-major.  Complex FP32 arithmetic with
 * compensated (two-sum) accumulation across blocks of the l-sum. */
edb_status edb_qcalc_calQ_batch_f32_device(edb_qcalc *q, int S, const float *d_fin,
                                           float *d_Qout, void *stream);

/* The batched kernel with an explicit variant and chunk count (no reference
 * counterpart; the autotuner and the serving engine choose these).
 * variants 0-4: solves staged as they are; 0/1: 16-solve groups (CTA <= 256
 * threads with the compensated sums in registers / <= 384 threads with them
 * in shared memory); 2: 4-solve groups; 3/4: 4 outputs per thread (2 CTAs
 * per SM / 384 threads).  Variants 5-9 are 0-4 on a solve-pair copy of the
 * input, kept by the handle.  chunks > 1 splits the l1 planes into that many
 * chunks whose compensated sums are added in order in FP64; d_partial
 * (device) then holds chunks x S x N^3 x 16 bytes.  For a given chunk count
 * the result of each solve does not depend on S or the variant.  Without
 * chunks, variants 0-4 on the tensor-copy path (N % 4 == 0) run as one
 * persistent grid of resident CTAs pulling the work items from a queue (a
 * stream-ordered counter, so the call may be recorded into a graph). */
edb_status edb_qcalc_calQ_batch_f32_ex(edb_qcalc *q, int S, int variant, int chunks,
                                       void *d_partial, const float *d_fin, float *d_Qout,
                                       void *stream);
/* Number of batched-kernel variants (valid variant arguments are 0 .. n-1). */
int edb_qcalc_batch_variants(void);

/* FP64 collision sum that allocates nothing, for callers that may not call
 * cudaMalloc (a host that owns a fixed device pool and accounts for every
 * byte, a plugin inside such a host, a real-time loop that cannot take
 * cudaMalloc's implicit synchronisation).  No counterpart in the reference.
 * The caller passes the FP64 table d_B (N^3 x N^3 doubles, the layout genB
 * produces; see edb_qcalc_copy_B), d_fin and d_Qout (N^3 complex doubles each,
 * FFTW order); the result agrees with edb_qcalc_calQ_device's to 1e-12
 * relative L2 (it runs the native-FP64 kernel on the full table, the handle
 * path by default the double-float kernel, in another summation order).  The
 * partial sums live in one fixed 5 MiB device array per device, which every
 * GPU that loads the library holds until exit; N must be in [3, 64].  The
 * first call on a device (and the first after its primary context was reset)
 * looks up that array's address, so make it before any stream capture.
 * Calls that overlap on the GPU share the array and race: serialise them. */
edb_status edb_calQ_fp64_noalloc(int N, int index_mode, const double *d_B, const double *d_fin,
                                 double *d_Qout, void *stream);

/* Batched Q-hat for several tables in ONE launch (no reference counterpart):
 * table i is handle qs[i] (ALIASED mode, genB done, N % 4 == 0) with S[i]
 * solves in d_fin[i] / d_Qout[i] (device, layout as
 * edb_qcalc_calQ_batch_f32_device).  1 to 16 tables.  A persistent grid
 * pulls work items (the CTAs of each table's own launch) from one queue and
 * reads each item's table descriptor (N, tile shape, tensor maps, buffers), so
 * one launch fills the GPU with a mix of tables that would each leave it
 * partly idle.  variant: a plain-layout variant 0-4 of
 * edb_qcalc_calQ_batch_f32_ex for every table, or -1 for the one the
 * heaviest table (S x N^6) was autotuned to (4 if untuned).  Results equal
 * edb_qcalc_calQ_batch_f32_ex(qs[i], S[i], any variant, 1, ...) bit for bit. */
edb_status edb_qcalc_calQ_batch_multi(int ntab, edb_qcalc *const *qs, const int *S,
                                      const float *const *d_fin, float *const *d_Qout,
                                      int variant, void *stream);

/* Times the grouped launch with each plain-layout variant on the caller's
 * buffers (one warm-up and two timed launches each, CUDA events on `stream`)
 * and returns the fastest in *chosen, for edb_qcalc_calQ_batch_multi. */
edb_status edb_qcalc_autotune_batch_multi(int ntab, edb_qcalc *const *qs, const int *S,
                                          const float *const *d_fin, float *const *d_Qout,
                                          void *stream, int *chosen);

/* Autotuner of the batched kernel (no reference counterpart): times each
 * launch variant (CTA size / k2-tile shape) on the caller's buffers and keeps
 * the fastest for S's size class; later batched calls on this handle use it.
 * edb_batch_load* runs it once per size class before the step graph is built. */
edb_status edb_qcalc_autotune_batch(edb_qcalc *q, int S, const float *d_fin, float *d_Qout,
                                    void *stream, int *chosen);

/* Device status words of the Q-hat kernels (no reference counterpart): bit 0
 * set when a bounded wait inside the batched kernel ran out, bit 1 when one
 * inside the double-float FP64 kernel did (that launch then returned early,
 * after its copies in flight had landed, and its output is invalid).
 * clear != 0 resets them.  The synchronous entry points (edb_qcalc_calQ,
 * edb_qcalc_genB, edb_solver_run, edb_batch_step with a NULL stream) read
 * and clear them themselves and return EDB_ETIMEDOUT; after stream-ordered
 * calls, read them here. */
edb_status edb_device_status(int *status, int clear);

/* Limit of each bounded wait inside the Q-hat kernels (no reference
 * counterpart), in nanoseconds: ns < 0 restores the default of 200 ms, and
 * 0 makes every wait run out at once, without polling.  It is
 * read at each launch (graphs captured earlier keep the limit they were
 * captured with).  For tests of the timeout path: a wait that runs out makes
 * the kernel drain the copies it issued and return, and the entry point
 * report EDB_ETIMEDOUT. */
edb_status edb_set_wait_limit_ns(long long ns);

/* Kernel of the FP64 collision sum (edb_qcalc_calQ, _device, the integrator).
 * EMULATED (default): FP64-accurate double-float arithmetic on the FP32 pipe,
 * reading the table pre-split into (hi, lo) floats (8 bytes per term, like
 * FP64); GB300's native FP64 rate would hold the B stream near a tenth of HBM
 * bandwidth.  NATIVE: the same sum with FP64 FMA.  No reference counterpart. */
#define EDB_FP64_EMULATED 0
#define EDB_FP64_NATIVE 1
/* ONTHEFLY: the double-float kernel with the pair entries formed per term from
 * the compact tables (no N^6 table read; aliased index shifts only, i.e.
 * ALIASED mode or odd N).  Used automatically after edb_qcalc_genB_compact. */
#define EDB_FP64_ONTHEFLY 2
edb_status edb_qcalc_set_fp64_kernel(edb_qcalc *q, int kind);

/* Launch shape of the double-float kernel (EDB_FP64_EMULATED), no reference
 * counterpart: CTA size and register cap, for the output-pair form (the pair
 * table with N % 4 == 0) the table rows per ring slot, and the rule that sizes
 * the l-line chunks (the second half of the shapes repeats the first with
 * chunks from a model of the schedule).  genB times every shape on the table
 * and keeps the fastest.  shape >= 0 overrides that choice
 * (shapes with another line-chunk count add the partial sums in another order:
 * the results agree to rounding), -1 leaves it; *current (may be NULL)
 * receives the shape in use. */
edb_status edb_qcalc_fp64_shape(edb_qcalc *q, int shape, int *current);
/* Number of launch shapes of the double-float kernel. */
int edb_qcalc_fp64_shapes(void);

/* genB without the N^6 table (QCalculator.h:158-229 restated per term): builds
 * only what the on-the-fly FP64 kernel reads, the F-table T(a, b) times the
 * kernel scale, split into (hi, lo) floats and kept for b = a mod 4 only
 * (about 19 MB at N = 32, 302 MB at N = 64, where the full FP64 table would be
 * 8.6 GB and 550 GB), and Bmm and the filter products per mode.  The FP64
 * calQ entry points then run EDB_FP64_ONTHEFLY; edb_qcalc_copy_B and the
 * batched entry points report EDB_ENOTREADY.  Aliased index shifts only
 * (ALIASED mode, or odd N); EDB_EINVAL otherwise. */
edb_status edb_qcalc_genB_compact(edb_qcalc *q);

/* Copies count entries of the FP64 B table starting at flat index first
 * (row-major [l][k], centred indices) to host memory. */
edb_status edb_qcalc_copy_B(edb_qcalc *q, long long first, long long count, double *host_out);
/* Sets the FP64 B table from host memory (all N^6 entries); used to run calQ
 * on a table produced elsewhere. */
edb_status edb_qcalc_set_B(edb_qcalc *q, const double *host_B);

typedef struct {
  int N, n, P;          /* P = 2n+1 (REFERENCE) or N (ALIASED): k extent per dimension */
  long long NQ;         /* N^3 */
  long long terms;      /* terms of one calQ: N^3 P^3 */
  long long B_bytes;    /* FP64 table bytes */
  int has_B32;          /* FP32 FFTW-order pair table present */
} edb_qcalc_info;
edb_status edb_qcalc_get_info(edb_qcalc *q, edb_qcalc_info *out);

/* ------------------------------------------------------------------ fft3d */

/* fft3d::fft(Nx,Ny,Nz, re, fre) (fft3d.h:25-30): fre = unnormalised forward
 * DFT (sign -1) of re.  Host buffers, FP64, synchronous. */
edb_status edb_fft3d_fft(int nx, int ny, int nz, const double *re, double *fre);
/* fft3d::ifft(Nx,Ny,Nz, re, fre) (fft3d.h:32-48): re = backward DFT of fre
 * times 1/(Nx Ny Nz).  Cubes only (the reference's normalisation loop uses
 * Ny for the third extent, :43). */
edb_status edb_fft3d_ifft(int nx, int ny, int nz, double *re, const double *fre);
/* Batched cubic transforms on device buffers: `batch` arrays of N^3 complex,
 * fp32 = 0 (double), 1 (float) or EDB_DFT_DOUBLE_FLOAT (double data, the
 * passes in double-float arithmetic on the FP32 pipe: about 2^-47 relative per
 * operation, several times faster than FP64 on GB300; the batch and the server
 * use it); inverse applies the 1/N^3 factor. */
#define EDB_DFT_DOUBLE_FLOAT 2
edb_status edb_fft3d_device(int N, int batch, const void *d_in, void *d_out, int inverse,
                            int fp32, void *stream);

/* ------------------------------------------------------------- EntropyFix */

typedef struct edb_efix edb_efix;
/* EntropyFix(Nt, eps) (EntropyFix.h:29-32). */
edb_status edb_efix_create(int Nt, double eps, edb_efix **out);
edb_status edb_efix_destroy(edb_efix *e);
/* setAverage(Nf, f) (EntropyFix.h:65-78): latches mean(f). */
edb_status edb_efix_set_average(edb_efix *e, int Nf, const double *f);
/* EntropyCal(Nf, f) (EntropyFix.h:124-161): mean of f log f over f > eps,
 * minus the latched average (latched from f on first use). */
edb_status edb_efix_entropy(edb_efix *e, int Nf, const double *f, double *H);
/* FixSol(Nf, f, aim) (EntropyFix.h:211-253): bisection for
 * f <- (1-beta) f + beta * average, in place. */
edb_status edb_efix_fixsol(edb_efix *e, int Nf, double *f, double aim);
edb_status edb_efix_get_average(edb_efix *e, double *avg, int *latched);

/* -------------------------------------------------------- BKW3D integrator */

typedef struct {
  int N;             /* grid points per dimension (BKW3D(N0, R), BKW.h:39) */
  double R;          /* computational domain [-R, R]^3 */
  int scheme;        /* EDB_SCHEME_* */
  int fix_entropy;   /* setFixEntropy (BKW.h:46); FE and CFE consult it, SSP3/RK4 fix regardless */
  double beta;       /* CFE / DUFORT parameter */
  edb_qcalc_desc kernel; /* the reference uses QCalculator(N0, 0): gamma 0, L 6.62132, filter on */
  int conserve;      /* 0: the reference's behaviour.  1: conservative mode (no reference
                        counterpart): after every step Fhat is projected back onto its initial
                        mass, momentum and energy, and the entropy fix blends toward the discrete
                        Maxwellian of f (moment-preserving) and is fed back into Fhat */
  int record_F;      /* 1: keep Re F after every step on the device, for edb_solver_F_history
                        and edb_solver_write_F_dat */
} edb_solver_desc;

typedef struct edb_solver edb_solver;
edb_status edb_solver_create(const edb_solver_desc *d, edb_solver **out);
edb_status edb_solver_destroy(edb_solver *s);
/* Initial data in real space (N^3 interleaved complex); NULL selects the
 * reference's setInitialValue (BKW.h:121-138, the live funExact branch).
 * EDB_EINVAL when it holds a NaN or an infinity. */
edb_status edb_solver_set_initial(edb_solver *s, const double *F0);
/* Runs the reference loop `do { t += dt; ... } while (t < TEnd)` of the
 * chosen scheme from T0 (BKW.h:218-248 etc.), entirely on the device: calQ
 * stages, stage updates, ifft, calEntropy and the entropy-fix rule. */
edb_status edb_solver_run(edb_solver *s, double T0, double TEnd, double dt, int *nsteps);
/* Final Fhat (reciprocal space) and F (real space, after any fix). */
edb_status edb_solver_get(edb_solver *s, double *Fhat, double *F);
/* Entropy after each step before / after the fix (BKW.h:226-235). */
edb_status edb_solver_trace(edb_solver *s, double *raw, double *fixed, int cap, int *n);
/* Re F after each step of the last run (record_F = 1): min(cap, steps) rows
 * of N^3 doubles; *n = steps. */
edb_status edb_solver_F_history(edb_solver *s, double *out, int cap, int *n);
/* The reference's output files, written with its stream formats:
 * F.dat (BKW.h:217-249; one row per step: t, then Re F of every grid point,
 * tab-separated; needs record_F = 1) and the slice along v1 through the grid
 * centre (BKW3D::outV1Direction, BKW.h:163-180: x, Re F, funExact(0, x, h/2,
 * h/2)); testBKW3D.cpp:44-45 names it "N<N>.dt<std::to_string(dt)>.dat". */
edb_status edb_solver_write_F_dat(edb_solver *s, const char *path);
edb_status edb_solver_out_v1_direction(edb_solver *s, const char *path);

/* ------------------------------------------- batched solves (FP32 Q-hat) */

typedef struct {
  int S;             /* number of independent solves */
  int N;             /* modes per dimension (all solves share the kernel table) */
  double R;          /* velocity box half-width */
  int scheme;        /* EDB_SCHEME_FE, EDB_SCHEME_SSP3 or EDB_SCHEME_RK4 */
  double dt;
  int fix_entropy;   /* apply the EntropyFix rule after each step (FP64) */
  int conserve;      /* conservative mode, as in edb_solver_desc */
} edb_batch_desc;

typedef struct edb_batch edb_batch;
/* Stage state is FP64 on the device; each Q-hat evaluation runs the FP32
 * compensated batched kernel on an FP32 copy of the stage input. */
edb_status edb_batch_create(edb_qcalc *q, const edb_batch_desc *d, edb_batch **out);
edb_status edb_batch_destroy(edb_batch *b);
/* Real-space initial data, S x N^3 doubles (real), host memory. */
edb_status edb_batch_load(edb_batch *b, const double *F0_real);
/* Same, device memory (S x N^3 doubles).  With stream = NULL it runs on the
 * batch's own stream after the work already queued on the default stream
 * (which may be what wrote d_F0_real), and returns when done. */
edb_status edb_batch_load_device(edb_batch *b, const double *d_F0_real, void *stream);
/* Advances every solve by nsteps steps (one CUDA graph launch per step). */
edb_status edb_batch_step(edb_batch *b, int nsteps, void *stream);
/* Real-space f (S x N^3 doubles) and Fhat (S x N^3 complex) to host memory;
 * either pointer may be NULL.  With fix_entropy on, f after a step is the
 * step's real-space output after the fix rule, as the reference's F after
 * BKW3D's post-step rule (BKW.h:497-515): the fix rewrites F, not Fhat, so
 * where it acted f differs from ifft(Fhat). */
edb_status edb_batch_read(edb_batch *b, double *F_real, double *Fhat);
/* Asynchronous forms (no reference counterpart): each queues its work on the
 * batch's own streams and returns; edb_batch_sync waits for all of it.  Host
 * buffers must stay valid and unchanged until then, and should be pinned
 * (page-locked) for the copies to overlap other work.  Two batches driven
 * this way overlap one's host copies with the other's steps.  The first
 * load of a batch whose S class is untuned still waits for the autotuner.
 * read_async: real-space f only (as edb_batch_read). */
edb_status edb_batch_load_async(edb_batch *b, const double *F0_real);
edb_status edb_batch_step_async(edb_batch *b, int nsteps);
edb_status edb_batch_read_async(edb_batch *b, double *F_real);
edb_status edb_batch_sync(edb_batch *b);
/* Real-space f (S x N^3 doubles, as edb_batch_read) into device memory,
 * stream-ordered (NULL: the batch's own stream after the default stream's
 * queued work, synchronous). */
edb_status edb_batch_read_device(edb_batch *b, double *d_F_real, void *stream);
/* Entropy of each solve's last step before and after the fix rule (S doubles
 * each, either may be NULL; NaN before the first step), calEntropy of the
 * step's F (BKW.h:140-152) as the reference's trace prints them. */
edb_status edb_batch_entropy(edb_batch *b, double *raw, double *fixed);
/* Per-solve moments of the current state: S x 5 doubles (mass, momentum x3,
 * energy) on the velocity grid, and the entropy H (S doubles). */
edb_status edb_batch_moments(edb_batch *b, double *moments, double *entropy);
/* Kernel launches per step of the captured graph. */
edb_status edb_batch_launches_per_step(edb_batch *b, int *n);

/* ------------------------------------------------------ serving engine */
/* No reference counterpart (the reference runs one solve per process).  A
 * device-resident request loop for many independent solves:
 *  - requests are grouped by kernel table (N, gamma, R); each group owns one
 *    FP32 table (edb_qcalc_genB_f32) and a solve arena in HBM;
 *  - a request is admitted at its group's next step boundary when its slot
 *    fits the HBM budget (tables + arenas) and the group's live-solve cap;
 *  - every live solve of a group advances one step per replay of a captured
 *    CUDA graph (one graph per bucket of 16 live solves); groups run on their
 *    own streams, so their work overlaps on the device;
 *  - finished solves are copied out and the arena is compacted, so requests
 *    that arrive while others run join without waiting for them (continuous
 *    batching).
 * Each solve's arithmetic is independent of the others in its batch. */
typedef struct {
  double hbm_budget_bytes; /* device bytes for tables plus solve arenas */
  int scheme;              /* EDB_SCHEME_FE, EDB_SCHEME_SSP3 or EDB_SCHEME_RK4 (all requests) */
  double dt;
  int fix_entropy;         /* entropy rule after each step, as edb_batch_desc */
  int conserve;            /* conservative mode, as edb_batch_desc */
  int filter;              /* filter of the kernel tables (1 = the reference default) */
  int max_live_per_group;  /* cap of live solves per group (bounds one step's time); 0 = no cap */
} edb_server_desc;

typedef struct {
  int N;              /* modes per dimension */
  double gamma;       /* VHS exponent of the kernel table */
  double R;           /* velocity box half-width (also the table's L) */
  int steps;          /* steps to advance */
  double arrival_s;   /* arrival on the server clock (seconds since the first
                         edb_server_run); < 0: arrives when submitted */
  int want_result;    /* 1: keep f (real space) and Fhat for edb_server_result */
} edb_request;

typedef struct {
  int state;          /* 0 queued, 1 running, 2 done, 3 refused (its table and slots could
                         not be fitted in the budget while nothing else ran), 4 cancelled,
                         5 failed (its state became non-finite; no result kept) */
  int N, steps;
  double t_arrival, t_admit, t_done; /* server clock, seconds (-1: not yet) */
} edb_request_info;

typedef struct {
  long long submitted, completed, live, queued;
  double tts_p50_s, tts_p99_s, tts_mean_s, tts_max_s; /* time to solution: arrival -> result */
  double wait_p50_s, wait_p99_s;                       /* arrival -> admission */
  double first_arrival_s, last_done_s;                 /* server clock */
  double throughput_rps;      /* completed / (last_done - first_arrival) */
  double qhat_evals;          /* Q-hat evaluations of live solves */
  double qhat_evals_padded;   /* including the padding of 16-solve buckets */
  double qhat_evals_per_s;    /* qhat_evals / (last_done - first_arrival) */
  long long steps_launched;   /* graph replays */
  long long kernel_launches;  /* kernels in those replays plus admission/retirement work */
  double hbm_bytes_peak;      /* tables + arenas */
  int groups;
  long long refused;          /* requests refused by the background loop (state 3) */
  long long cancelled;        /* requests cancelled (state 4) */
  long long failed;           /* solves whose state became non-finite (state 5) */
} edb_server_stats;

typedef struct edb_server edb_server;
edb_status edb_server_create(const edb_server_desc *d, edb_server **out);
edb_status edb_server_destroy(edb_server *s);
/* Builds the table of group (N, gamma, R) now (otherwise the first request of
 * the group pays for it). */
edb_status edb_server_prepare(edb_server *s, int N, double gamma, double R);
/* Queues a request; F0_real (N^3 doubles, host) is copied.  EDB_EINVAL when
 * it holds a NaN or an infinity, EDB_ENOMEM when its table plus one slot can
 * never fit the budget. */
edb_status edb_server_submit(edb_server *s, const edb_request *r, const double *F0_real,
                             long long *id);
/* Cancels a request: a queued (or not yet arrived) one is dropped at once, a
 * running one is retired at the end of its step in flight, which frees its
 * slot; no result is kept, and edb_server_wait reports EDB_ECANCELED.
 * EDB_EINVAL when the request has already finished. */
edb_status edb_server_cancel(edb_server *s, long long id);
/* Runs the request loop on the calling thread until every submitted request
 * is done or max_wall_s seconds (<= 0: no limit) have passed (EDB_EBUSY while
 * the background loop runs). */
edb_status edb_server_run(edb_server *s, double max_wall_s);
/* Runs the request loop on a background host thread until edb_server_stop:
 * edb_server_submit may then be called from any thread at any time (arrival
 * < 0 = now), and edb_server_wait blocks until a request is done.  Stop
 * drains the work on the device; it returns the loop's error, if any. */
edb_status edb_server_start(edb_server *s);
edb_status edb_server_stop(edb_server *s);
/* Waits until request id is done (timeout_s <= 0: no limit): EDB_OK, or
 * EDB_ETIMEDOUT, or EDB_ENOMEM if it was refused, EDB_ECANCELED if it was
 * cancelled, EDB_ENONFINITE if its state overflowed or became NaN. */
edb_status edb_server_wait(edb_server *s, long long id, double timeout_s);
/* f (N^3 doubles) and Fhat (N^3 complex) of a finished request kept with
 * want_result (either pointer may be NULL); info may be NULL. */
edb_status edb_server_result(edb_server *s, long long id, double *F_real, double *Fhat,
                             edb_request_info *info);
edb_status edb_server_get_stats(edb_server *s, edb_server_stats *out);
/* The server clock (seconds since the first edb_server_run; 0 before). */
edb_status edb_server_clock(edb_server *s, double *t);

/* ------------------------------------------- spatially inhomogeneous use */
/* No reference counterpart (the reference solves the space-homogeneous
 * equation only).  df/dt + v1 df/dx = Q(f) on a periodic x grid of C cells
 * [0, Lx) splits into this transport step and one homogeneous collision
 * step per cell (a batched solve with S = C: edb_batch_load_device, _step,
 * _read_device).  d_f / d_out: C x N^3 doubles, cells-major (one cell's
 * velocity distribution on the grid v_d = -R + i_d 2R/N is contiguous), on
 * the device, distinct.  Free streaming over dt by the semi-Lagrangian rule
 * with linear interpolation: out[c][v] = f at x_c - v1 dt, interpolated
 * between the two upstream cells.  The weights are non-negative and sum to
 * one per velocity, so each velocity slice's total (mass, momentum, energy)
 * is kept to rounding and f >= 0 stays so.  Stream-ordered. */
edb_status edb_cells_transport_x_device(int C, int N, double R, double Lx, double dt,
                                        const double *d_f, double *d_out, void *stream);

/* -------------------------------------------------------- conservation */
/* No reference counterpart: the moment functionals of conservative mode.
 * Grid moments h^3 sum_j Re F_j {1, v1, v2, v3, |v|^2} (v_j = -R + j h,
 * h = 2R/N) of S solves, computed from Fhat (S x N^3 complex, FFTW order,
 * device) into d_m (S x 5 doubles, device).  Synchronous. */
edb_status edb_moments_hat_device(int N, int S, double R, const double *d_Fhat, double *d_m,
                                  void *stream);
/* Minimum-norm (Euclidean) correction of each solve's Fhat so that its grid
 * moments equal d_m0 (S x 5): F <- F - C^T (C C^T)^-1 (C F - m0), applied on
 * the three axis lines of Fhat.  Synchronous. */
edb_status edb_moments_project_device(int N, int S, double R, double *d_Fhat, const double *d_m0,
                                      void *stream);
/* Discrete Maxwellian fit: for each of S solves with f = Re F (S x N^3
 * complex, device), finds M = exp(a + b.v + c|v|^2) whose grid moments equal
 * f's (Newton on the Lagrange multipliers), writes M into Im F, theta (S x 5:
 * a, b1, b2, b3, c) and status (S ints: Newton iterations, or -1 when f has
 * no positive mass/temperature or Newton failed).  Synchronous. */
edb_status edb_maxwellian_fit_device(int N, int S, double R, double *d_F, double *d_theta,
                                     int *d_status, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* EDB_H */
