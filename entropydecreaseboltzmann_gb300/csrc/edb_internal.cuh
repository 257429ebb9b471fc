// Internal declarations shared by the libedb translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/edb.h"

namespace edb {

// ---------------------------------------------------------------- errors
void set_error(const std::string &msg);
edb_status fail(edb_status s, const std::string &msg);
edb_status cuda_fail(cudaError_t e, const char *what);
void count_launch(int n = 1);

#define EDB_CUDA(call)                                       \
  do {                                                       \
    cudaError_t e__ = (call);                                \
    if (e__ != cudaSuccess) return ::edb::cuda_fail(e__, #call); \
  } while (0)

#define EDB_TRY(call)                  \
  do {                                 \
    edb_status s__ = (call);           \
    if (s__ != EDB_OK) return s__;     \
  } while (0)

// Launch check: records the launch and returns on a launch error.
#define EDB_LAUNCHED()                                        \
  do {                                                        \
    ::edb::count_launch();                                    \
    cudaError_t e__ = cudaGetLastError();                     \
    if (e__ != cudaSuccess) return ::edb::cuda_fail(e__, "kernel launch"); \
  } while (0)

edb_status ensure_device();
// Streaming multiprocessors of the current device (queried once per device;
// 1 if the query fails).  Launch sizing uses it instead of a fixed count.
int device_sm_count();

// Device allocation of `count` elements of T (EDB_ENOMEM on failure).
template <typename T>
inline edb_status dalloc(T **p, size_t count) {
  *p = nullptr;
  if (count == 0) return EDB_OK;
  cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(EDB_ENOMEM, std::string("cudaMalloc of ") + std::to_string(count * sizeof(T)) +
                                " bytes failed: " + cudaGetErrorString(e));
  }
  return EDB_OK;
}
template <typename T>
inline void dfree(T *&p) {
  if (p) cudaFree((void *)p);
  p = nullptr;
}

// ------------------------------------------------------------ parameters
// Index parameters of one collision sum (both index modes).  With i the
// centred l-index per dimension (i in [0,N)) and j the k-index (j in [0,P)):
//   f_l  = fin[(i + sL) mod N]            (FFTW index, per dimension)
//   f_m  = fin[(j - i + sM) mod N]
//   beta = B[lflat * KC + kflat]
// REFERENCE: P = 2n+1, sL = n+1, sM = 2n+1 (QCalculator.h:239-247 with the
// doubled f of transf :108-123).  ALIASED: P = N, sL = N-n, sM = 0.
struct QParams {
  int N, n, P, mode;
  int sL, sM;
  long long NQ, KC;  // N^3, P^3
};
QParams make_qparams(int N, int mode);

// ------------------------------------------------------------ kernels API
// genB: table of F(sqrt(a) lp, sqrt(b) lp) for a, b in [0, amax], a = b mod 4.
edb_status launch_ftable(int N, double gamma, double *d_T, int amax, cudaStream_t st);
// sigma (filter) per centred index and Bmm per flat centred index.
edb_status launch_bmm(int N, double gamma, double L, int filter, int mode, const double *d_T,
                      int amax, double *d_sigma, double *d_Bmm, cudaStream_t st);
// B64: [l][k] centred, N^3 x N^3 doubles.  B32 (optional): the FP32 pair table
// in FFTW order, [l1 l2][k1][l3][k2][k3] (see genB_kernel).
edb_status launch_genB(int N, double gamma, double L, int filter, int mode, const double *d_T,
                       int amax, const double *d_sigma, const double *d_Bmm, double *d_B64,
                       float *d_B32, cudaStream_t st);

// rval (the kernel scale) of an N-mode table with box half-width L.
double genb_rval(int N, double gamma, double L);

// FP64-accurate calQ with the pair entries formed on the fly (no N^6 table):
// tc = T(a, b) rval split, row a, column q for b = (a mod 4) + 4q
// ((amax + 1) x calq64f_row_len(amax) float2); bs = {Bmm, sigma3} split per
// mode in FFTW order (N^3 float4).  Aliased index shifts only.  d_partial
// holds calq64f_nchunk(p) * KC.
int calq64f_nchunk(const QParams &p);
int calq64f_row_len(int amax);
edb_status launch_calq64f_tables(int N, int filter, double rval, const double *d_T, int amax,
                                 const double *d_sigma, const double *d_Bmm, float2 *d_tc,
                                 float4 *d_bs, cudaStream_t st);
edb_status launch_calq64f(const QParams &p, int filter, int amax, const float2 *d_tc,
                          const float4 *d_bs, const float4 *d_fdf, double2 *d_partial,
                          double2 *d_Q, cudaStream_t st);

// QCalculator::funF (alpha 0/1 closed forms, other alpha -> 0) and
// ::filtering at n points.
edb_status launch_funF_points(int alpha, long long n, const double *d_xi, const double *d_eta,
                              double *d_out, cudaStream_t st);
edb_status launch_filtering_points(int N, long long n, const int *d_beta, double *d_out,
                                   cudaStream_t st);

// FP64 calQ: partial sums over l-chunks then an ordered reduction + output
// conversion.  d_partial holds nchunk * KC complex doubles.
int calq64_nchunk(const QParams &p);
edb_status launch_calq64(const QParams &p, const double *d_B, const double2 *d_fin,
                         double2 *d_partial, double2 *d_Q, cudaStream_t st);

edb_status launch_calq64_reduce(const QParams &p, int nchunk, const double2 *d_partial,
                                double2 *d_Q, cudaStream_t st);

// FP64-accurate calQ on the FP32 pipe (double-float arithmetic): B2 is the
// table split into (hi, lo) floats, fdf (N^3 float4) the input split into
// {re_hi, im_hi, re_lo, im_lo}.
// d_partial holds calq64x_nchunk(p) * KC.
int calq64x_nchunk(const QParams &p, int *J2T_out);
edb_status launch_split_f(long long n, const double2 *f, float4 *out, cudaStream_t st);
edb_status launch_split_B(long long n, const double *B, float2 *B2, cudaStream_t st);
// ALIASED tables: B2 = split of the symmetric pair table (B[l][k] + B[k-l][k]
// off the planes l1 = m1), read by launch_calq64x with paired = true.
edb_status launch_split_B_paired(int N, const double *B, float2 *B2, cudaStream_t st);
// shape in [0, calq64x_shapes()) selects the CTA size and register cap (timed
// per table at genB).  paired: B2 is the pair table and only the l1 planes
// with l1 <= m1 are visited.
int calq64x_shapes();
// d_in: f-hat (FP64); d_fdf: its split (work, NQ + 1 float4), written here.
edb_status launch_calq64x(const QParams &p, const float2 *d_B2, const double2 *d_in,
                          float4 *d_fdf, double2 *d_partial, double2 *d_Q, cudaStream_t st,
                          int shape, bool paired);

// Batched FP32 calQ (ALIASED): S solves, B32 the symmetric pair table in FFTW
// order (see genB_kernel).
//
// The FP32 pair table keeps, per output plane k1 (FFTW order), only the l1
// planes the batched kernel visits, l1 <= (k1 - l1) mod N: [0, k1/2] and
// [k1+1, (k1+N)/2], at list positions p = 0 .. c32_nlist - 1.  Layout
// [k1][p][l2][l3][k2][k3] with room for c32_maxlist planes per k1.
__host__ __device__ inline int c32_nlist(int N, int k1) {
  const int hi = (k1 + N) / 2 - k1;
  return k1 / 2 + 1 + (hi > 0 ? hi : 0);
}
__host__ __device__ inline int c32_maxlist(int N) { return N / 2 + 1; }  // max over k1 of c32_nlist
__host__ __device__ inline int c32_plane_pos(int N, int k1, int l1) {
  if (l1 <= k1 / 2) return l1;
  if (l1 > k1 && l1 <= (k1 + N) / 2) return k1 / 2 + 1 + (l1 - k1 - 1);
  return -1;
}
inline long long c32_table_floats(int N) {
  const long long NQ = (long long)N * N * N;
  return (long long)N * c32_maxlist(N) * N * NQ;
}
// variant in [0, calq32_variants()) selects the solve group and CTA shape
// (see the kernel).  C > 1 splits the l1 planes into C chunks reduced in
// order in FP64; d_partial then holds C * S * N^3 float4.  Pair variants
// (calq32_pair) first copy d_fin into d_pairs, calq32_pair_bytes(N, S) long.
int calq32_variants();
int calq32_group(int variant);  // solves per CTA group
bool calq32_pair(int variant);
size_t calq32_pair_bytes(int N, int S);
// persist: run the plain-layout, tensor-copy launches as one persistent grid.
// -1: only without chunks, where it is faster alone, with the CTA work items
// pulled from a queue (a stream-ordered counter: the items in flight stay
// together, and the table is read from HBM as often as by the plain grid);
// 1: also chunked, items taken round-robin (no counter to allocate, zero and
// free in every graph replay): slower alone, but the serving engine's groups
// overlap better on their streams (32 -> 36 requests/s); 0: never.
edb_status launch_calq32_batch(int N, int S, const float *d_B32, const float2 *d_fin,
                               float2 *d_Q, cudaStream_t st, int variant, int C = 1,
                               float4 *d_partial = nullptr, float4 *d_pairs = nullptr,
                               int persist = -1);
// One table of a grouped batched launch: S solves (fin / Q, S x N^3 float2)
// on the FP32 pair table B32 of their (N, gamma, L).
struct C32MultiIn {
  int N, S;
  const float *B32;
  const float2 *fin;
  float2 *Q;
  int C = 1;                  // l1-plane chunks (C > 1: partial sums, reduced by the caller)
  float4 *partial = nullptr;  // C x S x N^3 when C > 1
};
// Q-hat of several tables' solves in one persistent launch (1 to 16 tables,
// each with N % 4 == 0) with one plain-layout variant (0-4): the per-table
// results, bit for bit.  queue: CTAs pull work items from an atomic counter
// (stream-ordered allocation); otherwise they take them round-robin.
edb_status launch_calq32_multi(int ntab, const C32MultiIn *in, int variant, cudaStream_t st,
                               bool queue = true);
// Reads (and optionally clears) the batched kernel's / the double-float FP64
// kernel's status word: nonzero when a bounded wait inside it ran out.
edb_status read_calq32_status(int *status, bool clear);
edb_status read_calq64x_status(int *status, bool clear);
// Limit of every bounded mbarrier wait of the Q-hat kernels, passed to each
// launch (default 200 ms; see edb_set_wait_limit_ns).
unsigned long long wait_limit_ns();

// Batched cubic DFT (FP64 or FP32), out-of-place; d_tmp holds batch*N^3 complex.
edb_status launch_dft3d(int N, int batch, const void *d_in, void *d_out, void *d_tmp,
                        int inverse, int fp32, cudaStream_t st);

// Entropy / EntropyFix state per solve.
struct EfixState {
  double avg;       // Averagef (EntropyFix.h:20)
  int avg_flag;     // Average_flag (EntropyFix.h:22)
  int fixed;        // conservative mode: the last step's fix changed F
  double H_prev;    // entropy0 of the integrator loop
  int step;         // integrator step counter (BKW.h:216, 278, ...)
  int rec;          // trace records written
};

// calEntropy (BKW.h:140-152) of Re F for `batch` solves -> d_H.
edb_status launch_calentropy(int N, int batch, double R, const double2 *d_F, double *d_H,
                             cudaStream_t st);
// The integrator's post-step rule (compute H, fix on entropy rise, record
// trace, roll H_prev) for `batch` solves; fix_mode: 0 never, 1 after step>1
// if flag (FE), 2 if step (CFE with flag / SSP3 / RK4).  The trace records
// steps 0 .. trace_cap - 1, or with keep_last the last trace_cap steps (step
// r in slot r mod trace_cap).
edb_status launch_step_entropy(int N, int batch, double R, double2 *d_F, EfixState *d_state,
                               double eps, int fix_mode, double *d_trace_raw,
                               double *d_trace_fixed, int trace_cap, cudaStream_t st,
                               bool keep_last = false);
// EntropyFix primitives on one array (host API wrappers).
edb_status launch_efix_average(int Nf, const double *d_f, EfixState *d_state, cudaStream_t st);
edb_status launch_efix_entropy(int Nf, const double *d_f, EfixState *d_state, double eps,
                               double *d_H, cudaStream_t st);
edb_status launch_efix_fixsol(int Nf, double *d_f, EfixState *d_state, double eps, double aim,
                              cudaStream_t st);

// Stage updates of the integrators (see edb_kernels_misc.cu for the exact
// expressions).  launch_stage_f32q reads FP32 Q-hat arrays.
enum { STAGE_AXPY = 0, STAGE_SSP3_2 = 1, STAGE_SSP3_3 = 2, STAGE_RK4 = 3, STAGE_DUFORT = 4 };
edb_status launch_stage(long long n, int op, double c0, double c1, double c2, double2 *y,
                        const double2 *x, const double2 *z, const double2 *w, const double2 *q0,
                        const double2 *q1, const double2 *q2, const double2 *q3, float2 *y32,
                        cudaStream_t st);
edb_status launch_stage_f32q(long long n, int op, double c0, double c1, double c2, double2 *y,
                             const double2 *x, const double2 *z, const double2 *w,
                             const float2 *q0, const float2 *q1, const float2 *q2,
                             const float2 *q3, float2 *y32, cudaStream_t st);
edb_status launch_d2f(long long n, const double2 *x, float2 *y, cudaStream_t st);
edb_status launch_f2d(long long n, const float2 *x, double2 *y, cudaStream_t st);
edb_status launch_real_to_complex(long long n, const double *x, double2 *y, cudaStream_t st);
edb_status launch_complex_to_real(long long n, const double2 *y, double *x, cudaStream_t st);
edb_status launch_sinusoid_init(int N, double R, double2 *d_F, cudaStream_t st);
// BKW3D::funExact's live branch at n points (x[i], y, z).
edb_status launch_funexact_points(double R, int n, const double *d_x, double y, double z,
                                  double *d_out, cudaStream_t st);
// Re F into row (state->rec - 1) of hist (cap rows of N^3 doubles).
edb_status launch_record_re(long long NQ, const double2 *d_F, const EfixState *d_state,
                            double *d_hist, int cap, cudaStream_t st);
// moments (mass, momentum, energy) of Re F per solve, FP64.
edb_status launch_moments(int N, int batch, double R, const double2 *d_F, double *d_out,
                          cudaStream_t st);

// ---- QCalculator internals used by the serving engine (edb_capi.cu)
const float *qcalc_B32(const edb_qcalc *q);
// Batched-kernel variant for S solves (split: chunked launches); *tuned =
// false when S's size class has not been autotuned yet.
int qcalc_c32_variant(const edb_qcalc *q, int S, bool *tuned, bool split);
// Autotunes the chunked launch (C chunks, partial buffer) for S solves.
edb_status qcalc_autotune_split(edb_qcalc *q, int S, const float2 *d_fin, float2 *d_Qout,
                                cudaStream_t st, int C, float4 *d_partial);
// Device bytes held by the handle's tables.
long long qcalc_table_bytes(const edb_qcalc *q);

// ---- conservation (edb_kernels_conserve.cu)
// Table per (N, R): W1, W2 (N complex each), G^-1 (25), h^3.
inline int conserve_table_len(int N) { return 4 * N + 32; }
void build_conserve_table(int N, double R, std::vector<double> &tab);
// Grid moments h^3 sum F {1, v1, v2, v3, |v|^2} of S solves from F-hat.
edb_status launch_hat_moments(int N, int S, const double *d_tab, const double2 *d_Fhat,
                              double *d_out, cudaStream_t st);
// Minimum-norm correction of F-hat onto the moments d_m0 (S x 5).
edb_status launch_project_moments(int N, int S, const double *d_tab, double2 *d_Fhat,
                                  const double *d_m0, cudaStream_t st);
// Post-step rule with the moment-preserving fix (sets EfixState::fixed).
edb_status launch_step_entropy_conserve(int N, int batch, double R, double2 *d_F,
                                        EfixState *d_state, double eps, int fix_mode,
                                        double *d_trace_raw, double *d_trace_fixed,
                                        int trace_cap, cudaStream_t st, bool keep_last = false);
edb_status launch_maxwellian_fit(int N, int S, double R, double2 *d_F, double *d_theta,
                                 int *d_status, cudaStream_t st);
edb_status launch_state_from_entropy(int S, const double *d_H, EfixState *d_state,
                                     cudaStream_t st);
edb_status launch_masked_copy(long long NQ, int S, const EfixState *d_state,
                              const double2 *d_src, double2 *d_dst, cudaStream_t st);

}  // namespace edb
