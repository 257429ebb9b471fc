// C ABI of libedb.so (declared in include/edb.h): handles, host/device entry
// points, the device-resident BKW3D integrator and the batched solver.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <fstream>
#include <iomanip>
#include <mutex>
#include <string>
#include <vector>

#include "edb_internal.cuh"

namespace edb {

static thread_local std::string g_err;
static std::atomic<long long> g_launches{0};
static constexpr unsigned long long kDefaultWaitNs = 200000000ull;  // 200 ms
static std::atomic<unsigned long long> g_wait_ns{kDefaultWaitNs};

unsigned long long wait_limit_ns() { return g_wait_ns.load(std::memory_order_relaxed); }

// After a synchronous call's work has finished: EDB_ETIMEDOUT (and the words
// cleared) when a bounded wait inside a Q-hat kernel ran out, whose output is
// then invalid.
static edb_status check_device_waits(const char *what) {
  int a = 0, b = 0;
  EDB_TRY(read_calq32_status(&a, true));
  EDB_TRY(read_calq64x_status(&b, true));
  if (a || b)
    return fail(EDB_ETIMEDOUT, std::string(what) +
                                   ": a bounded wait inside a Q-hat kernel ran out; the "
                                   "result is invalid");
  return EDB_OK;
}

void set_error(const std::string &msg) { g_err = msg; }
edb_status fail(edb_status s, const std::string &msg) {
  g_err = msg;
  return s;
}
edb_status cuda_fail(cudaError_t e, const char *what) {
  g_err = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
  return EDB_ECUDA;
}
void count_launch(int n) { g_launches += n; }

int device_sm_count() {
  constexpr int kMaxDev = 64;
  static std::atomic<int> cache[kMaxDev];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return 1;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v > 0) return v;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1)
    return 1;
  cache[dev].store(v, std::memory_order_relaxed);
  return v;
}

edb_status ensure_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    return fail(EDB_ECUDA, std::string("no usable CUDA device: ") +
                               (e != cudaSuccess ? cudaGetErrorString(e) : "device count 0"));
  return EDB_OK;
}

}  // namespace edb

using namespace edb;

// ====================================================================== misc

extern "C" const char *edb_last_error(void) { return g_err.c_str(); }

extern "C" const char *edb_status_string(edb_status s) {
  switch (s) {
    case EDB_OK: return "EDB_OK";
    case EDB_EINVAL: return "EDB_EINVAL";
    case EDB_ENOMEM: return "EDB_ENOMEM";
    case EDB_ECUDA: return "EDB_ECUDA";
    case EDB_ETIMEDOUT: return "EDB_ETIMEDOUT";
    case EDB_ENOTREADY: return "EDB_ENOTREADY";
    case EDB_EBUSY: return "EDB_EBUSY";
    case EDB_ENOTFOUND: return "EDB_ENOTFOUND";
    case EDB_ECANCELED: return "EDB_ECANCELED";
    case EDB_ENONFINITE: return "EDB_ENONFINITE";
  }
  return "EDB_UNKNOWN";
}

extern "C" int edb_version(void) { return 100; }
extern "C" long long edb_kernel_launch_count(void) { return g_launches.load(); }

// Uploads the conservation table of (N, R) (see edb_kernels_conserve.cu).
static edb_status upload_conserve_table(int N, double R, double **d_tab) {
  std::vector<double> tab;
  build_conserve_table(N, R, tab);
  if (!*d_tab) EDB_TRY(dalloc(d_tab, tab.size()));
  EDB_CUDA(cudaMemcpy(*d_tab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice));
  return EDB_OK;
}

// =============================================================== QCalculator

struct edb_qcalc {
  edb_qcalc_desc d;
  QParams p;
  cudaStream_t st = nullptr;
  double *B64 = nullptr;    // [l][k] centred, N^3 x N^3 (flat stream of row stride KC)
  float2 *B2 = nullptr;     // B64 split into (hi, lo) floats, same layout
  float *B32 = nullptr;     // FP32 pair table, visited planes only (c32_table_floats; ALIASED)
  float4 *fdf = nullptr;    // input split for the double-float kernel
  // tables of the on-the-fly FP64 kernel (aliased index shifts): T rval split
  // (compressed over b = a mod 4) and {Bmm, sigma3} per mode
  float2 *tc = nullptr;
  float4 *bs = nullptr;
  int amax = 0;
  int fp64_kernel = EDB_FP64_EMULATED;
  int c64x_shape = 0;   // launch shape of the double-float kernel, tuned at genB
  double2 *partial = nullptr;
  double2 *fin = nullptr, *Q = nullptr;  // host-API staging
  int nchunk = 0;
  bool ready = false;
  int c32_variant[16];        // autotuned batched-kernel variant per S class, -1 = untuned
  int c32_variant_split[16];  // the same for chunked launches (serving engine)
  float4 *pairs = nullptr;    // solve-pair copy of the input for pair variants
  size_t pairs_bytes = 0;
};

// Grows the qcalc's solve-pair buffer to hold S solves (not under capture).
static edb_status qcalc_pairs(edb_qcalc *q, int S) {
  const size_t need = calq32_pair_bytes(q->d.N, S);
  if (need <= q->pairs_bytes) return EDB_OK;
  EDB_CUDA(cudaDeviceSynchronize());
  dfree(q->pairs);
  q->pairs_bytes = 0;
  EDB_TRY(dalloc(&q->pairs, need / sizeof(float4)));
  q->pairs_bytes = need;
  return EDB_OK;
}

// S class of the autotuner: floor(log2(S)), capped at 15.
static int s_bucket(int S) {
  int b = 0;
  while (S > 1 && b < 15) {
    S >>= 1;
    ++b;
  }
  return b;
}
static int c32_variant_for(const edb_qcalc *q, int S) {
  int v = q->c32_variant[s_bucket(S)];
  return v < 0 ? 0 : v;
}

static edb_status check_desc(const edb_qcalc_desc *d) {
  if (!d) return fail(EDB_EINVAL, "null descriptor");
  if (d->N < 3 || d->N > 64) return fail(EDB_EINVAL, "N must be in [3, 64]");
  if (!(d->gamma >= 0.0 && d->gamma <= 2.0)) return fail(EDB_EINVAL, "gamma must be in [0, 2]");
  if (!(d->L > 0.0)) return fail(EDB_EINVAL, "L must be positive");
  if (d->index_mode != EDB_INDEX_REFERENCE && d->index_mode != EDB_INDEX_ALIASED)
    return fail(EDB_EINVAL, "unknown index mode");
  return EDB_OK;
}

extern "C" edb_status edb_qcalc_desc_init(edb_qcalc_desc *d, int N, int alpha) {
  if (!d) return fail(EDB_EINVAL, "null descriptor");
  d->N = N;
  d->gamma = (double)alpha;
  d->L = EDB_R_REFERENCE;
  d->filter = 1;
  d->index_mode = EDB_INDEX_REFERENCE;
  return EDB_OK;
}

extern "C" edb_status edb_qcalc_create(const edb_qcalc_desc *d, edb_qcalc **out) {
  if (!out) return fail(EDB_EINVAL, "null output pointer");
  *out = nullptr;
  EDB_TRY(check_desc(d));
  EDB_TRY(ensure_device());
  edb_qcalc *q = new edb_qcalc();
  for (int &v : q->c32_variant) v = -1;
  for (int &v : q->c32_variant_split) v = -1;
  q->d = *d;
  q->p = make_qparams(d->N, d->index_mode);
  cudaError_t e = cudaStreamCreateWithFlags(&q->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete q;
    return cuda_fail(e, "cudaStreamCreate");
  }
  *out = q;
  return EDB_OK;
}

extern "C" edb_status edb_qcalc_destroy(edb_qcalc *q) {
  if (!q) return EDB_OK;
  if (q->st) cudaStreamSynchronize(q->st);
  dfree(q->B64);
  dfree(q->B2);
  dfree(q->B32);
  dfree(q->fdf);
  dfree(q->tc);
  dfree(q->bs);
  dfree(q->pairs);
  dfree(q->partial);
  dfree(q->fin);
  dfree(q->Q);
  if (q->st) cudaStreamDestroy(q->st);
  delete q;
  return EDB_OK;
}

extern "C" edb_status edb_qcalc_close_filter(edb_qcalc *q) {
  if (!q) return fail(EDB_EINVAL, "null handle");
  q->d.filter = 0;
  return EDB_OK;
}

static int amax_of(int N) {
  int n = (N - 1) / 2;
  int hi = 2 * (N - 1 - n);
  if (N - 1 > hi) hi = N - 1;
  return 3 * hi * hi;
}

// The double-float kernel's table: the symmetric pair table (half the l1
// planes are visited) in ALIASED mode and for odd N, where the REFERENCE index
// mode is the same aliased convolution (P = N, the same index shifts); else
// B split as it is.
static bool qcalc_b2_paired(const edb_qcalc *q) {
  return q->p.mode == EDB_INDEX_ALIASED || (q->p.N % 2 == 1 && q->p.P == q->p.N);
}
static edb_status qcalc_split_B2(edb_qcalc *q) {
  if (qcalc_b2_paired(q)) return launch_split_B_paired(q->p.N, q->B64, q->B2, q->st);
  return launch_split_B(q->p.NQ * q->p.NQ, q->B64, q->B2, q->st);
}

static edb_status qcalc_alloc_work(edb_qcalc *q) {
  if (!q->partial) {
    q->nchunk = calq64_nchunk(q->p);
    int nmax = calq64x_nchunk(q->p, nullptr);
    if (q->nchunk > nmax) nmax = q->nchunk;
    if (qcalc_b2_paired(q)) nmax = std::max(nmax, calq64f_nchunk(q->p));
    EDB_TRY(dalloc(&q->partial, (size_t)nmax * q->p.KC));
  }

  if (!q->fdf) EDB_TRY(dalloc(&q->fdf, (size_t)q->p.NQ + 1));  // split f (+ padding)
  if (!q->fin) EDB_TRY(dalloc(&q->fin, (size_t)q->p.NQ));
  if (!q->Q) EDB_TRY(dalloc(&q->Q, (size_t)q->p.NQ));
  return EDB_OK;
}

// Times every launch shape (CTA size, register cap) of the double-float
// kernel on this table (input: the zeroed staging buffer; the kernel's cost
// does not depend on the values) and keeps the fastest.
static edb_status qcalc_tune_fp64(edb_qcalc *q) {
  if (!q->B2) return EDB_OK;
  cudaStream_t st = q->st;
  EDB_CUDA(cudaMemsetAsync(q->fin, 0, sizeof(double2) * q->p.NQ, st));
  cudaEvent_t e0, e1;
  EDB_CUDA(cudaEventCreate(&e0));
  EDB_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int best_shape = 0;
  edb_status rc = EDB_OK;
  for (int shape = 0; shape < calq64x_shapes() && rc == EDB_OK; ++shape) {
    rc = launch_calq64x(q->p, q->B2, q->fin, q->fdf, q->partial, q->Q, st, shape,
                        qcalc_b2_paired(q));
    cudaEventRecord(e0, st);
    for (int r = 0; r < 2 && rc == EDB_OK; ++r)
      rc = launch_calq64x(q->p, q->B2, q->fin, q->fdf, q->partial, q->Q, st, shape,
                          qcalc_b2_paired(q));
    cudaEventRecord(e1, st);
    cudaError_t ce = cudaEventSynchronize(e1);
    if (ce != cudaSuccess) {
      rc = cuda_fail(ce, "fp64 tune");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) {
      best = ms;
      best_shape = shape;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  q->c64x_shape = best_shape;
  if (rc != EDB_OK) return rc;
  return check_device_waits("genB (FP64 kernel timing)");
}

// The on-the-fly kernel's tables from the FP64 F-table, sigma and Bmm.
static edb_status qcalc_build_compact(edb_qcalc *q, const double *T, const double *sigma,
                                      const double *Bmm) {
  const int N = q->d.N;
  q->amax = amax_of(N);
  if (!q->tc)
    EDB_TRY(dalloc(&q->tc, (size_t)(q->amax + 1) * (size_t)calq64f_row_len(q->amax)));
  if (!q->bs) EDB_TRY(dalloc(&q->bs, (size_t)q->p.NQ));
  return launch_calq64f_tables(N, q->d.filter, genb_rval(N, q->d.gamma, q->d.L), T, q->amax,
                               sigma, Bmm, q->tc, q->bs, q->st);
}

extern "C" edb_status edb_qcalc_genB(edb_qcalc *q) {
  if (!q) return fail(EDB_EINVAL, "null handle");
  const int N = q->d.N;
  const long long NQ = q->p.NQ;
  const int amax = amax_of(N);
  double *T = nullptr, *sigma = nullptr, *Bmm = nullptr;
  edb_status s = EDB_OK;
  if (!q->B64) EDB_TRY(dalloc(&q->B64, (size_t)NQ * NQ));
  if (!q->B2) EDB_TRY(dalloc(&q->B2, (size_t)NQ * NQ));
  if (q->d.index_mode == EDB_INDEX_ALIASED && !q->B32)
    EDB_TRY(dalloc(&q->B32, (size_t)c32_table_floats(N) + 64));  // +64: masked tail reads
  EDB_TRY(qcalc_alloc_work(q));
  s = dalloc(&T, (size_t)(amax + 1) * (amax + 1));
  if (s == EDB_OK) s = dalloc(&sigma, 64);
  if (s == EDB_OK) s = dalloc(&Bmm, (size_t)NQ);
  if (s == EDB_OK) s = launch_ftable(N, q->d.gamma, T, amax, q->st);
  if (s == EDB_OK)
    s = launch_bmm(N, q->d.gamma, q->d.L, q->d.filter, q->d.index_mode, T, amax, sigma, Bmm,
                   q->st);
  if (s == EDB_OK)
    s = launch_genB(N, q->d.gamma, q->d.L, q->d.filter, q->d.index_mode, T, amax, sigma, Bmm,
                    q->B64, q->B32, q->st);
  if (s == EDB_OK) s = qcalc_split_B2(q);
  if (s == EDB_OK && qcalc_b2_paired(q)) s = qcalc_build_compact(q, T, sigma, Bmm);
  cudaError_t e = cudaStreamSynchronize(q->st);
  dfree(T);
  dfree(sigma);
  dfree(Bmm);
  if (s != EDB_OK) return s;
  if (e != cudaSuccess) return cuda_fail(e, "genB");
  q->ready = true;
  return qcalc_tune_fp64(q);
}

extern "C" edb_status edb_qcalc_genB_compact(edb_qcalc *q) {
  if (!q) return fail(EDB_EINVAL, "null handle");
  if (!qcalc_b2_paired(q))
    return fail(EDB_EINVAL, "the compact tables need the aliased index shifts (ALIASED, or odd N)");
  const int N = q->d.N;
  const int amax = amax_of(N);
  double *T = nullptr, *sigma = nullptr, *Bmm = nullptr;
  EDB_TRY(qcalc_alloc_work(q));
  edb_status s = dalloc(&T, (size_t)(amax + 1) * (amax + 1));
  if (s == EDB_OK) s = dalloc(&sigma, 64);
  if (s == EDB_OK) s = dalloc(&Bmm, (size_t)q->p.NQ);
  if (s == EDB_OK) s = launch_ftable(N, q->d.gamma, T, amax, q->st);
  if (s == EDB_OK)
    s = launch_bmm(N, q->d.gamma, q->d.L, q->d.filter, q->d.index_mode, T, amax, sigma, Bmm,
                   q->st);
  if (s == EDB_OK) s = qcalc_build_compact(q, T, sigma, Bmm);
  cudaError_t e = cudaStreamSynchronize(q->st);
  dfree(T);
  dfree(sigma);
  dfree(Bmm);
  if (s != EDB_OK) return s;
  if (e != cudaSuccess) return cuda_fail(e, "genB_compact");
  q->ready = true;
  return EDB_OK;
}

extern "C" edb_status edb_funF(int alpha, long long n, const double *xi, const double *eta,
                               double *out) {
  if (n < 0 || (n > 0 && (!xi || !eta || !out))) return fail(EDB_EINVAL, "bad argument");
  if (n == 0) return EDB_OK;
  EDB_TRY(ensure_device());
  double *d = nullptr;
  EDB_TRY(dalloc(&d, (size_t)n * 3));
  cudaError_t e = cudaMemcpy(d, xi, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + n, eta, sizeof(double) * n, cudaMemcpyHostToDevice);
  edb_status rc = e == cudaSuccess ? launch_funF_points(alpha, n, d, d + n, d + 2 * n, nullptr)
                                   : cuda_fail(e, "funF upload");
  if (rc == EDB_OK) {
    e = cudaMemcpy(out, d + 2 * n, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = cuda_fail(e, "funF download");
  }
  dfree(d);
  return rc;
}

extern "C" edb_status edb_filtering(int N, long long n, const int *beta, double *out) {
  if (N < 3 || N > 64 || n < 0 || (n > 0 && (!beta || !out))) return fail(EDB_EINVAL, "bad argument");
  if (n == 0) return EDB_OK;
  EDB_TRY(ensure_device());
  int *db = nullptr;
  double *dout = nullptr;
  EDB_TRY(dalloc(&db, (size_t)n));
  edb_status rc = dalloc(&dout, (size_t)n);
  cudaError_t e = cudaSuccess;
  if (rc == EDB_OK) e = cudaMemcpy(db, beta, sizeof(int) * n, cudaMemcpyHostToDevice);
  if (rc == EDB_OK && e != cudaSuccess) rc = cuda_fail(e, "filtering upload");
  if (rc == EDB_OK) rc = launch_filtering_points(N, n, db, dout, nullptr);
  if (rc == EDB_OK) {
    e = cudaMemcpy(out, dout, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = cuda_fail(e, "filtering download");
  }
  dfree(db);
  dfree(dout);
  return rc;
}

extern "C" edb_status edb_qcalc_genB_f32(edb_qcalc *q) {
  if (!q) return fail(EDB_EINVAL, "null handle");
  if (q->d.index_mode != EDB_INDEX_ALIASED)
    return fail(EDB_EINVAL, "the FP32 table exists in ALIASED mode only");
  const int N = q->d.N;
  const long long NQ = q->p.NQ;
  const int amax = amax_of(N);
  if (!q->B32) EDB_TRY(dalloc(&q->B32, (size_t)c32_table_floats(N) + 64));  // +64: tail reads
  double *T = nullptr, *sigma = nullptr, *Bmm = nullptr;
  edb_status s = dalloc(&T, (size_t)(amax + 1) * (amax + 1));
  if (s == EDB_OK) s = dalloc(&sigma, 64);
  if (s == EDB_OK) s = dalloc(&Bmm, (size_t)NQ);
  if (s == EDB_OK) s = launch_ftable(N, q->d.gamma, T, amax, q->st);
  if (s == EDB_OK)
    s = launch_bmm(N, q->d.gamma, q->d.L, q->d.filter, q->d.index_mode, T, amax, sigma, Bmm,
                   q->st);
  if (s == EDB_OK)
    s = launch_genB(N, q->d.gamma, q->d.L, q->d.filter, q->d.index_mode, T, amax, sigma, Bmm,
                    nullptr, q->B32, q->st);
  cudaError_t e = cudaStreamSynchronize(q->st);
  dfree(T);
  dfree(sigma);
  dfree(Bmm);
  if (s != EDB_OK) return s;
  if (e != cudaSuccess) return cuda_fail(e, "genB_f32");
  return EDB_OK;
}

namespace edb {
const float *qcalc_B32(const edb_qcalc *q) { return q->B32; }
int qcalc_c32_variant(const edb_qcalc *q, int S, bool *tuned, bool split) {
  const int v = (split ? q->c32_variant_split : q->c32_variant)[s_bucket(S)];
  if (tuned) *tuned = v >= 0;
  return v < 0 ? 0 : v;
}
long long qcalc_table_bytes(const edb_qcalc *q) {
  long long b = 0;
  const long long e = q->p.NQ * q->p.NQ;
  if (q->B64) b += e * 8;
  if (q->B2) b += e * 8;
  if (q->B32) b += c32_table_floats(q->p.N) * 4 + 256;
  if (q->tc) b += (long long)(q->amax + 1) * calq64f_row_len(q->amax) * 8 + q->p.NQ * 16;
  return b;
}
}  // namespace edb

extern "C" edb_status edb_qcalc_set_B(edb_qcalc *q, const double *host_B) {
  if (!q || !host_B) return fail(EDB_EINVAL, "null argument");
  const long long NQ = q->p.NQ;
  if (!q->B64) EDB_TRY(dalloc(&q->B64, (size_t)NQ * NQ));
  EDB_TRY(qcalc_alloc_work(q));
  EDB_CUDA(cudaMemcpy(q->B64, host_B, sizeof(double) * NQ * NQ, cudaMemcpyHostToDevice));
  if (!q->B2) EDB_TRY(dalloc(&q->B2, (size_t)NQ * NQ));
  EDB_TRY(qcalc_split_B2(q));
  EDB_CUDA(cudaStreamSynchronize(q->st));
  dfree(q->B32);  // the FP32 copy no longer matches
  q->ready = true;
  return qcalc_tune_fp64(q);
}

extern "C" edb_status edb_qcalc_copy_B(edb_qcalc *q, long long first, long long count,
                                       double *host_out) {
  if (!q || !host_out) return fail(EDB_EINVAL, "null argument");
  if (!q->ready) return fail(EDB_ENOTREADY, "genB has not run");
  if (!q->B64) return fail(EDB_ENOTREADY, "the full table was not built (genB_compact)");
  const long long total = q->p.NQ * q->p.NQ;
  if (first < 0 || count < 0 || first + count > total) return fail(EDB_EINVAL, "range out of table");
  EDB_CUDA(cudaMemcpy(host_out, q->B64 + first, sizeof(double) * count, cudaMemcpyDeviceToHost));
  return EDB_OK;
}

extern "C" edb_status edb_qcalc_get_info(edb_qcalc *q, edb_qcalc_info *out) {
  if (!q || !out) return fail(EDB_EINVAL, "null argument");
  out->N = q->p.N;
  out->n = q->p.n;
  out->P = q->p.P;
  out->NQ = q->p.NQ;
  out->terms = q->p.NQ * q->p.KC;
  out->B_bytes = q->p.NQ * q->p.NQ * (long long)sizeof(double);
  out->has_B32 = q->B32 != nullptr;
  return EDB_OK;
}

// The FP64 collision sum with the handle's selected kernel (the on-the-fly
// one also whenever only the compact tables exist).
static edb_status qcalc_fp64(edb_qcalc *q, const double2 *in, double2 *out, cudaStream_t st) {
  if (q->fp64_kernel == EDB_FP64_ONTHEFLY || (!q->B64 && !q->B2)) {
    if (!q->tc) return fail(EDB_ENOTREADY, "the on-the-fly kernel's tables were not built");
    EDB_TRY(launch_split_f(q->p.NQ, in, q->fdf, st));
    return launch_calq64f(q->p, q->d.filter, q->amax, q->tc, q->bs, q->fdf, q->partial, out, st);
  }
  if (q->fp64_kernel == EDB_FP64_EMULATED && q->B2) {
    return launch_calq64x(q->p, q->B2, in, q->fdf, q->partial, out, st, q->c64x_shape,
                          qcalc_b2_paired(q));
  }
  return launch_calq64(q->p, q->B64, in, q->partial, out, st);
}

extern "C" edb_status edb_qcalc_set_fp64_kernel(edb_qcalc *q, int kind) {
  if (!q) return fail(EDB_EINVAL, "null handle");
  if (kind != EDB_FP64_EMULATED && kind != EDB_FP64_NATIVE && kind != EDB_FP64_ONTHEFLY)
    return fail(EDB_EINVAL, "unknown kind");
  q->fp64_kernel = kind;
  return EDB_OK;
}

extern "C" edb_status edb_qcalc_fp64_shape(edb_qcalc *q, int shape, int *current) {
  if (!q) return fail(EDB_EINVAL, "null handle");
  if (shape >= calq64x_shapes()) return fail(EDB_EINVAL, "unknown launch shape");
  if (shape >= 0) q->c64x_shape = shape;
  if (current) *current = q->c64x_shape;
  return EDB_OK;
}

extern "C" edb_status edb_qcalc_calQ_device(edb_qcalc *q, const double *d_fin, double *d_Qout,
                                            void *stream) {
  if (!q || !d_fin || !d_Qout) return fail(EDB_EINVAL, "null argument");
  if (!q->ready) return fail(EDB_ENOTREADY, "calQ before genB");
  return qcalc_fp64(q, (const double2 *)d_fin, (double2 *)d_Qout, (cudaStream_t)stream);
}

extern "C" edb_status edb_qcalc_calQ(edb_qcalc *q, const double *fin, double *Qout) {
  if (!q || !fin || !Qout) return fail(EDB_EINVAL, "null argument");
  if (!q->ready) return fail(EDB_ENOTREADY, "calQ before genB");
  const size_t bytes = sizeof(double2) * q->p.NQ;
  EDB_CUDA(cudaMemcpyAsync(q->fin, fin, bytes, cudaMemcpyHostToDevice, q->st));
  EDB_TRY(qcalc_fp64(q, q->fin, q->Q, q->st));
  EDB_CUDA(cudaMemcpyAsync(Qout, q->Q, bytes, cudaMemcpyDeviceToHost, q->st));
  EDB_CUDA(cudaStreamSynchronize(q->st));
  return check_device_waits("calQ");
}

extern "C" edb_status edb_qcalc_calQ_batch_f32_device(edb_qcalc *q, int S, const float *d_fin,
                                                      float *d_Qout, void *stream) {
  if (!q || !d_fin || !d_Qout) return fail(EDB_EINVAL, "null argument");
  if (S < 1) return fail(EDB_EINVAL, "S must be positive");
  if (q->d.index_mode != EDB_INDEX_ALIASED)
    return fail(EDB_EINVAL, "the batched path runs the ALIASED index mode");
  if (!q->B32) return fail(EDB_ENOTREADY, "batched calQ before genB");
  const int v = c32_variant_for(q, S);
  if (calq32_pair(v)) EDB_TRY(qcalc_pairs(q, S));
  return launch_calq32_batch(q->d.N, S, q->B32, (const float2 *)d_fin, (float2 *)d_Qout,
                             (cudaStream_t)stream, v, 1, nullptr, q->pairs);
}

// Times every variant of the batched kernel on the caller's buffers (chunk
// count C, partial buffer for C > 1; two launches each after one warm-up,
// CUDA events on `st`) and records the fastest for S's class.  The pair
// variants take part when the caller passes a pair buffer.
static edb_status autotune_c32(edb_qcalc *q, int S, const float2 *d_fin, float2 *d_Qout,
                               cudaStream_t st, int C, float4 *d_partial, float4 *d_pairs,
                               int *chosen, int persist = -1) {
  cudaEvent_t e0, e1;
  EDB_CUDA(cudaEventCreate(&e0));
  EDB_CUDA(cudaEventCreate(&e1));
  int best = 0;
  float best_ms = 1e30f;
  edb_status rc = EDB_OK;
  for (int v = 0; v < calq32_variants() && rc == EDB_OK; ++v) {
    if (calq32_pair(v) && !d_pairs) continue;
    if (calq32_group(v) < 16 && S > 64) continue;  // small groups are for few solves
    rc = launch_calq32_batch(q->d.N, S, q->B32, d_fin, d_Qout, st, v, C, d_partial, d_pairs,
                             persist);
    if (rc == EDB_EINVAL) {  // this variant does not fit this N: skip it
      rc = EDB_OK;
      continue;
    }
    if (rc != EDB_OK) break;
    cudaEventRecord(e0, st);
    for (int r = 0; r < 2 && rc == EDB_OK; ++r)
      rc = launch_calq32_batch(q->d.N, S, q->B32, d_fin, d_Qout, st, v, C, d_partial, d_pairs,
                               persist);
    cudaEventRecord(e1, st);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "autotune");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_ms) {
      best_ms = ms;
      best = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != EDB_OK) return rc;
  (C > 1 ? q->c32_variant_split : q->c32_variant)[s_bucket(S)] = best;
  if (chosen) *chosen = best;
  return EDB_OK;
}

namespace edb {
edb_status qcalc_autotune_split(edb_qcalc *q, int S, const float2 *d_fin, float2 *d_Qout,
                                cudaStream_t st, int C, float4 *d_partial) {
  // the serving engine launches persistent grids (see launch_calq32_batch)
  return autotune_c32(q, S, d_fin, d_Qout, st, C, d_partial, nullptr, nullptr, 1);
}
}  // namespace edb

extern "C" int edb_qcalc_batch_variants(void) { return calq32_variants(); }
extern "C" int edb_qcalc_fp64_shapes(void) { return calq64x_shapes(); }

extern "C" edb_status edb_qcalc_calQ_batch_f32_ex(edb_qcalc *q, int S, int variant, int chunks,
                                                  void *d_partial, const float *d_fin,
                                                  float *d_Qout, void *stream) {
  if (!q || !d_fin || !d_Qout) return fail(EDB_EINVAL, "null argument");
  if (S < 1) return fail(EDB_EINVAL, "S must be positive");
  if (variant < 0 || variant >= calq32_variants()) return fail(EDB_EINVAL, "unknown variant");
  if (chunks < 1 || chunks > q->d.N) return fail(EDB_EINVAL, "chunks must be in [1, N]");
  if (chunks > 1 && !d_partial) return fail(EDB_EINVAL, "chunks > 1 need a partial buffer");
  if (!q->B32) return fail(EDB_ENOTREADY, "batched calQ before genB");
  if (calq32_pair(variant)) EDB_TRY(qcalc_pairs(q, S));
  return launch_calq32_batch(q->d.N, S, q->B32, (const float2 *)d_fin, (float2 *)d_Qout,
                             (cudaStream_t)stream, variant, chunks, (float4 *)d_partial,
                             q->pairs);
}

// Table entries of a grouped launch (checked), and the variant the auto rule
// picks: the heaviest table's autotuned variant for its S (a pair variant's
// plain twin), else 4.
static edb_status multi_inputs(int ntab, edb_qcalc *const *qs, const int *S,
                               const float *const *d_fin, float *const *d_Qout, C32MultiIn *in,
                               int *auto_variant) {
  if (ntab < 1 || ntab > 16) return fail(EDB_EINVAL, "1 to 16 tables per launch");
  if (!qs || !S || !d_fin || !d_Qout) return fail(EDB_EINVAL, "null argument");
  double heaviest = -1.0;
  *auto_variant = 4;
  for (int i = 0; i < ntab; ++i) {
    if (!qs[i] || !d_fin[i] || !d_Qout[i]) return fail(EDB_EINVAL, "null table entry");
    if (S[i] < 1) return fail(EDB_EINVAL, "S must be positive");
    if (!qs[i]->B32) return fail(EDB_ENOTREADY, "grouped calQ before genB (ALIASED)");
    const int N = qs[i]->d.N;
    if (N % 4) return fail(EDB_EINVAL, "grouped calQ needs N % 4 == 0");
    in[i] = C32MultiIn{N, S[i], qs[i]->B32, (const float2 *)d_fin[i], (float2 *)d_Qout[i]};
    const double work = (double)S[i] * std::pow((double)N, 6.0);
    if (work > heaviest) {
      heaviest = work;
      bool tuned = false;
      const int v = qcalc_c32_variant(qs[i], S[i], &tuned, false);
      *auto_variant = !tuned ? 4 : (calq32_pair(v) ? v - 5 : v);
    }
  }
  return EDB_OK;
}

extern "C" edb_status edb_qcalc_calQ_batch_multi(int ntab, edb_qcalc *const *qs, const int *S,
                                                 const float *const *d_fin,
                                                 float *const *d_Qout, int variant,
                                                 void *stream) {
  C32MultiIn in[16];
  int v = 4;
  EDB_TRY(multi_inputs(ntab, qs, S, d_fin, d_Qout, in, &v));
  if (variant >= 0) v = variant;
  return launch_calq32_multi(ntab, in, v, (cudaStream_t)stream);
}

extern "C" edb_status edb_qcalc_autotune_batch_multi(int ntab, edb_qcalc *const *qs,
                                                     const int *S, const float *const *d_fin,
                                                     float *const *d_Qout, void *stream,
                                                     int *chosen) {
  if (!chosen) return fail(EDB_EINVAL, "null output");
  C32MultiIn in[16];
  int v0 = 4;
  EDB_TRY(multi_inputs(ntab, qs, S, d_fin, d_Qout, in, &v0));
  const cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t e0, e1;
  EDB_CUDA(cudaEventCreate(&e0));
  EDB_CUDA(cudaEventCreate(&e1));
  int best = -1;
  float best_ms = 1e30f;
  edb_status rc = EDB_OK;
  for (int v = 0; v < calq32_variants() && rc == EDB_OK; ++v) {
    if (calq32_pair(v)) continue;
    rc = launch_calq32_multi(ntab, in, v, st);  // warm-up; EINVAL: does not fit
    if (rc == EDB_EINVAL) {
      rc = EDB_OK;
      continue;
    }
    if (rc != EDB_OK) break;
    cudaEventRecord(e0, st);
    for (int r = 0; r < 2 && rc == EDB_OK; ++r) rc = launch_calq32_multi(ntab, in, v, st);
    cudaEventRecord(e1, st);
    const cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "grouped autotune");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_ms) {
      best_ms = ms;
      best = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != EDB_OK) return rc;
  if (best < 0) return fail(EDB_EINVAL, "no variant fits these tables");
  *chosen = best;
  return EDB_OK;
}

extern "C" edb_status edb_qcalc_autotune_batch(edb_qcalc *q, int S, const float *d_fin,
                                               float *d_Qout, void *stream, int *chosen) {
  if (!q || !d_fin || !d_Qout) return fail(EDB_EINVAL, "null argument");
  if (S < 1) return fail(EDB_EINVAL, "S must be positive");
  if (!q->B32) return fail(EDB_ENOTREADY, "autotune before genB (ALIASED)");
  EDB_TRY(qcalc_pairs(q, S));
  return autotune_c32(q, S, (const float2 *)d_fin, (float2 *)d_Qout, (cudaStream_t)stream, 1,
                      nullptr, q->pairs, chosen);
}

extern "C" edb_status edb_device_status(int *status, int clear) {
  if (!status) return fail(EDB_EINVAL, "null output");
  int a = 0, b = 0;
  EDB_TRY(read_calq32_status(&a, clear != 0));
  EDB_TRY(read_calq64x_status(&b, clear != 0));
  *status = (a ? 1 : 0) | (b ? 2 : 0);
  return EDB_OK;
}

extern "C" edb_status edb_set_wait_limit_ns(long long ns) {
  g_wait_ns.store(ns < 0 ? kDefaultWaitNs : (unsigned long long)ns, std::memory_order_relaxed);
  return EDB_OK;
}

// ===================================================================== fft3d

static edb_status fft_host(int nx, int ny, int nz, const double *in, double *out, int inverse) {
  if (!in || !out) return fail(EDB_EINVAL, "null argument");
  if (nx != ny || ny != nz) return fail(EDB_EINVAL, "fft3d: cubes only (fft3d.h:43)");
  EDB_TRY(ensure_device());
  const int N = nx;
  const size_t bytes = sizeof(double2) * (size_t)N * N * N;
  double2 *a = nullptr, *b = nullptr;
  EDB_TRY(dalloc(&a, (size_t)N * N * N));
  edb_status s = dalloc(&b, (size_t)N * N * N);
  if (s == EDB_OK) {
    cudaError_t e = cudaMemcpy(a, in, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) s = cuda_fail(e, "cudaMemcpy");
  }
  if (s == EDB_OK) s = launch_dft3d(N, 1, a, b, nullptr, inverse, 0, 0);
  if (s == EDB_OK) {
    cudaError_t e = cudaMemcpy(out, b, bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) s = cuda_fail(e, "cudaMemcpy");
  }
  dfree(a);
  dfree(b);
  return s;
}

extern "C" edb_status edb_fft3d_fft(int nx, int ny, int nz, const double *re, double *fre) {
  return fft_host(nx, ny, nz, re, fre, 0);
}
extern "C" edb_status edb_fft3d_ifft(int nx, int ny, int nz, double *re, const double *fre) {
  return fft_host(nx, ny, nz, fre, re, 1);
}
extern "C" edb_status edb_fft3d_device(int N, int batch, const void *d_in, void *d_out,
                                       int inverse, int fp32, void *stream) {
  if (!d_in || !d_out || batch < 1) return fail(EDB_EINVAL, "bad argument");
  if (fp32 < 0 || fp32 > EDB_DFT_DOUBLE_FLOAT) return fail(EDB_EINVAL, "unknown arithmetic mode");
  return launch_dft3d(N, batch, d_in, d_out, nullptr, inverse, fp32, (cudaStream_t)stream);
}

// ================================================================ EntropyFix

struct edb_efix {
  int Nt;
  double eps;
  EfixState *st = nullptr;
  double *f = nullptr, *H = nullptr;
};

extern "C" edb_status edb_efix_create(int Nt, double eps, edb_efix **out) {
  if (!out) return fail(EDB_EINVAL, "null output pointer");
  *out = nullptr;
  if (Nt < 1) return fail(EDB_EINVAL, "Nt must be positive");
  EDB_TRY(ensure_device());
  edb_efix *e = new edb_efix();
  e->Nt = Nt;
  e->eps = eps;
  edb_status s = dalloc(&e->st, 1);
  if (s == EDB_OK) s = dalloc(&e->f, (size_t)Nt);
  if (s == EDB_OK) s = dalloc(&e->H, 1);
  if (s == EDB_OK) {
    EfixState init = {1.0, 0, 0, 1.0, 0, 0};  // Averagef = 1.0, flag false (EntropyFix.h:20-22)
    cudaError_t ce = cudaMemcpy(e->st, &init, sizeof(init), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) s = cuda_fail(ce, "cudaMemcpy");
  }
  if (s != EDB_OK) {
    dfree(e->st);
    dfree(e->f);
    dfree(e->H);
    delete e;
    return s;
  }
  *out = e;
  return EDB_OK;
}

extern "C" edb_status edb_efix_destroy(edb_efix *e) {
  if (!e) return EDB_OK;
  dfree(e->st);
  dfree(e->f);
  dfree(e->H);
  delete e;
  return EDB_OK;
}

static edb_status efix_check(edb_efix *e, int Nf, const double *f) {
  if (!e || !f) return fail(EDB_EINVAL, "null argument");
  // the reference asserts Nf == Nt (EntropyFix.h:68, 127, 214)
  if (Nf != e->Nt) return fail(EDB_EINVAL, "Nf must equal Nt");
  return EDB_OK;
}

extern "C" edb_status edb_efix_set_average(edb_efix *e, int Nf, const double *f) {
  EDB_TRY(efix_check(e, Nf, f));
  EDB_CUDA(cudaMemcpy(e->f, f, sizeof(double) * Nf, cudaMemcpyHostToDevice));
  EDB_TRY(launch_efix_average(Nf, e->f, e->st, 0));
  EDB_CUDA(cudaDeviceSynchronize());
  return EDB_OK;
}

extern "C" edb_status edb_efix_entropy(edb_efix *e, int Nf, const double *f, double *H) {
  EDB_TRY(efix_check(e, Nf, f));
  if (!H) return fail(EDB_EINVAL, "null output");
  EDB_CUDA(cudaMemcpy(e->f, f, sizeof(double) * Nf, cudaMemcpyHostToDevice));
  EDB_TRY(launch_efix_entropy(Nf, e->f, e->st, e->eps, e->H, 0));
  EDB_CUDA(cudaMemcpy(H, e->H, sizeof(double), cudaMemcpyDeviceToHost));
  return EDB_OK;
}

extern "C" edb_status edb_efix_fixsol(edb_efix *e, int Nf, double *f, double aim) {
  EDB_TRY(efix_check(e, Nf, f));
  EDB_CUDA(cudaMemcpy(e->f, f, sizeof(double) * Nf, cudaMemcpyHostToDevice));
  EDB_TRY(launch_efix_fixsol(Nf, e->f, e->st, e->eps, aim, 0));
  EDB_CUDA(cudaMemcpy(f, e->f, sizeof(double) * Nf, cudaMemcpyDeviceToHost));
  return EDB_OK;
}

extern "C" edb_status edb_efix_get_average(edb_efix *e, double *avg, int *latched) {
  if (!e) return fail(EDB_EINVAL, "null handle");
  EfixState h;
  EDB_CUDA(cudaMemcpy(&h, e->st, sizeof(h), cudaMemcpyDeviceToHost));
  if (avg) *avg = h.avg;
  if (latched) *latched = h.avg_flag;
  return EDB_OK;
}

// ================================================================ integrator

struct edb_solver {
  edb_solver_desc d;
  edb_qcalc *q = nullptr;
  cudaStream_t st = nullptr;
  long long NQ = 0;
  double2 *F = nullptr, *Fhat = nullptr, *Fold = nullptr;
  double2 *Qs[4] = {nullptr, nullptr, nullptr, nullptr};
  double2 *Fs[3] = {nullptr, nullptr, nullptr};
  EfixState *state = nullptr;
  double *tr_raw = nullptr, *tr_fixed = nullptr;
  int trace_cap = 0, trace_n = 0;
  bool has_initial = false;
  std::vector<double> F0;
  // conservative mode: moment table, initial moments, forward-DFT scratch
  double *ctab = nullptr, *m0 = nullptr;
  double2 *tmp = nullptr;
  // record_F: Re F after every step (hist_cap rows of N^3) and the step times
  double *hist = nullptr;
  int hist_cap = 0;
  std::vector<double> times;
};

extern "C" edb_status edb_solver_create(const edb_solver_desc *d, edb_solver **out) {
  if (!d || !out) return fail(EDB_EINVAL, "null argument");
  *out = nullptr;
  if (d->scheme < EDB_SCHEME_FE || d->scheme > EDB_SCHEME_DUFORT)
    return fail(EDB_EINVAL, "unknown scheme");
  if (d->kernel.N != d->N) return fail(EDB_EINVAL, "kernel.N must equal N");
  if (!(d->R > 0)) return fail(EDB_EINVAL, "R must be positive");
  edb_solver *s = new edb_solver();
  s->d = *d;
  s->NQ = (long long)d->N * d->N * d->N;
  edb_status rc = edb_qcalc_create(&d->kernel, &s->q);
  if (rc == EDB_OK) rc = edb_qcalc_genB(s->q);
  if (rc == EDB_OK) {
    cudaError_t e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaStreamCreate");
  }
  const size_t NQ = (size_t)s->NQ;
  if (rc == EDB_OK) rc = dalloc(&s->F, NQ);
  if (rc == EDB_OK) rc = dalloc(&s->Fhat, NQ);
  if (rc == EDB_OK) rc = dalloc(&s->Fold, NQ);
  for (int i = 0; i < 4 && rc == EDB_OK; ++i) rc = dalloc(&s->Qs[i], NQ);
  for (int i = 0; i < 3 && rc == EDB_OK; ++i) rc = dalloc(&s->Fs[i], NQ);
  if (rc == EDB_OK) rc = dalloc(&s->state, 1);
  if (rc == EDB_OK && d->conserve) {
    rc = upload_conserve_table(d->N, d->R, &s->ctab);
    if (rc == EDB_OK) rc = dalloc(&s->m0, 5);
    if (rc == EDB_OK) rc = dalloc(&s->tmp, NQ);
  }
  if (rc != EDB_OK) {
    edb_solver_destroy(s);
    return rc;
  }
  *out = s;
  return EDB_OK;
}

extern "C" edb_status edb_solver_destroy(edb_solver *s) {
  if (!s) return EDB_OK;
  if (s->st) cudaStreamSynchronize(s->st);
  dfree(s->F);
  dfree(s->Fhat);
  dfree(s->Fold);
  for (auto &p : s->Qs) dfree(p);
  for (auto &p : s->Fs) dfree(p);
  dfree(s->state);
  dfree(s->tr_raw);
  dfree(s->tr_fixed);
  dfree(s->ctab);
  dfree(s->m0);
  dfree(s->tmp);
  dfree(s->hist);
  if (s->q) edb_qcalc_destroy(s->q);
  if (s->st) cudaStreamDestroy(s->st);
  delete s;
  return EDB_OK;
}

extern "C" edb_status edb_solver_set_initial(edb_solver *s, const double *F0) {
  if (!s) return fail(EDB_EINVAL, "null handle");
  if (F0)
    for (long long i = 0; i < 2 * s->NQ; ++i)
      if (!std::isfinite(F0[i]))
        return fail(EDB_EINVAL, "initial data contains a NaN or an infinity");
  if (F0)
    s->F0.assign(F0, F0 + 2 * s->NQ);
  else
    s->F0.clear();
  s->has_initial = true;
  return EDB_OK;
}

// Step counts of `do { t += dt; ... } while (t < TEnd)` with the reference's
// floating accumulation (BKW.h:218-248); DUFORT adds 8 RK2 start-up steps
// that advance t by dt/8 (:547-587).
static int count_steps(int scheme, double T0, double TEnd, double dt) {
  double t = T0;
  int n = 0;
  if (scheme == EDB_SCHEME_DUFORT) {
    for (int i = 0; i < 8; ++i) t += dt / 8;
    n = 8;
  }
  do {
    t += dt;
    ++n;
  } while (t < TEnd && n < 100000000);
  return n;
}

// One step of the chosen scheme on the device (the loop bodies of BKW.h).
static edb_status solver_step(edb_solver *s, double dt, bool dufort_startup) {
  const long long n = s->NQ;
  cudaStream_t st = s->st;
  edb_qcalc *q = s->q;
  double2 *Fh = s->Fhat, **Q = s->Qs, **F = s->Fs;
  auto calq = [&](const double2 *in, double2 *out) { return qcalc_fp64(q, in, out, st); };
  switch (s->d.scheme) {
    case EDB_SCHEME_FE:  // BKW.h:220-222
      EDB_TRY(calq(Fh, Q[0]));
      EDB_TRY(launch_stage(n, STAGE_AXPY, 0, dt, 0, Fh, Fh, 0, 0, Q[0], 0, 0, 0, 0, st));
      break;
    case EDB_SCHEME_CFE: {  // BKW.h:281-283
      const double beta = s->d.beta;
      EDB_TRY(calq(Fh, Q[0]));
      EDB_TRY(launch_stage(n, STAGE_AXPY, 0, (1. - exp(-beta * dt)) / beta, 0, Fh, Fh, 0, 0, Q[0],
                           0, 0, 0, 0, st));
      break;
    }
    case EDB_SCHEME_RK2:  // BKW.h:341-346
      EDB_TRY(calq(Fh, Q[0]));
      EDB_TRY(launch_stage(n, STAGE_AXPY, 0, 0.5 * dt, 0, F[0], Fh, 0, 0, Q[0], 0, 0, 0, 0, st));
      EDB_TRY(calq(F[0], Q[0]));
      EDB_TRY(launch_stage(n, STAGE_AXPY, 0, dt, 0, Fh, Fh, 0, 0, Q[0], 0, 0, 0, 0, st));
      break;
    case EDB_SCHEME_SSP3:  // BKW.h:416-424
      EDB_TRY(calq(Fh, Q[0]));
      EDB_TRY(launch_stage(n, STAGE_AXPY, 0, dt, 0, F[0], Fh, 0, 0, Q[0], 0, 0, 0, 0, st));
      EDB_TRY(calq(F[0], Q[0]));
      EDB_TRY(launch_stage(n, STAGE_SSP3_2, 0, 0.25 * dt, 0, F[1], Fh, F[0], 0, Q[0], 0, 0, 0, 0,
                           st));
      EDB_TRY(calq(F[1], Q[0]));
      EDB_TRY(launch_stage(n, STAGE_SSP3_3, 0, 2. / 3. * dt, 0, Fh, Fh, F[1], 0, Q[0], 0, 0, 0, 0,
                           st));
      break;
    case EDB_SCHEME_RK4:  // BKW.h:482-494
      EDB_TRY(calq(Fh, Q[0]));
      EDB_TRY(launch_stage(n, STAGE_AXPY, 0, 0.5 * dt, 0, F[0], Fh, 0, 0, Q[0], 0, 0, 0, 0, st));
      EDB_TRY(calq(F[0], Q[1]));
      EDB_TRY(launch_stage(n, STAGE_AXPY, 0, 0.5 * dt, 0, F[1], Fh, 0, 0, Q[1], 0, 0, 0, 0, st));
      EDB_TRY(calq(F[1], Q[2]));
      EDB_TRY(launch_stage(n, STAGE_AXPY, 0, dt, 0, F[2], Fh, 0, 0, Q[2], 0, 0, 0, 0, st));
      EDB_TRY(calq(F[2], Q[3]));
      EDB_TRY(launch_stage(n, STAGE_RK4, 0, dt / 6., 0, Fh, Fh, 0, 0, Q[0], Q[1], Q[2], Q[3], 0,
                           st));
      break;
    case EDB_SCHEME_DUFORT:
      if (dufort_startup) {  // BKW.h:551-556 (updates use dt, not dt/8)
        EDB_TRY(calq(Fh, Q[0]));
        EDB_TRY(
            launch_stage(n, STAGE_AXPY, 0, 0.5 * dt, 0, F[0], Fh, 0, 0, Q[0], 0, 0, 0, 0, st));
        EDB_TRY(calq(F[0], Q[0]));
        EDB_TRY(launch_stage(n, STAGE_AXPY, 0, dt, 0, Fh, Fh, 0, 0, Q[0], 0, 0, 0, 0, st));
      } else {  // BKW.h:595-598, then F_old = F1 (:630)
        const double beta = s->d.beta;
        EDB_TRY(calq(Fh, Q[0]));
        EDB_CUDA(cudaMemcpyAsync(F[0], Fh, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
        EDB_TRY(launch_stage(n, STAGE_DUFORT, 1. / (1. + beta * dt), dt, beta * dt, Fh, 0, F[0],
                             s->Fold, Q[0], 0, 0, 0, 0, st));
      }
      break;
  }
  // conservative mode: back onto the initial moments
  if (s->d.conserve) EDB_TRY(launch_project_moments(s->d.N, 1, s->ctab, Fh, s->m0, st));
  // fft3(isInverse) then calEntropy and the fix rule
  EDB_TRY(launch_dft3d(s->d.N, 1, Fh, s->F, nullptr, 1, 0, st));
  int fix_mode = 0;
  if (s->d.scheme == EDB_SCHEME_FE) fix_mode = s->d.fix_entropy ? 1 : 0;
  else if (s->d.scheme == EDB_SCHEME_CFE) fix_mode = s->d.fix_entropy ? 2 : 0;
  else if (s->d.scheme == EDB_SCHEME_SSP3 || s->d.scheme == EDB_SCHEME_RK4) fix_mode = 2;
  if (s->d.conserve) {
    // moment-preserving fix, fed back into Fhat
    EDB_TRY(launch_step_entropy_conserve(s->d.N, 1, s->d.R, s->F, s->state, 1.0e-10, fix_mode,
                                         s->tr_raw, s->tr_fixed, s->trace_cap, st));
    EDB_TRY(launch_dft3d(s->d.N, 1, s->F, s->tmp, nullptr, 0, 0, st));
    EDB_TRY(launch_masked_copy(n, 1, s->state, s->tmp, Fh, st));
  } else {
    EDB_TRY(launch_step_entropy(s->d.N, 1, s->d.R, s->F, s->state, 1.0e-10, fix_mode, s->tr_raw,
                                s->tr_fixed, s->trace_cap, st));
  }
  if (s->d.scheme == EDB_SCHEME_DUFORT && !dufort_startup)
    EDB_CUDA(cudaMemcpyAsync(s->Fold, F[0], sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
  if (s->hist) EDB_TRY(launch_record_re(n, s->F, s->state, s->hist, s->hist_cap, st));
  return EDB_OK;
}

extern "C" edb_status edb_solver_run(edb_solver *s, double T0, double TEnd, double dt,
                                     int *nsteps) {
  if (!s) return fail(EDB_EINVAL, "null handle");
  if (!(dt > 0)) return fail(EDB_EINVAL, "dt must be positive");
  const int total = count_steps(s->d.scheme, T0, TEnd, dt);
  const long long n = s->NQ;
  cudaStream_t st = s->st;
  dfree(s->tr_raw);
  dfree(s->tr_fixed);
  s->trace_cap = total;
  EDB_TRY(dalloc(&s->tr_raw, (size_t)total));
  EDB_TRY(dalloc(&s->tr_fixed, (size_t)total));
  dfree(s->hist);
  s->hist_cap = 0;
  if (s->d.record_F) {
    EDB_TRY(dalloc(&s->hist, (size_t)total * (size_t)n));
    s->hist_cap = total;
  }
  // the step times of the reference loop (t += dt; DUFORT's start-up steps dt/8)
  s->times.clear();
  {
    double t = T0;
    if (s->d.scheme == EDB_SCHEME_DUFORT)
      for (int i = 0; i < 8; ++i) s->times.push_back(t += dt / 8);
    while ((int)s->times.size() < total) s->times.push_back(t += dt);
  }
  // initial data -> F, Fhat = fft(F) (BKW.h:197-198)
  if (s->has_initial && !s->F0.empty())
    EDB_CUDA(cudaMemcpyAsync(s->F, s->F0.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, st));
  else
    EDB_TRY(launch_sinusoid_init(s->d.N, s->d.R, s->F, st));
  EDB_TRY(launch_dft3d(s->d.N, 1, s->F, s->Fhat, nullptr, 0, 0, st));
  if (s->d.conserve) EDB_TRY(launch_hat_moments(s->d.N, 1, s->ctab, s->Fhat, s->m0, st));
  if (s->d.scheme == EDB_SCHEME_DUFORT)
    EDB_CUDA(cudaMemcpyAsync(s->Fold, s->Fhat, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
  // entropy0 and the step counter: FE starts from calEntropy() and step 1
  // (BKW.h:214-216); the others from 1. and step 0.
  EfixState init = {1.0, 0, 0, 1.0, 0, 0};
  EDB_CUDA(cudaMemcpyAsync(s->state, &init, sizeof(init), cudaMemcpyHostToDevice, st));
  // conservative mode also starts from the initial entropy, so the fix can
  // act from the first step
  if (s->d.scheme == EDB_SCHEME_FE || s->d.conserve) {
    EDB_TRY(launch_calentropy(s->d.N, 1, s->d.R, s->F, &s->state->H_prev, st));
    int one = 1;
    EDB_CUDA(cudaMemcpyAsync(&s->state->step, &one, sizeof(int), cudaMemcpyHostToDevice, st));
  }
  EDB_CUDA(cudaStreamSynchronize(st));
  int done = 0;
  if (s->d.scheme == EDB_SCHEME_DUFORT) {
    for (int i = 0; i < 8; ++i, ++done) EDB_TRY(solver_step(s, dt, true));
    // step counter restarts at 0 (BKW.h:592); it gates no fix for DUFORT
  }
  // The steady-state step is captured once as a CUDA graph and replayed.
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const int remaining = total - done;
  if (remaining > 0) {
    EDB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    edb_status rc = solver_step(s, dt, false);
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (rc != EDB_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(graph);
      return cuda_fail(e, "cudaGraphInstantiate");
    }
    for (int i = 0; i < remaining; ++i) {
      e = cudaGraphLaunch(exec, st);
      if (e != cudaSuccess) break;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
  }
  EDB_CUDA(cudaStreamSynchronize(st));
  s->trace_n = total;
  if (nsteps) *nsteps = total;
  return check_device_waits("solver run");
}

extern "C" edb_status edb_solver_get(edb_solver *s, double *Fhat, double *F) {
  if (!s) return fail(EDB_EINVAL, "null handle");
  const size_t bytes = sizeof(double2) * s->NQ;
  if (Fhat) EDB_CUDA(cudaMemcpy(Fhat, s->Fhat, bytes, cudaMemcpyDeviceToHost));
  if (F) EDB_CUDA(cudaMemcpy(F, s->F, bytes, cudaMemcpyDeviceToHost));
  return EDB_OK;
}

extern "C" edb_status edb_solver_trace(edb_solver *s, double *raw, double *fixed, int cap, int *n) {
  if (!s) return fail(EDB_EINVAL, "null handle");
  int k = s->trace_n < cap ? s->trace_n : cap;
  if (k > 0 && raw) EDB_CUDA(cudaMemcpy(raw, s->tr_raw, sizeof(double) * k, cudaMemcpyDeviceToHost));
  if (k > 0 && fixed)
    EDB_CUDA(cudaMemcpy(fixed, s->tr_fixed, sizeof(double) * k, cudaMemcpyDeviceToHost));
  if (n) *n = s->trace_n;
  return EDB_OK;
}

extern "C" edb_status edb_solver_F_history(edb_solver *s, double *out, int cap, int *n) {
  if (!s) return fail(EDB_EINVAL, "null handle");
  if (!s->hist) return fail(EDB_ENOTREADY, "run with record_F = 1 first");
  const int k = s->trace_n < cap ? s->trace_n : cap;
  if (k > 0 && out)
    EDB_CUDA(cudaMemcpy(out, s->hist, sizeof(double) * (size_t)k * s->NQ, cudaMemcpyDeviceToHost));
  if (n) *n = s->trace_n;
  return EDB_OK;
}

extern "C" edb_status edb_solver_write_F_dat(edb_solver *s, const char *path) {
  if (!s || !path) return fail(EDB_EINVAL, "null argument");
  if (!s->hist) return fail(EDB_ENOTREADY, "run with record_F = 1 first");
  const int rows = s->trace_n < s->hist_cap ? s->trace_n : s->hist_cap;
  std::vector<double> h((size_t)rows * s->NQ);
  if (rows > 0)
    EDB_CUDA(cudaMemcpy(h.data(), s->hist, sizeof(double) * h.size(), cudaMemcpyDeviceToHost));
  // BKW.h:217-249: t, then every Re F, tab-separated, default stream format
  std::ofstream writeF(path);
  if (!writeF) return fail(EDB_EINVAL, std::string("cannot open ") + path);
  for (int r = 0; r < rows; ++r) {
    writeF << s->times[(size_t)r] << "\t";
    for (long long i = 0; i < s->NQ; ++i) writeF << h[(size_t)r * s->NQ + i] << "\t";
    writeF << "\n";
  }
  writeF.close();
  return writeF ? EDB_OK : fail(EDB_EINVAL, std::string("write failed: ") + path);
}

extern "C" edb_status edb_solver_out_v1_direction(edb_solver *s, const char *path) {
  if (!s || !path) return fail(EDB_EINVAL, "null argument");
  const int N0 = s->d.N;
  const double R = s->d.R;
  const double h = 2. * R / double(N0);
  std::vector<double> x((size_t)N0), fval((size_t)N0), F(2 * (size_t)s->NQ);
  for (int i = 0; i < N0; ++i) x[(size_t)i] = -R + i * h;
  double *d = nullptr;
  EDB_TRY(dalloc(&d, 2 * (size_t)N0));
  cudaError_t e = cudaMemcpy(d, x.data(), sizeof(double) * N0, cudaMemcpyHostToDevice);
  edb_status rc = e == cudaSuccess
                      ? launch_funexact_points(R, N0, d, h / 2, h / 2, d + N0, s->st)
                      : cuda_fail(e, "outV1Direction");
  if (rc == EDB_OK) {
    e = cudaMemcpyAsync(fval.data(), d + N0, sizeof(double) * N0, cudaMemcpyDeviceToHost, s->st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(F.data(), s->F, sizeof(double2) * s->NQ, cudaMemcpyDeviceToHost, s->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) rc = cuda_fail(e, "outV1Direction");
  }
  dfree(d);
  if (rc != EDB_OK) return rc;
  // BKW.h:163-180
  std::ofstream write(path);
  if (!write) return fail(EDB_EINVAL, std::string("cannot open ") + path);
  write << "# x\tf(t)\tf_0\n";
  for (int i = 0; i < N0; ++i) {
    const long long l = ((long long)i * N0 + N0 / 2) * N0 + N0 / 2;
    write << std::fixed << std::setprecision(8) << x[(size_t)i] << "\t" << F[2 * (size_t)l] << "\t"
          << fval[(size_t)i] << "\n";
  }
  write.close();
  return write ? EDB_OK : fail(EDB_EINVAL, std::string("write failed: ") + path);
}

// ============================================================ batched solves

struct edb_batch {
  edb_batch_desc d;
  edb_qcalc *q = nullptr;
  cudaStream_t st = nullptr;  // internal stream used when the caller passes NULL
  long long NQ = 0, n = 0;    // N^3, S*N^3
  double2 *Fhat = nullptr, *F = nullptr;
  double2 *Fs[3] = {nullptr, nullptr, nullptr};
  float2 *Qs[4] = {nullptr, nullptr, nullptr, nullptr};
  float2 *in32 = nullptr;
  float4 *pairs = nullptr;  // solve-pair copy of in32 for the pair variants
  EfixState *state = nullptr;
  EfixState *state_init = nullptr;  // the entropy bookkeeping's initial values, S copies
  double *tr_raw = nullptr, *tr_fixed = nullptr;
  double *mom = nullptr, *H = nullptr;
  double *ctab = nullptr, *m0 = nullptr;  // conservative mode
  cudaGraphExec_t exec = nullptr;
  cudaStream_t exec_stream = nullptr;
  int launches_per_step = 0;
  // F holds the real-space output of the current state: the loaded data, the
  // last step's F after the fix rule (the step computes it when the fix is
  // on), or a transform made by a reader.  The reference's output after a
  // step is that F, which its fix rewrites without touching F-hat.
  bool f_cur = false;
  // host transfers of load/read in cube chunks on their own stream, so the
  // copy of one chunk overlaps the transforms of the next
  cudaStream_t cst = nullptr;
  cudaEvent_t xev[8] = {};
  cudaEvent_t xdone = nullptr;  // the last D2H of a read (the staging buffer is free)
  // NULL-stream device calls: the batch's own (non-blocking) stream first
  // waits for the work the caller queued on the default stream
  cudaEvent_t join_ev = nullptr;
};

static constexpr int BATCH_XFER_CHUNKS = 8;

extern "C" edb_status edb_batch_create(edb_qcalc *q, const edb_batch_desc *d, edb_batch **out) {
  if (!q || !d || !out) return fail(EDB_EINVAL, "null argument");
  *out = nullptr;
  if (d->S < 1) return fail(EDB_EINVAL, "S must be positive");
  if (d->N != q->d.N) return fail(EDB_EINVAL, "batch N differs from the kernel table's N");
  if (d->scheme != EDB_SCHEME_FE && d->scheme != EDB_SCHEME_SSP3 && d->scheme != EDB_SCHEME_RK4)
    return fail(EDB_EINVAL, "batched schemes: FE, SSP3, RK4");
  if (q->d.index_mode != EDB_INDEX_ALIASED || !q->B32)
    return fail(EDB_ENOTREADY, "batched solves need an ALIASED table after genB");
  edb_batch *b = new edb_batch();
  b->d = *d;
  b->q = q;
  b->NQ = (long long)d->N * d->N * d->N;
  b->n = b->NQ * d->S;
  const size_t n = (size_t)b->n;
  edb_status rc = EDB_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) rc = cuda_fail(e, "cudaStreamCreate");
  if (rc == EDB_OK && (e = cudaStreamCreateWithFlags(&b->cst, cudaStreamNonBlocking)) != cudaSuccess)
    rc = cuda_fail(e, "cudaStreamCreate");
  for (int i = 0; i < BATCH_XFER_CHUNKS && rc == EDB_OK; ++i)
    if ((e = cudaEventCreateWithFlags(&b->xev[i], cudaEventDisableTiming)) != cudaSuccess)
      rc = cuda_fail(e, "cudaEventCreate");
  if (rc == EDB_OK &&
      (e = cudaEventCreateWithFlags(&b->join_ev, cudaEventDisableTiming)) != cudaSuccess)
    rc = cuda_fail(e, "cudaEventCreate");
  if (rc == EDB_OK &&
      (e = cudaEventCreateWithFlags(&b->xdone, cudaEventDisableTiming)) != cudaSuccess)
    rc = cuda_fail(e, "cudaEventCreate");
  if (rc == EDB_OK) rc = dalloc(&b->Fhat, n);
  if (rc == EDB_OK) rc = dalloc(&b->F, n);
  const int nstage = d->scheme == EDB_SCHEME_RK4 ? 3 : (d->scheme == EDB_SCHEME_SSP3 ? 2 : 0);
  const int nq = d->scheme == EDB_SCHEME_RK4 ? 4 : 1;
  for (int i = 0; i < nstage && rc == EDB_OK; ++i) rc = dalloc(&b->Fs[i], n);
  for (int i = 0; i < nq && rc == EDB_OK; ++i) rc = dalloc(&b->Qs[i], n);
  if (rc == EDB_OK) rc = dalloc(&b->in32, n);
  if (rc == EDB_OK) rc = dalloc(&b->pairs, calq32_pair_bytes(d->N, d->S) / sizeof(float4));
  if (rc == EDB_OK) rc = dalloc(&b->state, (size_t)d->S);
  if (rc == EDB_OK) rc = dalloc(&b->state_init, (size_t)d->S);
  if (rc == EDB_OK) {
    std::vector<EfixState> init((size_t)d->S, EfixState{1.0, 0, 0, 1.0, 0, 0});
    e = cudaMemcpy(b->state_init, init.data(), sizeof(EfixState) * d->S, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemcpy(batch state)");
  }
  if (rc == EDB_OK) rc = dalloc(&b->mom, (size_t)d->S * 5);
  if (rc == EDB_OK) rc = dalloc(&b->H, (size_t)d->S);
  if (rc == EDB_OK) rc = dalloc(&b->tr_raw, (size_t)d->S);
  if (rc == EDB_OK) rc = dalloc(&b->tr_fixed, (size_t)d->S);
  if (rc == EDB_OK && d->conserve) {
    rc = upload_conserve_table(d->N, d->R, &b->ctab);
    if (rc == EDB_OK) rc = dalloc(&b->m0, (size_t)d->S * 5);
    // the forward transform of a fixed F needs a scratch array
    if (rc == EDB_OK && nstage == 0) rc = dalloc(&b->Fs[0], n);
  }
  if (rc != EDB_OK) {
    edb_batch_destroy(b);
    return rc;
  }
  *out = b;
  return EDB_OK;
}

extern "C" edb_status edb_batch_destroy(edb_batch *b) {
  if (!b) return EDB_OK;
  if (b->cst) cudaStreamSynchronize(b->cst);
  if (b->st) cudaStreamSynchronize(b->st);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  dfree(b->Fhat);
  dfree(b->F);
  for (auto &p : b->Fs) dfree(p);
  for (auto &p : b->Qs) dfree(p);
  dfree(b->in32);
  dfree(b->pairs);
  dfree(b->state);
  dfree(b->state_init);
  dfree(b->mom);
  dfree(b->H);
  dfree(b->tr_raw);
  dfree(b->tr_fixed);
  dfree(b->ctab);
  dfree(b->m0);
  for (auto &ev : b->xev)
    if (ev) cudaEventDestroy(ev);
  if (b->join_ev) cudaEventDestroy(b->join_ev);
  if (b->xdone) cudaEventDestroy(b->xdone);
  if (b->cst) cudaStreamDestroy(b->cst);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
  return EDB_OK;
}

// transformed: Fhat already holds fft(F) (the chunked host load does it per
// chunk as the chunks arrive).
// sync = false: everything is queued on st and the call returns at once
// (after a one-time autotune, which waits).
static edb_status batch_init_state(edb_batch *b, cudaStream_t st, bool transformed = false,
                                   bool sync = true) {
  // Fhat = fft(F) in FP64, its FP32 copy, entropy bookkeeping reset
  if (!transformed)
    EDB_TRY(launch_dft3d(b->d.N, b->d.S, b->F, b->Fhat, nullptr, 0, EDB_DFT_DOUBLE_FLOAT, st));
  if (b->d.conserve) EDB_TRY(launch_hat_moments(b->d.N, b->d.S, b->ctab, b->Fhat, b->m0, st));
  EDB_TRY(launch_d2f(b->n, b->Fhat, b->in32, st));
  // pick the batched kernel's variant for this S on real data, before the
  // step graph is captured (the graph bakes the choice in)
  if (b->q->c32_variant[s_bucket(b->d.S)] < 0 && !b->exec)
    EDB_TRY(autotune_c32(b->q, b->d.S, b->in32, b->Qs[0], st, 1, nullptr, b->pairs, nullptr));
  EDB_CUDA(cudaMemcpyAsync(b->state, b->state_init, sizeof(EfixState) * b->d.S,
                           cudaMemcpyDeviceToDevice, st));
  // no step yet: the last-step entropies read as NaN (all-ones bytes)
  EDB_CUDA(cudaMemsetAsync(b->tr_raw, 0xff, sizeof(double) * b->d.S, st));
  EDB_CUDA(cudaMemsetAsync(b->tr_fixed, 0xff, sizeof(double) * b->d.S, st));
  if (b->d.conserve) {  // start the entropy rule from the initial entropy
    EDB_TRY(launch_calentropy(b->d.N, b->d.S, b->d.R, b->F, b->H, st));
    EDB_TRY(launch_state_from_entropy(b->d.S, b->H, b->state, st));
  }
  if (sync) EDB_CUDA(cudaStreamSynchronize(st));
  return EDB_OK;
}

// Between steps the first FP32 Q-hat stage array (S x N^3 float2, exactly
// S x N^3 doubles of bytes) is free; load and read stage real-space data in it.
static double *batch_staging(edb_batch *b) { return reinterpret_cast<double *>(b->Qs[0]); }

// Cube range [c0, c1) of transfer chunk i.
static void batch_chunk(const edb_batch *b, int i, int *c0, int *c1) {
  const int per = (b->d.S + BATCH_XFER_CHUNKS - 1) / BATCH_XFER_CHUNKS;
  *c0 = std::min(b->d.S, i * per);
  *c1 = std::min(b->d.S, *c0 + per);
}

// Host load: chunk copies on cst, transforms on st; sync = false returns with
// the work queued (the caller keeps F0_real unchanged until the batch syncs).
static edb_status batch_load_host(edb_batch *b, const double *F0_real, bool sync) {
  if (!b || !F0_real) return fail(EDB_EINVAL, "null argument");
  double *stage = batch_staging(b);
  const long long NQ = b->NQ;
  // the staging buffer is free once the previous work on st is done
  EDB_CUDA(cudaEventRecord(b->xev[0], b->st));
  EDB_CUDA(cudaStreamWaitEvent(b->cst, b->xev[0], 0));
  for (int i = 0; i < BATCH_XFER_CHUNKS; ++i) {  // copy chunk i while chunk i-1 transforms
    int c0, c1;
    batch_chunk(b, i, &c0, &c1);
    if (c1 <= c0) break;
    EDB_CUDA(cudaMemcpyAsync(stage + c0 * NQ, F0_real + c0 * NQ, sizeof(double) * (c1 - c0) * NQ,
                             cudaMemcpyHostToDevice, b->cst));
    EDB_CUDA(cudaEventRecord(b->xev[i], b->cst));
    EDB_CUDA(cudaStreamWaitEvent(b->st, b->xev[i], 0));
    EDB_TRY(launch_real_to_complex((c1 - c0) * NQ, stage + c0 * NQ, b->F + c0 * NQ, b->st));
    EDB_TRY(launch_dft3d(b->d.N, c1 - c0, b->F + c0 * NQ, b->Fhat + c0 * NQ, nullptr, 0,
                         EDB_DFT_DOUBLE_FLOAT, b->st));
  }
  EDB_TRY(batch_init_state(b, b->st, true, sync));
  b->f_cur = true;  // F holds the loaded data
  return EDB_OK;
}

extern "C" edb_status edb_batch_load(edb_batch *b, const double *F0_real) {
  return batch_load_host(b, F0_real, true);
}

extern "C" edb_status edb_batch_load_async(edb_batch *b, const double *F0_real) {
  return batch_load_host(b, F0_real, false);
}

// With a NULL stream the device-pointer calls run on the batch's own stream,
// which does not order against the default stream by itself: it first waits
// for what the caller queued there (e.g. the kernel that wrote the input).
static edb_status batch_join_default(edb_batch *b) {
  EDB_CUDA(cudaEventRecord(b->join_ev, cudaStreamLegacy));
  EDB_CUDA(cudaStreamWaitEvent(b->st, b->join_ev, 0));
  return EDB_OK;
}

extern "C" edb_status edb_batch_load_device(edb_batch *b, const double *d_F0_real, void *stream) {
  if (!b || !d_F0_real) return fail(EDB_EINVAL, "null argument");
  if (!stream) EDB_TRY(batch_join_default(b));
  cudaStream_t st = stream ? (cudaStream_t)stream : b->st;
  EDB_TRY(launch_real_to_complex(b->n, d_F0_real, b->F, st));
  EDB_TRY(batch_init_state(b, st));
  b->f_cur = true;
  return EDB_OK;
}

// One step for every solve: Q-hat stages on the FP32 copy of each stage
// input, stage updates in FP64 (each also refreshing the FP32 copy), then the
// FP64 ifft + entropy + fix rule when enabled.
static edb_status batch_step_record(edb_batch *b, cudaStream_t st) {
  const long long n = b->n;
  const int S = b->d.S, N = b->d.N;
  const double dt = b->d.dt;
  const float *B32 = b->q->B32;
  double2 *Fh = b->Fhat, **F = b->Fs;
  float2 **Q = b->Qs, *in = b->in32;
  const int variant = c32_variant_for(b->q, S);
  auto calq = [&](float2 *out) {
    return launch_calq32_batch(N, S, B32, in, out, st, variant, 1, nullptr, b->pairs);
  };
  switch (b->d.scheme) {
    case EDB_SCHEME_FE:
      EDB_TRY(calq(Q[0]));
      EDB_TRY(launch_stage_f32q(n, STAGE_AXPY, 0, dt, 0, Fh, Fh, 0, 0, Q[0], 0, 0, 0, in, st));
      break;
    case EDB_SCHEME_SSP3:
      EDB_TRY(calq(Q[0]));
      EDB_TRY(launch_stage_f32q(n, STAGE_AXPY, 0, dt, 0, F[0], Fh, 0, 0, Q[0], 0, 0, 0, in, st));
      EDB_TRY(calq(Q[0]));
      EDB_TRY(launch_stage_f32q(n, STAGE_SSP3_2, 0, 0.25 * dt, 0, F[1], Fh, F[0], 0, Q[0], 0, 0, 0,
                                in, st));
      EDB_TRY(calq(Q[0]));
      EDB_TRY(launch_stage_f32q(n, STAGE_SSP3_3, 0, 2. / 3. * dt, 0, Fh, Fh, F[1], 0, Q[0], 0, 0,
                                0, in, st));
      break;
    case EDB_SCHEME_RK4:
      EDB_TRY(calq(Q[0]));
      EDB_TRY(
          launch_stage_f32q(n, STAGE_AXPY, 0, 0.5 * dt, 0, F[0], Fh, 0, 0, Q[0], 0, 0, 0, in, st));
      EDB_TRY(calq(Q[1]));
      EDB_TRY(
          launch_stage_f32q(n, STAGE_AXPY, 0, 0.5 * dt, 0, F[1], Fh, 0, 0, Q[1], 0, 0, 0, in, st));
      EDB_TRY(calq(Q[2]));
      EDB_TRY(launch_stage_f32q(n, STAGE_AXPY, 0, dt, 0, F[2], Fh, 0, 0, Q[2], 0, 0, 0, in, st));
      EDB_TRY(calq(Q[3]));
      EDB_TRY(launch_stage_f32q(n, STAGE_RK4, 0, dt / 6., 0, Fh, Fh, 0, 0, Q[0], Q[1], Q[2], Q[3],
                                in, st));
      break;
  }
  if (b->d.conserve) {
    // back onto the initial moments; the fix (moment-preserving) feeds the
    // fixed F back into Fhat; the FP32 copy follows the final Fhat
    EDB_TRY(launch_project_moments(N, S, b->ctab, Fh, b->m0, st));
    if (b->d.fix_entropy) {
      EDB_TRY(launch_dft3d(N, S, Fh, b->F, nullptr, 1, EDB_DFT_DOUBLE_FLOAT, st));
      EDB_TRY(launch_step_entropy_conserve(N, S, b->d.R, b->F, b->state, 1.0e-10, 2, b->tr_raw,
                                           b->tr_fixed, 1, st, true));
      EDB_TRY(launch_dft3d(N, S, b->F, F[0], nullptr, 0, EDB_DFT_DOUBLE_FLOAT, st));
      EDB_TRY(launch_masked_copy(b->NQ, S, b->state, F[0], Fh, st));
    }
    EDB_TRY(launch_d2f(n, Fh, in, st));
  } else if (b->d.fix_entropy) {
    EDB_TRY(launch_dft3d(N, S, Fh, b->F, nullptr, 1, EDB_DFT_DOUBLE_FLOAT, st));
    EDB_TRY(launch_step_entropy(N, S, b->d.R, b->F, b->state, 1.0e-10, 2, b->tr_raw, b->tr_fixed,
                                1, st, true));
  }
  return EDB_OK;
}

extern "C" edb_status edb_batch_step(edb_batch *b, int nsteps, void *stream) {
  if (!b) return fail(EDB_EINVAL, "null handle");
  if (nsteps < 0) return fail(EDB_EINVAL, "nsteps must be >= 0");
  cudaStream_t st = stream ? (cudaStream_t)stream : b->st;
  if (!b->exec) {
    long long before = g_launches.load();
    cudaGraph_t graph = nullptr;
    EDB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    edb_status rc = batch_step_record(b, st);
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (rc != EDB_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    b->launches_per_step = (int)(g_launches.load() - before);
    g_launches -= b->launches_per_step;  // captured, not executed
  }
  for (int i = 0; i < nsteps; ++i) {
    EDB_CUDA(cudaGraphLaunch(b->exec, st));
    count_launch(b->launches_per_step);
  }
  if (nsteps > 0) b->f_cur = b->d.fix_entropy != 0;
  if (!stream) {
    EDB_CUDA(cudaStreamSynchronize(st));
    return check_device_waits("batch step");
  }
  return EDB_OK;
}

// Host read; sync = false returns with the copies queued: work queued later
// on st waits for them (they read the staging buffer the step writes).
static edb_status batch_read_host(edb_batch *b, double *F_real, double *Fhat, bool sync) {
  if (!b) return fail(EDB_EINVAL, "null handle");
  cudaStream_t st = b->st;
  if (sync) EDB_CUDA(cudaStreamSynchronize(st));
  if (Fhat)
    EDB_CUDA(cudaMemcpyAsync(Fhat, b->Fhat, sizeof(double2) * b->n, cudaMemcpyDeviceToHost, st));
  if (F_real) {  // inverse transform (unless F is current), real parts packed
                 // on the device, per chunk: chunk i copies out while chunk i+1
                 // transforms
    double *stage = batch_staging(b);
    const long long NQ = b->NQ;
    for (int i = 0; i < BATCH_XFER_CHUNKS; ++i) {
      int c0, c1;
      batch_chunk(b, i, &c0, &c1);
      if (c1 <= c0) break;
      if (!b->f_cur)
        EDB_TRY(launch_dft3d(b->d.N, c1 - c0, b->Fhat + c0 * NQ, b->F + c0 * NQ, nullptr, 1,
                             EDB_DFT_DOUBLE_FLOAT, st));
      EDB_TRY(launch_complex_to_real((c1 - c0) * NQ, b->F + c0 * NQ, stage + c0 * NQ, st));
      EDB_CUDA(cudaEventRecord(b->xev[i], st));
      EDB_CUDA(cudaStreamWaitEvent(b->cst, b->xev[i], 0));
      EDB_CUDA(cudaMemcpyAsync(F_real + c0 * NQ, stage + c0 * NQ, sizeof(double) * (c1 - c0) * NQ,
                               cudaMemcpyDeviceToHost, b->cst));
    }
    EDB_CUDA(cudaEventRecord(b->xdone, b->cst));
    EDB_CUDA(cudaStreamWaitEvent(st, b->xdone, 0));
    if (sync) EDB_CUDA(cudaStreamSynchronize(b->cst));
    b->f_cur = true;
  }
  if (sync) EDB_CUDA(cudaStreamSynchronize(st));
  return EDB_OK;
}

extern "C" edb_status edb_batch_read(edb_batch *b, double *F_real, double *Fhat) {
  return batch_read_host(b, F_real, Fhat, true);
}

extern "C" edb_status edb_batch_read_async(edb_batch *b, double *F_real) {
  if (!F_real) return fail(EDB_EINVAL, "null argument");
  return batch_read_host(b, F_real, nullptr, false);
}

extern "C" edb_status edb_batch_step_async(edb_batch *b, int nsteps) {
  if (!b) return fail(EDB_EINVAL, "null handle");
  return edb_batch_step(b, nsteps, (void *)b->st);
}

extern "C" edb_status edb_batch_sync(edb_batch *b) {
  if (!b) return fail(EDB_EINVAL, "null handle");
  EDB_CUDA(cudaStreamSynchronize(b->cst));
  EDB_CUDA(cudaStreamSynchronize(b->st));
  return check_device_waits("batch");
}

extern "C" edb_status edb_batch_read_device(edb_batch *b, double *d_F_real, void *stream) {
  if (!b || !d_F_real) return fail(EDB_EINVAL, "null argument");
  if (!stream) EDB_TRY(batch_join_default(b));
  cudaStream_t st = stream ? (cudaStream_t)stream : b->st;
  if (!b->f_cur)
    EDB_TRY(launch_dft3d(b->d.N, b->d.S, b->Fhat, b->F, nullptr, 1, EDB_DFT_DOUBLE_FLOAT, st));
  b->f_cur = true;
  EDB_TRY(launch_complex_to_real(b->n, b->F, d_F_real, st));
  if (!stream) EDB_CUDA(cudaStreamSynchronize(st));
  return EDB_OK;
}

extern "C" edb_status edb_batch_moments(edb_batch *b, double *moments, double *entropy) {
  if (!b) return fail(EDB_EINVAL, "null handle");
  cudaStream_t st = b->st;
  if (!b->f_cur)
    EDB_TRY(launch_dft3d(b->d.N, b->d.S, b->Fhat, b->F, nullptr, 1, EDB_DFT_DOUBLE_FLOAT, st));
  b->f_cur = true;
  EDB_TRY(launch_moments(b->d.N, b->d.S, b->d.R, b->F, b->mom, st));
  EDB_TRY(launch_calentropy(b->d.N, b->d.S, b->d.R, b->F, b->H, st));
  if (moments)
    EDB_CUDA(cudaMemcpyAsync(moments, b->mom, sizeof(double) * 5 * b->d.S, cudaMemcpyDeviceToHost,
                             st));
  if (entropy)
    EDB_CUDA(cudaMemcpyAsync(entropy, b->H, sizeof(double) * b->d.S, cudaMemcpyDeviceToHost, st));
  EDB_CUDA(cudaStreamSynchronize(st));
  return EDB_OK;
}

extern "C" edb_status edb_batch_entropy(edb_batch *b, double *raw, double *fixed) {
  if (!b || (!raw && !fixed)) return fail(EDB_EINVAL, "null argument");
  cudaStream_t st = b->st;
  if (raw)
    EDB_CUDA(cudaMemcpyAsync(raw, b->tr_raw, sizeof(double) * b->d.S, cudaMemcpyDeviceToHost, st));
  if (fixed)
    EDB_CUDA(
        cudaMemcpyAsync(fixed, b->tr_fixed, sizeof(double) * b->d.S, cudaMemcpyDeviceToHost, st));
  EDB_CUDA(cudaStreamSynchronize(st));
  return EDB_OK;
}

extern "C" edb_status edb_batch_launches_per_step(edb_batch *b, int *n) {
  if (!b || !n) return fail(EDB_EINVAL, "null argument");
  *n = b->launches_per_step;
  return EDB_OK;
}

// ============================================================ conservation

extern "C" edb_status edb_moments_hat_device(int N, int S, double R, const double *d_Fhat,
                                             double *d_m, void *stream) {
  if (N < 3 || N > 64 || S < 1 || !(R > 0) || !d_Fhat || !d_m)
    return fail(EDB_EINVAL, "bad argument");
  EDB_TRY(ensure_device());
  double *tab = nullptr;
  EDB_TRY(upload_conserve_table(N, R, &tab));
  cudaStream_t st = (cudaStream_t)stream;
  edb_status rc = launch_hat_moments(N, S, tab, (const double2 *)d_Fhat, d_m, st);
  cudaError_t e = cudaStreamSynchronize(st);
  dfree(tab);
  if (rc != EDB_OK) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "moments");
  return EDB_OK;
}

extern "C" edb_status edb_moments_project_device(int N, int S, double R, double *d_Fhat,
                                                 const double *d_m0, void *stream) {
  if (N < 3 || N > 64 || S < 1 || !(R > 0) || !d_Fhat || !d_m0)
    return fail(EDB_EINVAL, "bad argument");
  EDB_TRY(ensure_device());
  double *tab = nullptr;
  EDB_TRY(upload_conserve_table(N, R, &tab));
  cudaStream_t st = (cudaStream_t)stream;
  edb_status rc = launch_project_moments(N, S, tab, (double2 *)d_Fhat, d_m0, st);
  cudaError_t e = cudaStreamSynchronize(st);
  dfree(tab);
  if (rc != EDB_OK) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "moment projection");
  return EDB_OK;
}

extern "C" edb_status edb_maxwellian_fit_device(int N, int S, double R, double *d_F,
                                                double *d_theta, int *d_status, void *stream) {
  if (N < 3 || N > 64 || S < 1 || !(R > 0) || !d_F || !d_theta || !d_status)
    return fail(EDB_EINVAL, "bad argument");
  EDB_TRY(ensure_device());
  cudaStream_t st = (cudaStream_t)stream;
  EDB_TRY(launch_maxwellian_fit(N, S, R, (double2 *)d_F, d_theta, d_status, st));
  EDB_CUDA(cudaStreamSynchronize(st));
  return EDB_OK;
}

// ============================================================ measurement aid
// FP32 FMA issue-rate probe: every thread runs 8 independent FFMA chains.
// Used as the measured denominator of the FP32 roofline fraction.
__global__ void ffma_peak_kernel(int iters, float seed, float *out) {
  float a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = seed + threadIdx.x * 1e-7f + j;
  const float m = 0.999999f, c = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = fmaf(a[j], m, c);
  }
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += a[j];
  if (s == 12345.678f) out[blockIdx.x] = s;  // keeps the chains alive
}

extern "C" edb_status edb_measure_fp32_peak(double *tflops) {
  if (!tflops) return fail(EDB_EINVAL, "null output");
  EDB_TRY(ensure_device());
  int dev = 0, sms = 0;
  EDB_CUDA(cudaGetDevice(&dev));
  EDB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  float *out = nullptr;
  EDB_TRY(dalloc(&out, (size_t)sms * 8));
  const int iters = 20000, threads = 512, blocks = sms * 4;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  ffma_peak_kernel<<<blocks, threads>>>(iters / 10, 1.0f, out);  // warm-up
  cudaEventRecord(e0);
  ffma_peak_kernel<<<blocks, threads>>>(iters, 1.0f, out);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  dfree(out);
  if (e != cudaSuccess) return cuda_fail(e, "ffma probe");
  double flops = 2.0 * 8.0 * iters * (double)threads * blocks;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return EDB_OK;
}

// Packed FP32 (fma.rn.f32x2) issue-rate probe: 8 independent packed chains per
// thread, 2 FP32 FMAs per instruction.  Compared with edb_measure_fp32_peak it
// shows whether packed issue raises the FP32 datapath ceiling or only frees
// issue slots.
__global__ void ffma2_peak_kernel(int iters, float seed, float *out) {
  unsigned long long a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float x = seed + threadIdx.x * 1e-7f + j;
    asm("mov.b64 %0, {%1, %1};" : "=l"(a[j]) : "f"(x));
  }
  unsigned long long m, c;
  asm("mov.b64 %0, {%1, %1};" : "=l"(m) : "f"(0.999999f));
  asm("mov.b64 %0, {%1, %1};" : "=l"(c) : "f"(1e-7f));
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) asm("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(a[j]) : "l"(m), "l"(c));
  }
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a[j]));
    s += lo + hi;
  }
  if (s == 12345.678f) out[blockIdx.x] = s;
}

extern "C" edb_status edb_measure_fp32x2_peak(double *tflops) {
  if (!tflops) return fail(EDB_EINVAL, "null output");
  EDB_TRY(ensure_device());
  int dev = 0, sms = 0;
  EDB_CUDA(cudaGetDevice(&dev));
  EDB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  float *out = nullptr;
  EDB_TRY(dalloc(&out, (size_t)sms * 8));
  const int iters = 20000, threads = 512, blocks = sms * 4;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  ffma2_peak_kernel<<<blocks, threads>>>(iters / 10, 1.0f, out);
  cudaEventRecord(e0);
  ffma2_peak_kernel<<<blocks, threads>>>(iters, 1.0f, out);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  dfree(out);
  if (e != cudaSuccess) return cuda_fail(e, "ffma2 probe");
  double flops = 2.0 * 2.0 * 8.0 * iters * (double)threads * blocks;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return EDB_OK;
}
