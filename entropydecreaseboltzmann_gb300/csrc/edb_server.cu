// Serving engine: a device-resident request loop with continuous batching of
// independent solves (declared in include/edb.h, "serving engine").
//
// Layout.  Requests are grouped by kernel table (N, gamma, R).  A group owns
// its FP32 table and an arena of `cap` solve slots in HBM: FP64 f-hat, the
// stage arrays, the FP32 stage-input copy, the entropy state and (conservative
// mode) the target moments.  Live solves occupy slots [0, live).
//
// Loop (host thread, one CUDA stream per group):
//   arrivals      requests whose arrival time has passed join their group's
//                 FIFO queue;
//   completion    when a group's step event has fired, every live solve has
//                 advanced one step; finished solves are inverse-transformed,
//                 copied out, and the arena is compacted (the last live slots
//                 move into the holes) so live solves stay a prefix;
//   admission     queued requests take slots while the group's live cap and
//                 the HBM budget allow (arenas grow by doubling, shrink when
//                 mostly empty); their initial data is uploaded and
//                 transformed in chunks;
//   step          one replay of the group's captured CUDA graph for the
//                 bucket S = live rounded up to 4 (the batched kernel's
//                 smallest solve group) advances every live solve by one
//                 step; padding slots hold zero solves.  Q-hat runs chunked
//                 over the l1 planes (4 chunks, fixed per group), so a few
//                 live solves still fill the GPU and a result does not depend
//                 on the bucket it ran in.
// Groups run concurrently on their own streams.  Each solve's arithmetic
// depends only on its own slot, so a result is the same alone and in a mix.
#include <math.h>

#include <cmath>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <thread>
#include <tuple>
#include <vector>

#include "edb_internal.cuh"

namespace edb {
namespace {

constexpr int BUCKET = 4;   // graph bucket granularity (solves)
constexpr int XFER = 64;    // solves per admission / retirement transfer chunk

using Clock = std::chrono::steady_clock;

struct Req {
  edb_request r;
  std::vector<double> F0;
  double t_arrival = -1, t_admit = -1, t_done = -1;
  // 0 queued / not arrived, 1 running, 2 done, 3 refused (cannot fit),
  // 4 cancelled, 5 failed (its state became non-finite)
  int state = 0;
  bool cancel = false;  // running: retire at the next step boundary without a result
  int group = -1;
  int remaining = 0;
  std::vector<double> F, Fhat;  // results (want_result)
};

struct Group {
  int N = 0;
  double gamma = 0, R = 0;
  long long NQ = 0;
  edb_qcalc *q = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  int cap = 0, live = 0;
  // arena (cap slots)
  double2 *Fhat = nullptr, *F = nullptr, *Fs[3] = {nullptr, nullptr, nullptr};
  float2 *Qs[4] = {nullptr, nullptr, nullptr, nullptr}, *in32 = nullptr;
  EfixState *state = nullptr;
  double *m0 = nullptr, *H = nullptr;
  float4 *part = nullptr;  // chunk partial sums of one Q-hat stage
  int C = 1;               // l1-plane chunks of the batched kernel
  // fixed per group
  double *ctab = nullptr, *trd = nullptr, *xin = nullptr;
  double2 *xo = nullptr, *xF = nullptr;
  double *h_in = nullptr;
  double2 *h_F = nullptr, *h_Fhat = nullptr;
  std::vector<long long> slot_req;
  std::map<int, std::pair<cudaGraphExec_t, int>> graphs;  // bucket -> (exec, launches)
  std::deque<long long> queue;
  bool inflight = false;
  int inflight_live = 0;
  long long table_bytes = 0, fixed_bytes = 0, arena_bytes = 0;
};

double pct(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double x = p * (double)(v.size() - 1);
  const size_t i = (size_t)x;
  const double f = x - (double)i;
  return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

}  // namespace
}  // namespace edb

using namespace edb;

struct edb_server {
  edb_server_desc d;
  int nstage = 0, nq = 0, stages = 0;
  std::vector<std::unique_ptr<Group>> groups;
  std::map<std::tuple<int, double, double>, int> gidx;
  std::vector<Req> reqs;            // index = id
  std::vector<long long> pending;   // submitted, not yet arrived (sorted by arrival)
  size_t pending_head = 0;
  bool pending_sorted = true;
  bool clock_started = false;
  Clock::time_point t0;
  long long bytes_used = 0;
  double bytes_peak = 0;
  long long steps_launched = 0, launches = 0, completed = 0, refused = 0;
  long long cancelled = 0, failed = 0;
  double evals = 0, evals_padded = 0;
  // every field above is guarded by mu once the background loop runs
  std::mutex mu;
  std::condition_variable cv_work;  // submissions and stop wake the loop
  std::condition_variable cv_done;  // completions wake waiters
  std::thread th;
  bool started = false, stop_req = false;
  edb_status loop_status = EDB_OK;
  std::string loop_msg;
  int device = 0;
};

namespace {

double now_s(const edb_server *s) {
  if (!s->clock_started) return 0.0;
  return std::chrono::duration<double>(Clock::now() - s->t0).count();
}

// Requests that need no more work (done, refused, cancelled or failed).
long long settled(const edb_server *s) {
  return s->completed + s->refused + s->cancelled + s->failed;
}

// Chunk count of the batched kernel for a table of N (fixed per N).
// l1-plane chunks of a group's batched launches, fixed per group so a result
// does not depend on its bucket.  Measured on the serving mix (persistent
// launches): 4 chunks 36.1-36.2 requests/s, p50 1.33 s, uneven batch 28.7 s;
// 8 chunks 35.5-36.2, p50 1.41-1.46 s, 29.3-29.7 s; 16 chunks 33.1, 1.61 s, 30.8 s.
int chunks_of(int N) { return N < 4 ? N : 4; }

long long slot_bytes(const edb_server *s, int N) {
  // Fhat, F (complex FP64), stage arrays, FP32 Q-hat stages, FP32 input copy,
  // chunk partial sums
  const long long NQ = (long long)N * N * N;
  const int nst = s->nstage > 0 ? s->nstage : ((s->d.conserve && s->d.fix_entropy) ? 1 : 0);
  return NQ * (16 + 16 + 16LL * nst + 8LL * s->nq + 8 + 16LL * chunks_of(N)) +
         (long long)sizeof(EfixState) + 48;
}

// The FP32 pair table of edb_qcalc_genB_f32 (visited planes only).
long long table_bytes_of(int N) { return c32_table_floats(N) * 4 + 256; }

long long fixed_bytes_of(int N) {
  const long long NQ = (long long)N * N * N;
  return (long long)XFER * NQ * (8 + 16 + 16) + 4096;
}

void account(edb_server *s, long long delta) {
  s->bytes_used += delta;
  if ((double)s->bytes_used > s->bytes_peak) s->bytes_peak = (double)s->bytes_used;
}

void free_arena(Group &g) {
  dfree(g.Fhat);
  dfree(g.F);
  for (auto &p : g.Fs) dfree(p);
  for (auto &p : g.Qs) dfree(p);
  dfree(g.in32);
  dfree(g.state);
  dfree(g.m0);
  dfree(g.H);
  dfree(g.part);
}

void drop_graphs(Group &g) {
  for (auto &kv : g.graphs) cudaGraphExecDestroy(kv.second.first);
  g.graphs.clear();
}

void destroy_group(Group &g) {
  if (g.st) cudaStreamSynchronize(g.st);
  drop_graphs(g);
  free_arena(g);
  dfree(g.ctab);
  dfree(g.trd);
  dfree(g.xin);
  dfree(g.xo);
  dfree(g.xF);
  if (g.h_in) cudaFreeHost(g.h_in);
  if (g.h_F) cudaFreeHost(g.h_F);
  if (g.h_Fhat) cudaFreeHost(g.h_Fhat);
  if (g.ev) cudaEventDestroy(g.ev);
  if (g.st) cudaStreamDestroy(g.st);
  if (g.q) edb_qcalc_destroy(g.q);
}

edb_status get_group(edb_server *s, int N, double gamma, double R, int *out) {
  const auto key = std::make_tuple(N, gamma, R);
  auto it = s->gidx.find(key);
  if (it != s->gidx.end()) {
    *out = it->second;
    return EDB_OK;
  }
  const long long need = table_bytes_of(N) + fixed_bytes_of(N);
  if (s->bytes_used + need > (long long)s->d.hbm_budget_bytes)
    return fail(EDB_ENOMEM, "HBM budget exhausted by other groups' tables");
  auto g = std::make_unique<Group>();
  g->N = N;
  g->gamma = gamma;
  g->R = R;
  g->NQ = (long long)N * N * N;
  g->C = chunks_of(N);
  const size_t NQ = (size_t)g->NQ;
  edb_qcalc_desc qd;
  qd.N = N;
  qd.gamma = gamma;
  qd.L = R;
  qd.filter = s->d.filter;
  qd.index_mode = EDB_INDEX_ALIASED;
  edb_status rc = edb_qcalc_create(&qd, &g->q);
  if (rc == EDB_OK) rc = edb_qcalc_genB_f32(g->q);
  if (rc == EDB_OK) {
    cudaError_t e = cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&g->h_in, sizeof(double) * XFER * NQ);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&g->h_F, sizeof(double2) * XFER * NQ);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&g->h_Fhat, sizeof(double2) * XFER * NQ);
    if (e != cudaSuccess) rc = cuda_fail(e, "server group setup");
  }
  if (rc == EDB_OK) rc = dalloc(&g->xin, XFER * NQ);
  if (rc == EDB_OK) rc = dalloc(&g->xo, XFER * NQ);
  if (rc == EDB_OK) rc = dalloc(&g->xF, XFER * NQ);
  if (rc == EDB_OK) rc = dalloc(&g->trd, 1);
  if (rc == EDB_OK && s->d.conserve) {
    std::vector<double> tab;
    build_conserve_table(N, R, tab);
    rc = dalloc(&g->ctab, tab.size());
    if (rc == EDB_OK) {
      cudaError_t e = cudaMemcpy(g->ctab, tab.data(), sizeof(double) * tab.size(),
                                 cudaMemcpyHostToDevice);
      if (e != cudaSuccess) rc = cuda_fail(e, "conservation table");
    }
  }
  if (rc != EDB_OK) {
    destroy_group(*g);
    return rc;
  }
  g->table_bytes = qcalc_table_bytes(g->q);
  g->fixed_bytes = fixed_bytes_of(N);
  account(s, g->table_bytes + g->fixed_bytes);
  s->groups.push_back(std::move(g));
  *out = (int)s->groups.size() - 1;
  s->gidx[key] = *out;
  return EDB_OK;
}

// Resizes the arena to newcap slots, keeping the live prefix.
edb_status resize_arena(edb_server *s, Group &g, int newcap) {
  if (g.st) EDB_CUDA(cudaStreamSynchronize(g.st));
  const long long nb = (long long)newcap * slot_bytes(s, g.N);
  if (s->bytes_used - g.arena_bytes + nb > (long long)s->d.hbm_budget_bytes)
    return fail(EDB_ENOMEM, "HBM budget");
  Group ng;  // new arrays only
  const size_t n = (size_t)newcap * (size_t)g.NQ;
  const int nst = s->nstage > 0 ? s->nstage : ((s->d.conserve && s->d.fix_entropy) ? 1 : 0);
  edb_status rc = dalloc(&ng.Fhat, n);
  if (rc == EDB_OK) rc = dalloc(&ng.F, n);
  for (int i = 0; i < nst && rc == EDB_OK; ++i) rc = dalloc(&ng.Fs[i], n);
  for (int i = 0; i < s->nq && rc == EDB_OK; ++i) rc = dalloc(&ng.Qs[i], n);
  if (rc == EDB_OK) rc = dalloc(&ng.in32, n);
  if (rc == EDB_OK) rc = dalloc(&ng.state, (size_t)newcap);
  if (rc == EDB_OK) rc = dalloc(&ng.m0, (size_t)newcap * 5);
  if (rc == EDB_OK) rc = dalloc(&ng.H, (size_t)newcap);
  if (rc == EDB_OK && g.C > 1) rc = dalloc(&ng.part, n * (size_t)g.C);
  if (rc != EDB_OK) {
    free_arena(ng);
    return rc;
  }
  cudaError_t e = cudaSuccess;
  // zeroed slots are valid (zero) solves: padding never produces NaN
  e = cudaMemsetAsync(ng.Fhat, 0, sizeof(double2) * n, g.st);
  if (e == cudaSuccess) e = cudaMemsetAsync(ng.in32, 0, sizeof(float2) * n, g.st);
  if (e == cudaSuccess) e = cudaMemsetAsync(ng.state, 0, sizeof(EfixState) * newcap, g.st);
  if (e == cudaSuccess) e = cudaMemsetAsync(ng.m0, 0, sizeof(double) * 5 * newcap, g.st);
  const size_t keep = (size_t)g.live * (size_t)g.NQ;
  if (g.live > 0) {
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(ng.Fhat, g.Fhat, sizeof(double2) * keep, cudaMemcpyDeviceToDevice, g.st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(ng.in32, g.in32, sizeof(float2) * keep, cudaMemcpyDeviceToDevice, g.st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(ng.state, g.state, sizeof(EfixState) * g.live, cudaMemcpyDeviceToDevice,
                          g.st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(ng.m0, g.m0, sizeof(double) * 5 * g.live, cudaMemcpyDeviceToDevice,
                          g.st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(g.st);
  if (e != cudaSuccess) {
    free_arena(ng);
    return cuda_fail(e, "arena resize");
  }
  drop_graphs(g);
  free_arena(g);
  g.Fhat = ng.Fhat;
  g.F = ng.F;
  for (int i = 0; i < 3; ++i) g.Fs[i] = ng.Fs[i];
  for (int i = 0; i < 4; ++i) g.Qs[i] = ng.Qs[i];
  g.in32 = ng.in32;
  g.state = ng.state;
  g.m0 = ng.m0;
  g.H = ng.H;
  g.part = ng.part;
  ng = Group();
  account(s, nb - g.arena_bytes);
  g.arena_bytes = nb;
  g.cap = newcap;
  g.slot_req.resize((size_t)newcap, -1);
  return EDB_OK;
}

// One step of every solve in slots [0, S) (the batched solver's step).
edb_status record_step(edb_server *s, Group &g, int S, cudaStream_t st) {
  const long long n = (long long)S * g.NQ;
  const int N = g.N;
  const double dt = s->d.dt;
  const float *B32 = qcalc_B32(g.q);
  double2 *Fh = g.Fhat, **F = g.Fs;
  float2 **Q = g.Qs, *in = g.in32;
  const int variant = qcalc_c32_variant(g.q, S, nullptr, g.C > 1);
  auto calq = [&](float2 *out) {
    // persistent grids, chunked too: they overlap better with the other groups'
    // launches on their streams (the serving mix: 32 -> 36 requests/s)
    return launch_calq32_batch(N, S, B32, in, out, st, variant, g.C, g.part, nullptr, 1);
  };
  switch (s->d.scheme) {
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
    default:  // RK4
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
  if (s->d.conserve) {
    EDB_TRY(launch_project_moments(N, S, g.ctab, Fh, g.m0, st));
    if (s->d.fix_entropy) {
      EDB_TRY(launch_dft3d(N, S, Fh, g.F, nullptr, 1, EDB_DFT_DOUBLE_FLOAT, st));
      EDB_TRY(launch_step_entropy_conserve(N, S, g.R, g.F, g.state, 1.0e-10, 2, g.trd, g.trd, 0,
                                           st));
      EDB_TRY(launch_dft3d(N, S, g.F, F[0], nullptr, 0, EDB_DFT_DOUBLE_FLOAT, st));
      EDB_TRY(launch_masked_copy(g.NQ, S, g.state, F[0], Fh, st));
    }
    EDB_TRY(launch_d2f(n, Fh, in, st));
  } else if (s->d.fix_entropy) {
    EDB_TRY(launch_dft3d(N, S, Fh, g.F, nullptr, 1, EDB_DFT_DOUBLE_FLOAT, st));
    EDB_TRY(launch_step_entropy(N, S, g.R, g.F, g.state, 1.0e-10, 2, g.trd, g.trd, 0, st));
  }
  return EDB_OK;
}

edb_status step_graph(edb_server *s, Group &g, int S, cudaGraphExec_t *exec, int *nl) {
  auto it = g.graphs.find(S);
  if (it != g.graphs.end()) {
    *exec = it->second.first;
    *nl = it->second.second;
    return EDB_OK;
  }
  bool tuned = false;
  qcalc_c32_variant(g.q, S, &tuned, g.C > 1);
  if (!tuned)  // before capture: the graph bakes the variant in
    EDB_TRY(qcalc_autotune_split(g.q, S, g.in32, g.Qs[0], g.st, g.C, g.part));
  const long long before = edb_kernel_launch_count();
  cudaGraph_t graph = nullptr;
  EDB_CUDA(cudaStreamBeginCapture(g.st, cudaStreamCaptureModeThreadLocal));
  edb_status rc = record_step(s, g, S, g.st);
  cudaError_t e = cudaStreamEndCapture(g.st, &graph);
  const int n = (int)(edb_kernel_launch_count() - before);
  count_launch(-n);  // captured, not executed
  if (rc != EDB_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  cudaGraphExec_t ex = nullptr;
  e = cudaGraphInstantiate(&ex, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  g.graphs[S] = std::make_pair(ex, n);
  *exec = ex;
  *nl = n;
  return EDB_OK;
}

int bucket_of(int live, int cap) {
  const int b = ((live + BUCKET - 1) / BUCKET) * BUCKET;
  return b < cap ? b : cap;
}

// Frees the arenas of idle groups (no live, queued or running solves) other
// than `keep`, returning their budget.
edb_status reclaim_idle(edb_server *s, Group &keep) {
  for (auto &gp : s->groups) {
    Group &o = *gp;
    if (&o == &keep || o.cap == 0 || o.live > 0 || o.inflight || !o.queue.empty()) continue;
    EDB_TRY(resize_arena(s, o, 0));
  }
  return EDB_OK;
}

edb_status admit(edb_server *s, Group &g, int gi) {
  const int limit = s->d.max_live_per_group > 0 ? s->d.max_live_per_group : (1 << 30);
  while (!g.queue.empty() && g.live < limit) {
    int k = (int)std::min<size_t>(g.queue.size(), (size_t)XFER);
    k = std::min(k, limit - g.live);
    if (g.live + k > g.cap) {
      int want = std::max(g.cap * 2, ((g.live + k + BUCKET - 1) / BUCKET) * BUCKET);
      if (s->d.max_live_per_group > 0)
        want = std::min(want, ((limit + BUCKET - 1) / BUCKET) * BUCKET);
      const long long sb = slot_bytes(s, g.N);
      auto fit = [&]() {  // largest capacity (whole buckets) the budget allows
        const long long avail = (long long)s->d.hbm_budget_bytes - (s->bytes_used - g.arena_bytes);
        return (int)(avail / sb) / BUCKET * BUCKET;
      };
      if (fit() < want) {
        EDB_TRY(reclaim_idle(s, g));
        want = std::min(want, fit());
      }
      if (want > g.cap) {
        edb_status rc = resize_arena(s, g, want);
        if (rc != EDB_OK && g.cap == 0) return rc;
      }
      k = std::min(k, g.cap - g.live);
      if (k <= 0) return EDB_OK;  // wait for slots to free up
    }
    const size_t NQ = (size_t)g.NQ;
    const double t = now_s(s);
    for (int j = 0; j < k; ++j) {
      Req &r = s->reqs[(size_t)g.queue[(size_t)j]];
      memcpy(g.h_in + (size_t)j * NQ, r.F0.data(), sizeof(double) * NQ);
    }
    const size_t base = (size_t)g.live * NQ;
    cudaStream_t st = g.st;
    EDB_CUDA(cudaMemcpyAsync(g.xin, g.h_in, sizeof(double) * k * NQ, cudaMemcpyHostToDevice, st));
    EDB_TRY(launch_real_to_complex((long long)k * g.NQ, g.xin, g.F + base, st));
    EDB_TRY(
        launch_dft3d(g.N, k, g.F + base, g.Fhat + base, nullptr, 0, EDB_DFT_DOUBLE_FLOAT, st));
    if (s->d.conserve)
      EDB_TRY(launch_hat_moments(g.N, k, g.ctab, g.Fhat + base, g.m0 + (size_t)g.live * 5, st));
    EDB_TRY(launch_d2f((long long)k * g.NQ, g.Fhat + base, g.in32 + base, st));
    std::vector<EfixState> init((size_t)k, EfixState{1.0, 0, 0, 1.0, 0, 0});
    EDB_CUDA(cudaMemcpyAsync(g.state + g.live, init.data(), sizeof(EfixState) * k,
                             cudaMemcpyHostToDevice, st));
    if (s->d.conserve) {
      EDB_TRY(launch_calentropy(g.N, k, g.R, g.F + base, g.H + g.live, st));
      EDB_TRY(launch_state_from_entropy(k, g.H + g.live, g.state + g.live, st));
    }
    EDB_CUDA(cudaStreamSynchronize(st));  // h_in and `init` are reused
    for (int j = 0; j < k; ++j) {
      const long long id = g.queue.front();
      g.queue.pop_front();
      Req &r = s->reqs[(size_t)id];
      r.state = 1;
      r.t_admit = t;
      r.group = gi;
      r.remaining = r.r.steps;
      std::vector<double>().swap(r.F0);
      g.slot_req[(size_t)(g.live + j)] = id;
    }
    g.live += k;
  }
  return EDB_OK;
}

// After a step: retire finished solves (results out, arena compacted).
edb_status complete(edb_server *s, Group &g) {
  std::vector<int> fin;
  for (int i = 0; i < g.inflight_live; ++i) {
    Req &r = s->reqs[(size_t)g.slot_req[(size_t)i]];
    if (--r.remaining <= 0 || r.cancel) fin.push_back(i);  // finished or cancelled
  }
  if (fin.empty()) return EDB_OK;
  const size_t NQ = (size_t)g.NQ;
  cudaStream_t st = g.st;
  for (size_t c0 = 0; c0 < fin.size(); c0 += XFER) {
    const int k = (int)std::min(fin.size() - c0, (size_t)XFER);
    bool want_hat = false;
    // the result is the last step's real-space output: with the fix rule on,
    // the step computed it (after the fix, which leaves F-hat alone, as the
    // reference's BKW3D does); otherwise it is the transform of F-hat
    const bool have_F = s->d.fix_entropy != 0;
    for (int j = 0; j < k; ++j) {
      const int slot = fin[c0 + (size_t)j];
      EDB_CUDA(cudaMemcpyAsync(g.xo + (size_t)j * NQ, g.Fhat + (size_t)slot * NQ,
                               sizeof(double2) * NQ, cudaMemcpyDeviceToDevice, st));
      if (have_F)
        EDB_CUDA(cudaMemcpyAsync(g.xF + (size_t)j * NQ, g.F + (size_t)slot * NQ,
                                 sizeof(double2) * NQ, cudaMemcpyDeviceToDevice, st));
      want_hat |= s->reqs[(size_t)g.slot_req[(size_t)slot]].r.want_result != 0;
    }
    if (!have_F) EDB_TRY(launch_dft3d(g.N, k, g.xo, g.xF, nullptr, 1, EDB_DFT_DOUBLE_FLOAT, st));
    EDB_CUDA(cudaMemcpyAsync(g.h_F, g.xF, sizeof(double2) * k * NQ, cudaMemcpyDeviceToHost, st));
    if (want_hat)
      EDB_CUDA(
          cudaMemcpyAsync(g.h_Fhat, g.xo, sizeof(double2) * k * NQ, cudaMemcpyDeviceToHost, st));
    EDB_CUDA(cudaStreamSynchronize(st));
    const double t = now_s(s);
    for (int j = 0; j < k; ++j) {
      Req &r = s->reqs[(size_t)g.slot_req[(size_t)fin[c0 + (size_t)j]]];
      r.t_done = t;
      if (r.cancel) {  // its slot is freed; no result
        r.state = 4;
        ++s->cancelled;
        continue;
      }
      // a solve whose state overflowed or became NaN is reported as failed
      bool finite = true;
      for (size_t i = 0; i < NQ && finite; ++i) finite = std::isfinite(g.h_F[(size_t)j * NQ + i].x);
      if (!finite) {
        r.state = 5;
        ++s->failed;
        continue;
      }
      if (r.r.want_result) {
        r.F.resize(NQ);
        for (size_t i = 0; i < NQ; ++i) r.F[i] = g.h_F[(size_t)j * NQ + i].x;
        r.Fhat.assign((const double *)(g.h_Fhat + (size_t)j * NQ),
                      (const double *)(g.h_Fhat + (size_t)(j + 1) * NQ));
      }
      r.state = 2;
      ++s->completed;
    }
    s->cv_done.notify_all();
  }
  // compaction: survivors past the new end move into the holes below it
  const int old_live = g.inflight_live;
  const int new_live = old_live - (int)fin.size();
  std::vector<char> is_fin((size_t)old_live, 0);
  for (int i : fin) is_fin[(size_t)i] = 1;
  std::vector<int> holes, movers;
  for (int i = 0; i < new_live; ++i)
    if (is_fin[(size_t)i]) holes.push_back(i);
  for (int i = new_live; i < old_live; ++i)
    if (!is_fin[(size_t)i]) movers.push_back(i);
  for (size_t j = 0; j < holes.size(); ++j) {
    const int dst = holes[j], src = movers[j];
    EDB_CUDA(cudaMemcpyAsync(g.Fhat + (size_t)dst * NQ, g.Fhat + (size_t)src * NQ,
                             sizeof(double2) * NQ, cudaMemcpyDeviceToDevice, st));
    EDB_CUDA(cudaMemcpyAsync(g.in32 + (size_t)dst * NQ, g.in32 + (size_t)src * NQ,
                             sizeof(float2) * NQ, cudaMemcpyDeviceToDevice, st));
    EDB_CUDA(cudaMemcpyAsync(g.state + dst, g.state + src, sizeof(EfixState),
                             cudaMemcpyDeviceToDevice, st));
    EDB_CUDA(cudaMemcpyAsync(g.m0 + (size_t)dst * 5, g.m0 + (size_t)src * 5, sizeof(double) * 5,
                             cudaMemcpyDeviceToDevice, st));
    g.slot_req[(size_t)dst] = g.slot_req[(size_t)src];
  }
  // the vacated tail becomes zero solves (bucket padding)
  const size_t nv = (size_t)(old_live - new_live);
  EDB_CUDA(cudaMemsetAsync(g.Fhat + (size_t)new_live * NQ, 0, sizeof(double2) * nv * NQ, st));
  EDB_CUDA(cudaMemsetAsync(g.in32 + (size_t)new_live * NQ, 0, sizeof(float2) * nv * NQ, st));
  EDB_CUDA(cudaMemsetAsync(g.state + new_live, 0, sizeof(EfixState) * nv, st));
  EDB_CUDA(cudaMemsetAsync(g.m0 + (size_t)new_live * 5, 0, sizeof(double) * 5 * nv, st));
  for (int i = new_live; i < old_live; ++i) g.slot_req[(size_t)i] = -1;
  g.live = new_live;
  // shrink a mostly empty arena
  if (g.cap > 2 * BUCKET && g.live * 4 < g.cap && g.queue.empty()) {
    const int want = std::max(BUCKET, ((2 * g.live + BUCKET - 1) / BUCKET) * BUCKET);
    EDB_TRY(resize_arena(s, g, want));
  }
  return EDB_OK;
}

edb_status tick(edb_server *s, Group &g) {
  const int S = bucket_of(g.live, g.cap);
  cudaGraphExec_t ex = nullptr;
  int nl = 0;
  EDB_TRY(step_graph(s, g, S, &ex, &nl));
  EDB_CUDA(cudaGraphLaunch(ex, g.st));
  EDB_CUDA(cudaEventRecord(g.ev, g.st));
  count_launch(nl);
  g.inflight = true;
  g.inflight_live = g.live;
  s->steps_launched += 1;
  s->launches += nl;
  s->evals += (double)g.live * s->stages;
  s->evals_padded += (double)S * s->stages;
  return EDB_OK;
}

void sort_pending(edb_server *s) {
  if (s->pending_sorted) return;
  std::stable_sort(s->pending.begin() + (long)s->pending_head, s->pending.end(),
                   [s](long long a, long long b) {
                     return s->reqs[(size_t)a].t_arrival < s->reqs[(size_t)b].t_arrival;
                   });
  s->pending_sorted = true;
}

}  // namespace

extern "C" edb_status edb_server_create(const edb_server_desc *d, edb_server **out) {
  if (!d || !out) return fail(EDB_EINVAL, "null argument");
  *out = nullptr;
  if (d->scheme != EDB_SCHEME_FE && d->scheme != EDB_SCHEME_SSP3 && d->scheme != EDB_SCHEME_RK4)
    return fail(EDB_EINVAL, "served schemes: FE, SSP3, RK4");
  if (!(d->dt > 0)) return fail(EDB_EINVAL, "dt must be positive");
  if (!(d->hbm_budget_bytes > 0)) return fail(EDB_EINVAL, "budget must be positive");
  if (d->max_live_per_group < 0) return fail(EDB_EINVAL, "max_live_per_group must be >= 0");
  EDB_TRY(ensure_device());
  edb_server *s = new edb_server();
  s->d = *d;
  s->nstage = d->scheme == EDB_SCHEME_RK4 ? 3 : (d->scheme == EDB_SCHEME_SSP3 ? 2 : 0);
  s->nq = d->scheme == EDB_SCHEME_RK4 ? 4 : 1;
  s->stages = d->scheme == EDB_SCHEME_RK4 ? 4 : (d->scheme == EDB_SCHEME_SSP3 ? 3 : 1);
  *out = s;
  return EDB_OK;
}

extern "C" edb_status edb_server_destroy(edb_server *s) {
  if (!s) return EDB_OK;
  edb_server_stop(s);
  for (auto &g : s->groups) destroy_group(*g);
  delete s;
  return EDB_OK;
}

extern "C" edb_status edb_server_prepare(edb_server *s, int N, double gamma, double R) {
  if (!s) return fail(EDB_EINVAL, "null handle");
  if (N < 3 || N > 64 || !(R > 0) || !(gamma >= 0 && gamma <= 2))
    return fail(EDB_EINVAL, "bad group");
  std::lock_guard<std::mutex> lk(s->mu);
  int gi = 0;
  return get_group(s, N, gamma, R, &gi);
}

extern "C" edb_status edb_server_submit(edb_server *s, const edb_request *r, const double *F0_real,
                                        long long *id) {
  if (!s || !r || !F0_real) return fail(EDB_EINVAL, "null argument");
  if (r->N < 3 || r->N > 64) return fail(EDB_EINVAL, "N must be in [3, 64]");
  if (!(r->R > 0)) return fail(EDB_EINVAL, "R must be positive");
  if (!(r->gamma >= 0 && r->gamma <= 2)) return fail(EDB_EINVAL, "gamma must be in [0, 2]");
  if (r->steps < 1) return fail(EDB_EINVAL, "steps must be >= 1");
  const long long NQ = (long long)r->N * r->N * r->N;
  for (long long i = 0; i < NQ; ++i)
    if (!std::isfinite(F0_real[i]))
      return fail(EDB_EINVAL, "initial data contains a NaN or an infinity (entry " +
                                  std::to_string(i) + ")");
  if (table_bytes_of(r->N) + fixed_bytes_of(r->N) + BUCKET * slot_bytes(s, r->N) >
      (long long)s->d.hbm_budget_bytes)
    return fail(EDB_ENOMEM, "request cannot fit the HBM budget");
  std::unique_lock<std::mutex> lk(s->mu);
  Req q;
  q.r = *r;
  q.F0.assign(F0_real, F0_real + NQ);
  q.t_arrival = r->arrival_s >= 0 ? r->arrival_s : now_s(s);
  const long long nid = (long long)s->reqs.size();
  if (!s->pending.empty() && s->pending_head < s->pending.size() &&
      s->reqs[(size_t)s->pending.back()].t_arrival > q.t_arrival)
    s->pending_sorted = false;
  s->reqs.push_back(std::move(q));
  s->pending.push_back(nid);
  if (id) *id = nid;
  lk.unlock();
  s->cv_work.notify_one();
  return EDB_OK;
}

namespace {
// One pass of the request loop (the caller holds s->mu): arrivals join their
// group's queue; groups whose step finished retire and compact; queues admit;
// live groups step.  *busy: work is on the device.  *stuck: requests are
// queued, nothing runs and none could be admitted (the budget is held by
// other groups' tables).
edb_status iterate(edb_server *s, bool *busy, bool *stuck) {
  const double now = now_s(s);
  sort_pending(s);
  while (s->pending_head < s->pending.size()) {
    const long long id = s->pending[s->pending_head];
    Req &r = s->reqs[(size_t)id];
    if (r.t_arrival > now) break;
    if (r.state == 4) {  // cancelled before it arrived
      ++s->pending_head;
      continue;
    }
    int gi = 0;
    EDB_TRY(get_group(s, r.r.N, r.r.gamma, r.r.R, &gi));
    s->groups[(size_t)gi]->queue.push_back(id);
    ++s->pending_head;
  }
  bool running = false, queued = false;
  for (size_t gi = 0; gi < s->groups.size(); ++gi) {
    Group &g = *s->groups[gi];
    if (g.inflight) {
      cudaError_t e = cudaEventQuery(g.ev);
      if (e == cudaErrorNotReady) {
        running = true;
        continue;
      }
      if (e != cudaSuccess) return cuda_fail(e, "server step");
      g.inflight = false;
      EDB_TRY(complete(s, g));
    }
    if (!g.queue.empty()) EDB_TRY(admit(s, g, (int)gi));
    if (g.live > 0) {
      EDB_TRY(tick(s, g));
      running = true;
    }
    queued |= !g.queue.empty();
  }
  *busy = running;
  *stuck = !running && queued;
  return EDB_OK;
}

// Retires what is still on the device (results to host, streams idle).
edb_status drain(edb_server *s) {
  for (auto &g : s->groups)
    if (g->inflight) {
      EDB_CUDA(cudaEventSynchronize(g->ev));
      g->inflight = false;
      EDB_TRY(complete(s, *g));
    }
  return EDB_OK;
}

void start_clock(edb_server *s) {
  if (!s->clock_started) {
    s->clock_started = true;
    s->t0 = Clock::now();
  }
}

// The background request loop (edb_server_start).
void loop_main(edb_server *s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (!s->stop_req) {
    bool busy = false, stuck = false;
    edb_status rc = iterate(s, &busy, &stuck);
    if (rc == EDB_OK && stuck) {
      // nothing runs and nothing fits: refuse the head of each blocked queue
      for (auto &g : s->groups)
        if (!g->queue.empty() && g->live == 0) {
          s->reqs[(size_t)g->queue.front()].state = 3;
          ++s->refused;
          g->queue.pop_front();
        }
      s->cv_done.notify_all();
    }
    if (rc != EDB_OK) {
      s->loop_status = rc;
      s->loop_msg = edb_last_error();
      break;
    }
    if (busy) {
      lk.unlock();
      std::this_thread::sleep_for(std::chrono::microseconds(20));
      lk.lock();
    } else {
      double wait = 0.002;
      if (s->pending_head < s->pending.size())
        wait = std::min(wait, s->reqs[(size_t)s->pending[s->pending_head]].t_arrival - now_s(s));
      if (wait > 0) s->cv_work.wait_for(lk, std::chrono::duration<double>(wait));
    }
  }
  if (s->loop_status == EDB_OK) {
    edb_status rc = drain(s);
    if (rc != EDB_OK) {
      s->loop_status = rc;
      s->loop_msg = edb_last_error();
    }
  }
  s->cv_done.notify_all();
}
}  // namespace

extern "C" edb_status edb_server_run(edb_server *s, double max_wall_s) {
  if (!s) return fail(EDB_EINVAL, "null handle");
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->started) return fail(EDB_EBUSY, "the background loop is running");
  start_clock(s);
  const double t_start = now_s(s);
  for (;;) {
    bool busy = false, stuck = false;
    EDB_TRY(iterate(s, &busy, &stuck));
    if (settled(s) == (long long)s->reqs.size()) break;
    if (max_wall_s > 0 && now_s(s) - t_start > max_wall_s) break;
    if (stuck) return fail(EDB_ENOMEM, "queued requests cannot be admitted within the HBM budget");
    lk.unlock();
    if (busy) {
      std::this_thread::sleep_for(std::chrono::microseconds(20));
    } else if (s->pending_head < s->pending.size()) {
      const double next = s->reqs[(size_t)s->pending[s->pending_head]].t_arrival;
      const double wait = std::min(next - now_s(s), 0.001);
      if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(wait));
    }
    lk.lock();
  }
  return drain(s);
}

extern "C" edb_status edb_server_start(edb_server *s) {
  if (!s) return fail(EDB_EINVAL, "null handle");
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->started) return fail(EDB_EBUSY, "already started");
  EDB_CUDA(cudaGetDevice(&s->device));
  start_clock(s);
  s->stop_req = false;
  s->loop_status = EDB_OK;
  try {
    s->th = std::thread(loop_main, s);
  } catch (...) {
    return fail(EDB_ENOMEM, "cannot start the request loop thread");
  }
  s->started = true;
  return EDB_OK;
}

extern "C" edb_status edb_server_stop(edb_server *s) {
  if (!s) return fail(EDB_EINVAL, "null handle");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->started) return EDB_OK;
    s->stop_req = true;
  }
  s->cv_work.notify_all();
  s->th.join();
  std::lock_guard<std::mutex> lk(s->mu);
  s->started = false;
  if (s->loop_status != EDB_OK) return fail(s->loop_status, s->loop_msg);
  return EDB_OK;
}

extern "C" edb_status edb_server_wait(edb_server *s, long long id, double timeout_s) {
  if (!s) return fail(EDB_EINVAL, "null handle");
  std::unique_lock<std::mutex> lk(s->mu);
  if (id < 0 || id >= (long long)s->reqs.size()) return fail(EDB_ENOTFOUND, "unknown request");
  auto done = [&] {
    return s->reqs[(size_t)id].state >= 2 || s->loop_status != EDB_OK || !s->started;
  };
  if (timeout_s > 0) {
    if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done))
      return fail(EDB_ETIMEDOUT, "request not finished within the timeout");
  } else {
    s->cv_done.wait(lk, done);
  }
  if (s->loop_status != EDB_OK) return fail(s->loop_status, s->loop_msg);
  const int st = s->reqs[(size_t)id].state;
  if (st == 3) return fail(EDB_ENOMEM, "request refused: it cannot fit the HBM budget");
  if (st == 4) return fail(EDB_ECANCELED, "request cancelled");
  if (st == 5) return fail(EDB_ENONFINITE, "the solve's state became non-finite");
  if (st != 2) return fail(EDB_ENOTREADY, "the loop stopped before the request finished");
  return EDB_OK;
}

extern "C" edb_status edb_server_cancel(edb_server *s, long long id) {
  if (!s) return fail(EDB_EINVAL, "null handle");
  std::unique_lock<std::mutex> lk(s->mu);
  if (id < 0 || id >= (long long)s->reqs.size()) return fail(EDB_ENOTFOUND, "unknown request");
  Req &r = s->reqs[(size_t)id];
  if (r.state == 1) {  // running: retired (slot freed) when its step in flight ends
    r.cancel = true;
    return EDB_OK;
  }
  if (r.state != 0) return fail(EDB_EINVAL, "request already finished");
  // queued in its group (arrived) or still pending (not arrived)
  for (auto &g : s->groups) {
    auto it = std::find(g->queue.begin(), g->queue.end(), id);
    if (it != g->queue.end()) {
      g->queue.erase(it);
      break;
    }
  }
  r.state = 4;
  r.t_done = now_s(s);
  std::vector<double>().swap(r.F0);
  ++s->cancelled;
  lk.unlock();
  s->cv_done.notify_all();
  s->cv_work.notify_one();
  return EDB_OK;
}

extern "C" edb_status edb_server_result(edb_server *s, long long id, double *F_real, double *Fhat,
                                        edb_request_info *info) {
  if (!s) return fail(EDB_EINVAL, "null handle");
  std::lock_guard<std::mutex> lk(s->mu);
  if (id < 0 || id >= (long long)s->reqs.size()) return fail(EDB_ENOTFOUND, "unknown request");
  const Req &r = s->reqs[(size_t)id];
  if (info) {
    info->state = r.state;
    info->N = r.r.N;
    info->steps = r.r.steps;
    info->t_arrival = r.t_arrival;
    info->t_admit = r.t_admit;
    info->t_done = r.t_done;
  }
  if (!F_real && !Fhat) return EDB_OK;
  if (r.state != 2) return fail(EDB_ENOTREADY, "request not finished");
  if (!r.r.want_result) return fail(EDB_ENOTFOUND, "result not kept (want_result = 0)");
  if (F_real) memcpy(F_real, r.F.data(), sizeof(double) * r.F.size());
  if (Fhat) memcpy(Fhat, r.Fhat.data(), sizeof(double) * r.Fhat.size());
  return EDB_OK;
}

extern "C" edb_status edb_server_clock(edb_server *s, double *t) {
  if (!s || !t) return fail(EDB_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  *t = now_s(s);
  return EDB_OK;
}

extern "C" edb_status edb_server_get_stats(edb_server *s, edb_server_stats *o) {
  if (!s || !o) return fail(EDB_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  memset(o, 0, sizeof(*o));
  std::vector<double> tts, wait;
  double first = 1e300, last = 0;
  long long live = 0, queued = 0;
  for (const Req &r : s->reqs) {
    if (r.state == 2) {
      tts.push_back(r.t_done - r.t_arrival);
      wait.push_back(r.t_admit - r.t_arrival);
      first = std::min(first, r.t_arrival);
      last = std::max(last, r.t_done);
    } else if (r.state == 1) {
      ++live;
    } else if (r.state == 0) {
      ++queued;
    }
  }
  o->submitted = (long long)s->reqs.size();
  o->completed = s->completed;
  o->live = live;
  o->queued = queued;
  o->tts_p50_s = pct(tts, 0.50);
  o->tts_p99_s = pct(tts, 0.99);
  double sum = 0, mx = 0;
  for (double v : tts) {
    sum += v;
    mx = std::max(mx, v);
  }
  o->tts_mean_s = tts.empty() ? 0 : sum / (double)tts.size();
  o->tts_max_s = mx;
  o->wait_p50_s = pct(wait, 0.50);
  o->wait_p99_s = pct(wait, 0.99);
  o->first_arrival_s = tts.empty() ? 0 : first;
  o->last_done_s = last;
  const double span = tts.empty() ? 0 : last - first;
  o->throughput_rps = span > 0 ? (double)tts.size() / span : 0;
  o->qhat_evals = s->evals;
  o->qhat_evals_padded = s->evals_padded;
  o->qhat_evals_per_s = span > 0 ? s->evals / span : 0;
  o->steps_launched = s->steps_launched;
  o->kernel_launches = s->launches;
  o->hbm_bytes_peak = s->bytes_peak;
  o->groups = (int)s->groups.size();
  o->refused = s->refused;
  o->cancelled = s->cancelled;
  o->failed = s->failed;
  return EDB_OK;
}
