// FP64 collision sum for callers that cannot allocate device memory.
//
// edb_qcalc_calQ_device needs a partial-sum buffer that its handle allocates
// with cudaMalloc.  Some callers of this library may not call cudaMalloc at all:
// a host application that owns a fixed device pool and accounts for every
// byte of it, a plugin loaded into such a host, or a real-time loop that
// cannot afford the implicit device-wide synchronisation of cudaMalloc and
// cudaFree.  edb_calQ_fp64_noalloc serves them: the caller passes the table,
// the input and the output (all memory it already owns), and the partial sums
// live in the fixed device array below, which the CUDA runtime places in the
// module's global memory when the module loads on a device.
//
// The array's name, used in host code, is only a host-side stand-in for the
// device symbol and is never handed to a kernel.  Its device address is
// looked up with cudaGetSymbolAddress once per device context, with that
// device current, on the entry point's first call there (and again after the
// device's primary context was reset, which reloads the module at another
// address); that first call should therefore come before any stream capture.  Every call on a device reuses
// the same array, so calls that overlap on the GPU (two streams, or two host
// threads) race on it; serialise them.  The array keeps the previous call's
// contents; nothing needs clearing, because every partial sum is written
// before it is read.
#include <cuda.h>

#include <mutex>

#include "edb_internal.cuh"

namespace {

// 5 MiB of partial sums: 327,680 complex doubles.  The FP64 sum uses
// nchunk * P^3 of them (nchunk l-chunks of the P^3 outputs); the largest
// need for any N in [3, 64] is 297,754 (N = 53).
constexpr long long kNoallocScratchEntries = 327680;
static __device__ __align__(256) double2 g_noalloc_scratch[kNoallocScratchEntries];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
double2 *g_scratch_addr[kMaxDevices] = {};
CUcontext g_scratch_ctx[kMaxDevices] = {};  // context the address belongs to

// cuCtxGetCurrent from the driver, through the runtime's entry-point query
// (the library links no driver stub).
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
CtxGetCurrentFn ctx_get_current() {
  static const CtxGetCurrentFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<CtxGetCurrentFn>(p);
  }();
  return fn;
}

}  // namespace

using namespace edb;

extern "C" edb_status edb_calQ_fp64_noalloc(int N, int index_mode, const double *d_B,
                                            const double *d_fin, double *d_Qout, void *stream) {
  if (!d_B || !d_fin || !d_Qout) return fail(EDB_EINVAL, "null device pointer");
  if (N < 3 || N > 64) return fail(EDB_EINVAL, "noalloc calQ: N must be in [3, 64]");
  if (index_mode != EDB_INDEX_REFERENCE && index_mode != EDB_INDEX_ALIASED)
    return fail(EDB_EINVAL, "unknown index mode");
  const QParams p = make_qparams(N, index_mode);
  const long long need = (long long)calq64_nchunk(p) * p.KC;
  if (need > kNoallocScratchEntries)
    return fail(EDB_EINVAL, "noalloc calQ: needs " + std::to_string(need * 16) +
                                " bytes of partial sums, above the fixed 5 MiB array");
  int dev = 0;
  EDB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(EDB_EINVAL, "device ordinal out of range");
  // the runtime makes the device's primary context current on its first call;
  // cudaFree(0) would too, but this entry point must not call it
  CUcontext ctx = nullptr;
  const CtxGetCurrentFn get_ctx = ctx_get_current();
  if (!get_ctx) return fail(EDB_ECUDA, "noalloc calQ: cuCtxGetCurrent is not available");
  double2 *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (get_ctx(&ctx) != CUDA_SUCCESS) ctx = nullptr;
    if (!g_scratch_addr[dev] || !ctx || ctx != g_scratch_ctx[dev]) {
      void *addr = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
      if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(noalloc scratch)");
      g_scratch_addr[dev] = static_cast<double2 *>(addr);
      // the symbol lookup has made the primary context current
      if (get_ctx(&ctx) != CUDA_SUCCESS) ctx = nullptr;
      g_scratch_ctx[dev] = ctx;
    }
    scratch = g_scratch_addr[dev];
  }
  return launch_calq64(p, d_B, reinterpret_cast<const double2 *>(d_fin), scratch,
                       reinterpret_cast<double2 *>(d_Qout), (cudaStream_t)stream);
}
