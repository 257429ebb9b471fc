// Free streaming in x for spatially inhomogeneous use of the collision step.
//
// The reference solves the space-homogeneous equation only (BKW.h integrates
// df/dt = Q(f) for one velocity distribution).  The inhomogeneous equation
//   df/dt + v1 df/dx = Q(f)
// on a periodic 1-D x grid of C cells splits into a transport step (this
// kernel) and one homogeneous collision step per cell (the batched solver,
// one solve per cell), e.g. Strang: transport dt/2, collide dt, transport dt/2.
//
// Layout: cells-major, f[c][v] with v the N^3 velocity grid points
// v_d = -R + i_d h, h = 2R/N (row-major [i1][i2][i3], as BKW.h:124-133), so
// one cell's distribution is the contiguous N^3 block a batched solve reads.
//
// Scheme: semi-Lagrangian with linear interpolation.  The foot of the
// characteristic through x_c is x_c - v1 dt, s = v1 dt / dx cells upstream,
// s = n + theta with n = floor(s):
//   f_out[c][v] = (1 - theta) f[(c - n) mod C][v] + theta f[(c - n - 1) mod C][v].
// For each velocity the weights sum to one over the periodic grid, so the
// total of every velocity slice (and with it mass, momentum and energy) is
// kept exactly up to rounding; the weights are non-negative, so f >= 0 is
// kept; theta = 0 (an integer shift) is exact.  HBM-bound: one read of two
// neighbours and one write per entry, coalesced along v.
#include <math.h>

#include <cmath>

#include "edb_internal.cuh"

namespace edb {

__global__ void transport_x_kernel(int C, int N, double R, double dx, double dt,
                                   const double *__restrict__ f, double *__restrict__ out) {
  const long long NQ = (long long)N * N * N;
  const long long total = (long long)C * NQ;
  const double h = 2.0 * R / N;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long c = idx / NQ, v = idx - c * NQ;
    const int i1 = (int)(v / ((long long)N * N));
    const double v1 = -R + i1 * h;
    const double s = v1 * dt / dx;
    const double fl = floor(s);
    const double theta = s - fl;
    // n mod C as a non-negative shift (|n| may exceed C for large dt)
    long long n = (long long)fl % C;
    if (n < 0) n += C;
    long long c0 = c - n;
    if (c0 < 0) c0 += C;
    const long long c1 = (c0 == 0) ? C - 1 : c0 - 1;
    const double a = __ldg(f + c0 * NQ + v), b = __ldg(f + c1 * NQ + v);
    out[idx] = (1.0 - theta) * a + theta * b;
  }
}

edb_status launch_transport_x(int C, int N, double R, double Lx, double dt, const double *d_f,
                              double *d_out, cudaStream_t st) {
  const long long total = (long long)C * N * N * N;
  const long long cap = 32LL * device_sm_count();
  const long long blocks = (total + 255) / 256 < cap ? (total + 255) / 256 : cap;
  transport_x_kernel<<<(unsigned)blocks, 256, 0, st>>>(C, N, R, Lx / C, dt, d_f, d_out);
  EDB_LAUNCHED();
  return EDB_OK;
}

}  // namespace edb

using namespace edb;

extern "C" edb_status edb_cells_transport_x_device(int C, int N, double R, double Lx, double dt,
                                                   const double *d_f, double *d_out,
                                                   void *stream) {
  if (C < 1 || N < 3 || N > 64 || !(R > 0) || !(Lx > 0) || !std::isfinite(dt))
    return fail(EDB_EINVAL, "transport: bad argument");
  if (!d_f || !d_out) return fail(EDB_EINVAL, "transport: null device pointer");
  if (d_f == d_out) return fail(EDB_EINVAL, "transport: input and output must differ");
  EDB_TRY(ensure_device());
  return launch_transport_x(C, N, R, Lx, dt, d_f, d_out, (cudaStream_t)stream);
}
