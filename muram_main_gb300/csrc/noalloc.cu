// MHD_Residual's CFL time step without any device allocation.
//
// Some callers hold device pointers to MURaM's fields but must not allocate
// device memory themselves: a MURaM build whose arrays belong to the OpenACC
// runtime (acc_create / present clauses) must not allocate behind that
// runtime's back, and a time-step loop cannot afford cudaMalloc, which may
// synchronise the whole device.  gpumhd_cfl_dt_noalloc serves them: it reads
// the caller's primitive state and pressure, and writes dt_mhd to the
// caller's device double, using only the fixed scratch array below.
//
// The scratch is a file-scope __device__ array of GPUMHD_NOALLOC_MAX_PLANES
// doubles (32 KiB): one partial maximum per z plane of the box including its
// ghost layers.  Every GPU that loads the library holds it until the process
// exits.  All calls share it, and it keeps the last call's contents; each call
// rewrites every slot it later reads, so nothing from an earlier call is used,
// but calls that overlap on the GPU (e.g. on two streams at once) race on it.
//
// Compiled like kernels_f64.cu (no FMA contraction): the CFL speed of each
// cell is the same expression as in the per-routine MHD_Residual path.
#include <cuda_runtime.h>

#include "../../include/gpumhd.h"
#include "gpumhd_dev.cuh"

using namespace gpumhd;

#define GPUMHD_NOALLOC_MAX_PLANES 4096
#define GPUMHD_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double g_noalloc_scratch[GPUMHD_NOALLOC_MAX_PLANES];

namespace {

// Host-side address of the scratch array on each device (the symbol name
// itself is only a host stand-in, not a device address).
double* g_scratch_ptr[GPUMHD_NOALLOC_MAX_DEVICES] = {nullptr};

// One block per z plane: the CFL speed over the plane's cells that
// MHD_Residual's pencils visit -- interior cells, and the face ghosts (one
// coordinate in a ghost layer, the other two interior).  The block maximum,
// NaN ignored as std::max does in the reference, goes to partial[k].
__global__ void k_cfl_planes(Geom g, const double* __restrict__ U, const double* __restrict__ P, double inv_va2max,
                             double* __restrict__ partial) {
  const int k = blockIdx.x;
  const bool kin = (k >= GH && k < GH + g.nz);
  double cm = 0.0;
  for (int t = threadIdx.x; t < g.sx * g.sy; t += blockDim.x) {
    const int i = t % g.sx, j = t / g.sx;
    const bool iin = (i >= GH && i < GH + g.nx), jin = (j >= GH && j < GH + g.ny);
    const int outside = (iin ? 0 : 1) + (jin ? 0 : 1) + (kin ? 0 : 1);
    if (outside > 1) continue;
    const long long id = cidx(g, i, j, k);
    const double v = cmax_cell<double>(U[id], U[g.N + id], U[2 * g.N + id], U[3 * g.N + id], U[5 * g.N + id],
                                       U[6 * g.N + id], U[7 * g.N + id], P[id], inv_va2max);
    cm = smax(cm, v);
  }
  cm = warp_max_nonnan(cm);
  __shared__ double wm[32];
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = cm;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) m = smax(m, wm[w]);
    partial[k] = m;
  }
}

// One block: maximum of the plane partials, then dt_mhd = dxmin / cmax.
__global__ void k_cfl_finish(int nplanes, double dxmin, const double* __restrict__ partial, double* __restrict__ dt_out) {
  double cm = 0.0;
  for (int k = threadIdx.x; k < nplanes; k += blockDim.x) cm = smax(cm, partial[k]);
  cm = warp_max_nonnan(cm);
  __shared__ double wm[32];
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = cm;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) m = smax(m, wm[w]);
    *dt_out = dxmin / m;
  }
}

}  // namespace

extern "C" int gpumhd_cfl_dt_noalloc(const double* U_prim, const double* pres, int nx, int ny, int nz,
                                     const double dx[3], double inv_va2max, void* stream, double* dt_out) {
  if (!U_prim || !pres || !dx || !dt_out || nx < 4 || ny < 4 || nz < 4) return GPUMHD_E_INVALID;
  if (nz + 2 * GH > GPUMHD_NOALLOC_MAX_PLANES) return GPUMHD_E_INVALID;  // more planes than the scratch holds
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= GPUMHD_NOALLOC_MAX_DEVICES) return GPUMHD_E_CUDA;
  if (!g_scratch_ptr[dev]) {
    // first call on this device: look up the device address of the scratch array
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return GPUMHD_E_CUDA;
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  Geom g;
  g.nx = nx; g.ny = ny; g.nz = nz;
  g.sx = nx + 2 * GH; g.sy = ny + 2 * GH; g.sz = nz + 2 * GH;
  g.N = (long long)g.sx * g.sy * g.sz;
  g.periodic_x = 1;
  g.N32 = (unsigned)g.N;
  double dxmin = dx[0];
  for (int d = 1; d < 3; d++) dxmin = (dx[d] < dxmin) ? dx[d] : dxmin;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_cfl_planes<<<g.sz, 256, 0, s>>>(g, U_prim, pres, inv_va2max, g_scratch_ptr[dev]);
  k_cfl_finish<<<1, 256, 0, s>>>(g.sz, dxmin, g_scratch_ptr[dev], dt_out);
  return cudaGetLastError() == cudaSuccess ? GPUMHD_OK : GPUMHD_E_CUDA;
}
