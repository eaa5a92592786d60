// ela3d_noalloc.cu -- total energy of caller-owned device fields without any
// device allocation (ela3d_energy_noalloc).
//
// Who needs it: some callers cannot allocate device memory at the moment
// they want the number -- code running inside a memory-pool or allocator
// hook, host callbacks in which CUDA calls that allocate are not allowed,
// or tight real-time loops where cudaMalloc's implicit synchronisation of
// the device is unacceptable.  The plan-based ela3d_energy uses a reduction
// accumulator that its engine allocated; this entry point keeps its
// intermediate sums in a fixed array compiled into the library instead.
//
// Scratch: one double per z-plane, at most kNoAllocMaxPlanes planes
// (16384 -> 128 KiB), in the file-scope device array below.  Larger grids
// are rejected with ELA3D_ERR_INVALID_ARG.  No scratch content has to start
// at zero: each call writes every per-plane sum before it reads it.
// Calls that overlap in time on one device (other streams, other host
// threads) share that array and race with each other; serialise them.
//
// The scratch address is looked up (cudaGetSymbolAddress, on the current
// device) at every call; the first call on a device is its set-up, which
// also loads the library's kernels there.  If you capture work into a CUDA
// graph, make that first call on each device before the capture begins.
//
// Energy per cell, accumulated in FP64 (the same definition as the plan's
// stability monitor): 1/2 rho |v|^2 + (1/(4 mu)) sigma:sigma
// - lambda / (4 mu (3 lambda + 2 mu)) tr(sigma)^2 (tr(sigma)^2 / (18 lambda)
// where mu = 0), times the cell volume dx dy dz.  Per-plane sums are added
// in plane order by one block, so repeated calls give identical results.
#include <cuda_runtime.h>

#include <string>

#include "ela3d_engine.h"

namespace {
constexpr int kNoAllocMaxPlanes = 16384;
constexpr int kNoAllocThreads = 256;
}  // namespace

static __device__ __align__(256) double g_noalloc_plane_energy[kNoAllocMaxPlanes];

namespace ela3d {
namespace {

struct NoAllocFields {
  const float *f[9];  // vx vy vz sxx syy szz sxy sxz syz
  const float *cp, *cs, *rho;
  int nx, ny, nz;
  long long pitch;    // elements per row
};

__device__ __forceinline__ double block_sum(double v, double *part) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) part[warp] = v;
  __syncthreads();
  v = 0.0;
  if (warp == 0) {
    v = lane < (int)(blockDim.x >> 5) ? part[lane] : 0.0;
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  }
  return v;  // valid in thread 0
}

// One block per z-plane: the plane's energy sum into plane_sum[k].
__global__ void __launch_bounds__(kNoAllocThreads) plane_energy_kernel(NoAllocFields a, double *plane_sum) {
  __shared__ double part[kNoAllocThreads / 32];
  const int k = blockIdx.x;
  // 64-bit cell index: nx * ny may come within a block's stride of 2^31
  const long long cells = (long long)a.nx * a.ny;
  double acc = 0.0;
  for (long long q = threadIdx.x; q < cells; q += blockDim.x) {
    const long long y = q / a.nx, x = q - y * a.nx;
    const long long o = ((long long)k * a.ny + y) * a.pitch + x;
    const double rho = a.rho[o], cp = a.cp[o], cs = a.cs[o];
    const double mu = rho * cs * cs, lam = rho * (cp * cp - 2.0 * cs * cs);
    const double vx = a.f[0][o], vy = a.f[1][o], vz = a.f[2][o];
    const double sxx = a.f[3][o], syy = a.f[4][o], szz = a.f[5][o];
    const double sxy = a.f[6][o], sxz = a.f[7][o], syz = a.f[8][o];
    double e = 0.5 * rho * (vx * vx + vy * vy + vz * vz);
    const double tr = sxx + syy + szz;
    if (mu > 0.0) {
      const double ss = sxx * sxx + syy * syy + szz * szz + 2.0 * (sxy * sxy + sxz * sxz + syz * syz);
      e += ss / (4.0 * mu) - lam / (4.0 * mu * (3.0 * lam + 2.0 * mu)) * tr * tr;
    } else if (lam > 0.0) {
      e += tr * tr / (18.0 * lam);
    }
    acc += e;
  }
  acc = block_sum(acc, part);
  if (threadIdx.x == 0) plane_sum[k] = acc;
}

// One block: the per-plane sums in a fixed order, times the cell volume.
__global__ void __launch_bounds__(kNoAllocThreads) sum_planes_kernel(const double *plane_sum, int nz, double volume,
                                                                     double *out) {
  __shared__ double part[kNoAllocThreads / 32];
  double acc = 0.0;
  for (int k = threadIdx.x; k < nz; k += blockDim.x) acc += plane_sum[k];
  acc = block_sum(acc, part);
  if (threadIdx.x == 0) *out = acc * volume;
}

// The scratch array's device address on the current device.  It is looked
// up on every call (cudaGetSymbolAddress allocates nothing), so a device or
// context reset, after which the library's module is loaded again and the
// array may sit elsewhere, needs no special care.  The first call on a
// device also loads the library's kernels there.
ela3d_status noalloc_scratch(double **out) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_plane_energy);
  if (e != cudaSuccess) return status_from_cuda(e, "cudaGetSymbolAddress");
  *out = static_cast<double *>(p);
  return ELA3D_OK;
}

}  // namespace
}  // namespace ela3d

using namespace ela3d;

extern "C" ela3d_status ela3d_energy_noalloc(const float *const *fields, const float *cp, const float *cs,
                                             const float *rho, int32_t nx, int32_t ny, int32_t nz, int32_t pitch_x,
                                             double dx, double dy, double dz, double *out, void *stream) {
  if (!fields || !cp || !cs || !rho || !out) {
    set_last_error("ela3d_energy_noalloc: null pointer");
    return ELA3D_ERR_INVALID_ARG;
  }
  for (int c = 0; c < 9; ++c)
    if (!fields[c]) {
      set_last_error("ela3d_energy_noalloc: field " + std::to_string(c) + " is null");
      return ELA3D_ERR_INVALID_ARG;
    }
  if (nx < 1 || ny < 1 || nz < 1 || pitch_x < nx || !(dx > 0 && dy > 0 && dz > 0)) {
    set_last_error("ela3d_energy_noalloc: grid sizes and spacings must be positive and pitch_x >= nx");
    return ELA3D_ERR_INVALID_ARG;
  }
  if (nz > kNoAllocMaxPlanes) {
    set_last_error("ela3d_energy_noalloc: nz = " + std::to_string(nz) + " exceeds the " +
                   std::to_string(kNoAllocMaxPlanes) + " planes its fixed scratch holds");
    return ELA3D_ERR_INVALID_ARG;
  }
  if ((long long)nx * ny > (1ll << 31) - 1) {
    set_last_error("ela3d_energy_noalloc: nx * ny must fit in 31 bits");
    return ELA3D_ERR_INVALID_ARG;
  }
  double *scratch = nullptr;
  ela3d_status st = noalloc_scratch(&scratch);
  if (st != ELA3D_OK) return st;
  NoAllocFields a{};
  for (int c = 0; c < 9; ++c) a.f[c] = fields[c];
  a.cp = cp;
  a.cs = cs;
  a.rho = rho;
  a.nx = nx;
  a.ny = ny;
  a.nz = nz;
  a.pitch = pitch_x;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  plane_energy_kernel<<<nz, kNoAllocThreads, 0, s>>>(a, scratch);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return status_from_cuda(e, "plane_energy_kernel launch");
  sum_planes_kernel<<<1, kNoAllocThreads, 0, s>>>(scratch, nz, dx * dy * dz, out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return status_from_cuda(e, "sum_planes_kernel launch");
  return ELA3D_OK;
}
