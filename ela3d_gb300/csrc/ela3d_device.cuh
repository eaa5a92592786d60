// ela3d_device.cuh -- device-side data structures and PTX helpers shared by
// the stencil kernels (ela3d_stencil.cu), the auxiliary kernels
// (ela3d_aux.cu) and the host engine (ela3d_engine.cu).
//
// Device layout of one shot (all arrays 256-byte aligned):
//   fields vx vy vz sxx syy szz sxy sxz syz and model cp cs rho:
//     [nz][ny][px], x fastest, px = nx rounded up to 128 bytes; the columns
//     [nx, px) are zero and never updated.
//   C-PML memory variables only inside the six PML slabs, six per axis
//   (three for the stress half-step, three for the velocity half-step):
//     x slab: [6][nz][ny][xw], cells x < xl and x >= xr (xw = xl + px - xr)
//     y slab: [6][nz][yw][px], rows  y < yl and y >= yr (yw = yl + ny - yr)
//     z slab: [6][zw][ny][px], planes z < zl and z >= zr (zw = zl + nz - zr)
//   Outside the slabs the reference's memory variables stay exactly 0
//   (a = 0 there, so psi = b*0 + 0*d = 0), which is why they are not stored.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace ela3d {

// Device error bits, OR-ed into the engine's error word.
enum : unsigned {
  DEV_ERR_TIMEOUT = 1u,     // an mbarrier wait exceeded its limit
  DEV_ERR_BAD_ITEM = 2u,    // a work item outside its shot's grid
};

// Wall-clock limit of one device-side wait (ns).  A wait normally ends in
// microseconds; the limit only turns a lost transfer into an error status.
constexpr unsigned long long kWaitLimitNs = 2000000000ull;
// Limit used when a test asks for the timeout path (20 ms).
constexpr unsigned long long kTestWaitLimitNs = 20000000ull;

// Kernel control word.  CTL_WITHHOLD_LOADS makes the producer issue no
// loads, so every consumer wait expires and the kernel returns
// DEV_ERR_TIMEOUT: the failure path of a lost transfer, exercised without a
// fault (the waits are bounded, nothing spins forever).
// CTL_PF_X lets the producer warp prefetch into L1 the C-PML memory
// variables of the x slab, CTL_PF_YZ those of the y and z slabs into L2
// (performance hints; results do not depend on them).
enum : int { CTL_WITHHOLD_LOADS = 1, CTL_PF_X = 2, CTL_PF_YZ = 4 };

// How a kernel's loading warp fills a stage: one lane issues TMA tiled loads
// (LOAD_TMA, every production variant), or all 32 lanes copy 16-byte chunks
// with cp.async (LOAD_CP_ASYNC, kept as the measured alternative).
enum : int { LOAD_TMA = 0, LOAD_CP_ASYNC = 1 };

// Which psi variable of an axis.  Stress half-step: S0..S2, velocity: V0..V2.
//  x: S0 dvx_dx(half) S1 dvy_dx S2 dvz_dx | V0 dsxx_dx V1 dsxy_dx(half) V2 dsxz_dx(half)
//  y: S0 dvy_dy S1 dvx_dy(half) S2 dvz_dy(half) | V0 dsxy_dy V1 dsyy_dy(half) V2 dsyz_dy
//  z: S0 dvz_dz S1 dvx_dz(half) S2 dvy_dz(half) | V0 dsxz_dz V1 dsyz_dz V2 dszz_dz(half)
enum { PSI_S0 = 0, PSI_S1, PSI_S2, PSI_V0, PSI_V1, PSI_V2 };

// Profile array order inside prof (per axis, n = px for x, ny, nz):
//  a_full b_full iK_full a_half b_half iK_half  (iK = 1/K)
enum { PR_A = 0, PR_B, PR_IK, PR_AH, PR_BH, PR_IKH };

template <typename T>
struct ShotDesc {
  int nx, ny, nz, px;
  int tick0;          // step it of this shot = tick - tick0 (1-based)
  int nstep;
  int xl, xr, xw;
  int yl, yr, yw;
  int zl, zr, zw;
  int src_i, src_j, src_k, src_kind;
  int nrec, nsamp, sampgat;
  T dt, idx, idy, idz;
  T src_w[3];         // force weights
  T expl_w[3];        // explosive weights for sxx, syy, szz
  T *f[9];            // vx vy vz sxx syy szz sxy sxz syz
  const T *cp, *cs, *rho;
  T *psi_x, *psi_y, *psi_z;
  long long psx, psy, psz;   // elements per psi variable
  const T *prof_x, *prof_y, *prof_z;
  const T *stf;              // nstep values, stf[it-1]
  const int *rec_plane;      // nz+1 offsets into rec_sorted
  const int4 *rec_sorted;    // (i, j, k, receiver index) sorted by (k, j, i)
  T *seis;                   // [nrec][3][nsamp]
  T *src_trace;              // [3][nstep + 1]: the source cell's injected components
                             // (sxx syy szz, or vx vy vz for a force) after step it's
                             // injection at index it; index 0 stays 0
  int *flow_flags;           // dataflow kernel: completion counters [2][flow_chunks][tiles]
  int flow_chunks;           // z-chunks of the dataflow schedule (0: none)
};

// Tensor maps of one shot.  Box shapes (TX, TY = tile; H = 16 bytes of T):
//  stress:   0 vx (TX+H)x(TY+1) at (x0,y0)     1 vy (TX+H)x(TY+1) at (x0-H,y0-1)
//            2 vz (TX+H)x(TY+1) at (x0-H,y0)   3 cs, 4 rho like vz
//            5 cp, 6..11 sxx syy szz sxy sxz syz  TX x TY at (x0,y0)
//  velocity: 0 sxx (TX+H)xTY at (x0-H,y0)      1 syy TXx(TY+1) at (x0,y0)
//            2 szz TXxTY                       3 sxy (TX+H)x(TY+1) at (x0,y0-1)
//            4 sxz (TX+H)xTY at (x0,y0)        5 syz TXx(TY+1) at (x0,y0-1)
//            6 rho (TX+H)x(TY+1) at (x0-H,y0)  7 vx, 8 vy, 9 vz  TX x TY
struct ShotMaps {
  CUtensorMap stress[12];
  CUtensorMap vel[10];
};

// One work item: a z-run [k0, k1) of one x-y tile of one shot.
struct Item {
  int shot, tile, k0, k1;
};

// A work item of the dataflow kernel: the stress (kind 0) or velocity
// (kind 1) half-step of one item at step `step` of the launch, in z-chunk
// `chunk` of the shot's dataflow schedule.
struct FlowItem {
  Item it;
  int kind, step, chunk, pad;
};

// ---------------------------------------------------------------- PTX ----
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Waits for the phase with the given parity to complete.  Returns false if
// the wall-clock limit passed first (the caller reports DEV_ERR_TIMEOUT).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  unsigned long long limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (globaltimer_ns() - t0 > limit_ns) return false;
  }
}

// 3-D tiled TMA load of one box into shared memory, completing on bar.
// x must be a multiple of 16 bytes of elements (all boxes here start at
// x0 or x0 - 16 bytes with x0 a multiple of the tile width).
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cta.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// 16-byte asynchronous copy global -> shared through L2 (cp.async.cg);
// the first src_bytes (0..16) are read, the rest of the 16 are zero-filled.
// Both addresses 16-byte aligned.
__device__ __forceinline__ void cp_async_16(void *dst, const void *src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}

// Arrive on bar once every cp.async this thread issued before has landed
// (the barrier's expected count includes this arrival).
__device__ __forceinline__ void cp_async_arrive_noinc(uint64_t *bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap *map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// 16-byte vector of T (the TMA x granule).
template <typename T> struct Vec;
template <> struct Vec<float> {
  static constexpr int N = 4;
  using V = float4;
};
template <> struct Vec<double> {
  static constexpr int N = 2;
  using V = double2;
};

// N consecutive T as one load/store (N * sizeof(T) = 4 .. 16 bytes).
template <typename T, int N> struct VType;
template <> struct VType<float, 4> { using V = float4; };
template <> struct VType<float, 2> { using V = float2; };
template <> struct VType<float, 1> { using V = float; };
template <> struct VType<double, 2> { using V = double2; };
template <> struct VType<double, 1> { using V = double; };

template <typename T, int N>
__device__ __forceinline__ void unpack(const typename VType<T, N>::V &v, T (&o)[N]) {
  if constexpr (N == 4) {
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  } else if constexpr (N == 2) {
    o[0] = v.x; o[1] = v.y;
  } else {
    o[0] = v;
  }
}

template <typename T, int N>
__device__ __forceinline__ typename VType<T, N>::V pack(const T (&o)[N]) {
  typename VType<T, N>::V v;
  if constexpr (N == 4) {
    v.x = o[0]; v.y = o[1]; v.z = o[2]; v.w = o[3];
  } else if constexpr (N == 2) {
    v.x = o[0]; v.y = o[1];
  } else {
    v = o[0];
  }
  return v;
}

template <typename T, int N>
__device__ __forceinline__ void ld_vec(const T *p, T (&o)[N]) {
  unpack<T, N>(*reinterpret_cast<const typename VType<T, N>::V *>(p), o);
}

// read-only path (profiles)
template <typename T, int N>
__device__ __forceinline__ void ld_vec_global(const T *p, T (&o)[N]) {
  unpack<T, N>(__ldg(reinterpret_cast<const typename VType<T, N>::V *>(p)), o);
}

// Plain (coherent) load, for data written by earlier kernels of the same
// stream that this kernel may also write (psi).
template <typename T, int N>
__device__ __forceinline__ void ld_vec_rw(const T *p, T (&o)[N]) {
  unpack<T, N>(*reinterpret_cast<const typename VType<T, N>::V *>(p), o);
}

template <typename T, int N>
__device__ __forceinline__ void st_vec(T *p, const T (&o)[N]) {
  *reinterpret_cast<typename VType<T, N>::V *>(p) = pack<T, N>(o);
}

}  // namespace ela3d
