// ela3d_stencil.cuh -- the two time-loop kernels: stress half-step and
// velocity half-step, templated on the real type and the x-y tile.
//
// Scheme (2.5-D z-march, one launch per half-step):
//  - a block owns a list of work items (shot, x-y tile, z-run [k0, k1));
//  - one producer warp walks the block's planes and, for each, issues TMA
//    tiled loads of every input array's x-y tile (with the one-cell halos
//    the stencil needs) into a ring of NS shared-memory stages; each stage
//    has a "full" mbarrier (TMA bytes landed) and an "empty" mbarrier (all
//    consumer warps done), so refills start as soon as a stage is released;
//  - out-of-grid halo cells arrive as zeros (the TMA fill), which is also
//    the zero plane above k = nz-1 that the reference's sigma_xz/sigma_yz
//    loop reads (simpelmodel.cpp:450,477);
//  - consumer warps compute plane k from stages k and k+1 (the z+1
//    neighbours) and keep the z-1 neighbours in registers; each thread owns
//    16 bytes of consecutive x cells of one row (float4 / double2);
//  - C-PML memory variables are read and written only in the PML slabs;
//  - cells outside the update ranges of the reference's loops keep their
//    value (the Dirichlet edges); receivers are sampled after the velocity
//    update and the force source is added after that (simpelmodel.cpp:592-622).
// Every wait is bounded: on expiry the kernel ORs DEV_ERR_TIMEOUT into the
// error word, the producer waits (bounded) for its issued copies, and the
// threads return.
#pragma once

#include <type_traits>

#include "ela3d_device.cuh"

namespace ela3d {

template <typename T, int TX_, int TY_, int NS_, int CPT_ = Vec<T>::N, int MINB_ = 0>
struct Geo {
  static constexpr int VEC = CPT_;       // cells per thread (consecutive in x)
  static constexpr int H = Vec<T>::N;    // halo width in x (16 bytes, the TMA x alignment)
  static constexpr int TX = TX_, TY = TY_, NS = NS_;
  static constexpr int NTX = TX / VEC;
  static constexpr int NT = NTX * TY;      // consumer threads
  static constexpr int NCW = NT / 32;      // consumer warps
  static constexpr int THREADS = NT + 32;  // + one producer warp
  // blocks per SM the register budget is sized for (64K registers per SM):
  // two blocks of four warps keep 255 registers per thread; fewer cells per
  // thread trade registers for resident warps
  static constexpr int MINB = MINB_ ? MINB_ : (THREADS <= 128 ? 2 : 1);
  static constexpr int WW = TX + H;
  static_assert(H % VEC == 0 && TX % H == 0 && TX + H <= 256 && TY + 1 <= 256, "tile shape");
  static_assert(NT % 32 == 0, "consumer threads must fill whole warps");
  __host__ __device__ static constexpr int al(int b) { return (b + 127) & ~127; }
  static constexpr int C = TX * TY;          // center box
  static constexpr int W1 = WW * (TY + 1);   // wide box with one extra row
  static constexpr int W0 = WW * TY;         // wide box
  static constexpr int Y1 = TX * (TY + 1);   // narrow box with one extra row
  __host__ __device__ static constexpr int sz(int e) { return al(e * (int)sizeof(T)); }
  static constexpr int SC = (C * (int)sizeof(T) + 127) & ~127;  // bytes of a centre box
  // stress stage: vx vy vz cs rho (W1), cp s0..s5 (C)
  static constexpr int S_VX = 0;
  static constexpr int S_VY = S_VX + sz(W1);
  static constexpr int S_VZ = S_VY + sz(W1);
  static constexpr int S_CS = S_VZ + sz(W1);
  static constexpr int S_RHO = S_CS + sz(W1);
  static constexpr int S_CP = S_RHO + sz(W1);
  static constexpr int S_SIG = S_CP + sz(C);  // six centre boxes follow
  static constexpr int S_STAGE = S_SIG + 6 * sz(C);
  static constexpr int S_TX = (int)sizeof(T) * (5 * W1 + 7 * C);
  // velocity stage
  static constexpr int V_SXX = 0;                 // W0
  static constexpr int V_SYY = V_SXX + sz(W0);    // Y1
  static constexpr int V_SZZ = V_SYY + sz(Y1);    // C
  static constexpr int V_SXY = V_SZZ + sz(C);     // W1
  static constexpr int V_SXZ = V_SXY + sz(W1);    // W0
  static constexpr int V_SYZ = V_SXZ + sz(W0);    // Y1
  static constexpr int V_RHO = V_SYZ + sz(Y1);    // W1
  static constexpr int V_V = V_RHO + sz(W1);      // vx vy vz (C)
  static constexpr int V_STAGE = V_V + 3 * sz(C);
  static constexpr int V_TX = (int)sizeof(T) * (2 * W0 + 2 * Y1 + 4 * C + 2 * W1);
  // mbarriers (full[NS], empty[NS]) live after the stages, so the TMA
  // destinations start at the (aligned) base of dynamic shared memory
  static constexpr int S_SMEM = NS * S_STAGE + 16 * NS;
  static constexpr int V_SMEM = NS * V_STAGE + 16 * NS;
};

template <typename T>
__device__ __forceinline__ int tiles_x_of(const ShotDesc<T> &s, int TX) {
  return (s.nx + TX - 1) / TX;
}

// dt / rho_avg: FP32 uses the hardware reciprocal-based divide (<= 2 ulp
// from the IEEE quotient); FP64 keeps the IEEE division.
__device__ __forceinline__ float div_fast(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double div_fast(double a, double b) { return a / b; }

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// L1 prefetch of every 128-byte line of [p, p + bytes).
__device__ __forceinline__ void prefetch_l1(const void *p, int bytes) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(p);
  for (uintptr_t q = a & ~uintptr_t(127); q < a + (uintptr_t)bytes; q += 128)
    asm volatile("prefetch.global.L1 [%0];" ::"l"(q));
}

// L1 prefetch of the x-slab C-PML memory variables var0 .. var0+2 that the
// consumers of a tile will load: every row of the tile crosses the x slab
// at the tile's edge columns, so without it every consumer warp waits on
// DRAM once per plane.  Issued by the producer warp's lanes (one (variable,
// row) pair per lane) when a plane's stage is requested, NS-2 planes ahead
// of the consumers.  A hint: no result depends on it.  (Prefetching the y
// and z slabs into L1 the same way measured slower: whole warps load those
// rows and planes, and the extra lines crowd L1.)
// The y- and z-slab rows are brought into L2 instead (CTL_PF_YZ), with bulk
// prefetches that need no L1 space.
__device__ __forceinline__ void prefetch_l2_bulk(const void *p, int bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

template <typename T, int TX, int TY>
struct PsiPrefetch {
  const T *left = nullptr, *right = nullptr;  // this lane's x-slab segments at plane 0
  const T *yrow = nullptr, *zrow = nullptr;   // this lane's y-slab row at plane 0, z-slab row at slab plane 0
  int lbytes = 0, rbytes = 0, wbytes = 0;
  long long pstride = 0, ystride = 0, zstride = 0;  // elements per plane of the x, y and z slabs
  int nz = 0, zl = 0, zr = 0;
  __device__ __forceinline__ void begin(const ShotDesc<T> &sd, int x0, int y0, int var0, int lane, int ctl) {
    const int rows = min(TY, sd.ny - y0);
    lbytes = rbytes = wbytes = 0;
    yrow = zrow = nullptr;
    nz = sd.nz;
    zl = sd.zl;
    zr = sd.zr;
    pstride = (long long)sd.ny * sd.xw;
    ystride = (long long)sd.yw * sd.px;
    zstride = (long long)sd.ny * sd.px;
    if (lane >= 3 * rows) return;
    const int var = var0 + lane / rows, y = y0 + lane % rows;
    if (ctl & CTL_PF_X) {
      const T *row = sd.psi_x + var * sd.psx + (long long)y * sd.xw;
      const int xb = min(x0 + TX, sd.xl);
      const int xc = max(x0, sd.xr), xd = min(x0 + TX, sd.px);
      if (x0 < xb) { left = row + x0; lbytes = (xb - x0) * (int)sizeof(T); }
      if (xc < xd) { right = row + sd.xl + (xc - sd.xr); rbytes = (xd - xc) * (int)sizeof(T); }
    }
    if (ctl & CTL_PF_YZ) {
      wbytes = min(TX, sd.px - x0) * (int)sizeof(T);
      if (y < sd.yl || y >= sd.yr) {
        const int ys = y < sd.yl ? y : sd.yl + (y - sd.yr);
        yrow = sd.psi_y + var * sd.psy + (long long)ys * sd.px + x0;
      }
      zrow = sd.psi_z + var * sd.psz + (long long)y * sd.px + x0;
    }
  }
  __device__ __forceinline__ void plane(int k) const {
    if (k < 0 || k >= nz) return;
    if (lbytes) prefetch_l1(left + k * pstride, lbytes);
    if (rbytes) prefetch_l1(right + k * pstride, rbytes);
    if (yrow) prefetch_l2_bulk(yrow + k * ystride, wbytes);
    if (zrow && (k < zl || k >= zr)) prefetch_l2_bulk(zrow + (k < zl ? k : zl + (k - zr)) * zstride, wbytes);
  }
};

// cp.async counterpart of one TMA box load: the BW x BH box of plane k of
// `base` with origin (x, y), stored densely row by row like the TMA box;
// cells outside [0, nx) x [0, ny) x [0, nz) read as zeros.  Each lane copies
// every 32nd 16-byte chunk.
template <typename T, int BW, int BH>
__device__ __forceinline__ void copy_box_async(unsigned char *dst, const T *base, const ShotDesc<T> &sd, int x, int y,
                                               int k, int lane) {
  constexpr int E = 16 / (int)sizeof(T);  // elements per chunk
  constexpr int CPR = BW / E, N = CPR * BH;
  static_assert(BW % E == 0, "box rows are whole chunks");
  const bool kin = k >= 0 && k < sd.nz;
  for (int c = lane; c < N; c += 32) {
    const int r = c / CPR, xx = x + (c - r * CPR) * E, yy = y + r;
    uint32_t bytes = 0;
    const T *src = base;
    if (kin && yy >= 0 && yy < sd.ny && xx >= 0 && xx < sd.nx) {
      bytes = (uint32_t)(min(E, sd.nx - xx) * (int)sizeof(T));
      src = base + ((long long)k * sd.ny + yy) * sd.px + xx;
    }
    cp_async_16(dst + (size_t)c * 16, src, bytes);
  }
}


// Producer warp: walks the block's items and issues every plane's loads
// (lane 0) and the plane's memory-variable prefetches (all lanes).  Load n
// goes to stage n % NS; before reusing a stage lane 0 waits for the
// consumers' release of load n - NS on that stage's empty barrier.  Item i
// contributes planes k0 .. k1 (k1 is the look-ahead plane, possibly nz,
// which the TMA fills with zeros).
// With ASYNC every lane copies a share of each plane's boxes (cp.async)
// instead of lane 0 issuing TMA loads.
template <int NS, bool ASYNC, typename Issue, typename Prefetch>
__device__ __forceinline__ bool produce_item(const Item &it, unsigned &n, uint64_t *full, uint64_t *empty,
                                             Issue issue, Prefetch &prefetch, int lane) {
  prefetch.begin(it);
  for (int k = it.k0; k <= it.k1; ++k, ++n) {
    const int slot = (int)(n % NS);
    int good = 1;
    if (lane == 0 && n >= NS) good = mbar_wait_bounded(&empty[slot], (uint32_t)(((n / NS) - 1) & 1));
    if (!__shfl_sync(0xffffffffu, good, 0)) return false;
    if (ASYNC || lane == 0) issue(it, k, slot, &full[slot], lane);
    prefetch.plane(k);
  }
  return true;
}

// The block must not exit with copies in flight: waits (bounded) for the
// last NS loads, and reports a timeout seen earlier.
template <int NS, bool ASYNC>
__device__ __forceinline__ void produce_drain(unsigned n, bool ok, uint64_t *full, unsigned *__restrict__ err,
                                              int lane) {
  if (ASYNC) cp_async_wait_all();
  if (lane != 0) return;
  if (!ok) atomicOr(err, DEV_ERR_TIMEOUT);
  for (unsigned q = (n > NS ? n - NS : 0); q < n; ++q)
    mbar_wait_bounded(&full[q % NS], (uint32_t)((q / NS) & 1), 200000000ull);
}

template <int NS, bool ASYNC, typename Issue, typename Prefetch>
__device__ __forceinline__ void produce(const Item *__restrict__ items, int2 range, uint64_t *full, uint64_t *empty,
                                        Issue issue, Prefetch &prefetch, unsigned *__restrict__ err, int ctl,
                                        int lane) {
  if (ctl & CTL_WITHHOLD_LOADS) return;  // test mode: no stage is ever filled
  unsigned n = 0;
  bool ok = true;
  for (int ii = range.x; ii < range.y && ok; ++ii) ok = produce_item<NS, ASYNC>(items[ii], n, full, empty, issue,
                                                                                 prefetch, lane);
  produce_drain<NS, ASYNC>(n, ok, full, err, lane);
}

// The producer lanes' memory-variable prefetcher for one half-step (var0 =
// PSI_S0 for the stress half-step, PSI_V0 for the velocity half-step).
template <typename T, int TX, int TY>
struct ItemPrefetch {
  PsiPrefetch<T, TX, TY> pf;
  const ShotDesc<T> *shots;
  int lane, ctl, var0;
  __device__ __forceinline__ void begin(const Item &it) {
    const ShotDesc<T> &sd = shots[it.shot];
    const int txs = tiles_x_of(sd, TX);
    pf.begin(sd, (it.tile % txs) * TX, (it.tile / txs) * TY, var0, lane, ctl);
  }
  __device__ __forceinline__ void plane(int k) const { pf.plane(k); }
};

// ------------------------------------------------------- stage loads ----
// One stress plane: vx vy vz cs rho with their halos, cp and the six
// stresses of the tile (box shapes in ela3d_device.cuh, ShotMaps).
template <typename T, int TX, int TY, int NS, int CPT, int MB, int LOAD>
__device__ __forceinline__ void stress_issue(const ShotDesc<T> *__restrict__ shots,
                                             const ShotMaps *__restrict__ maps, const Item &it, int k,
                                             unsigned char *st, uint64_t *bar, int lane) {
  using G = Geo<T, TX, TY, NS, CPT, MB>;
  constexpr int H = G::H;
  const int txs = tiles_x_of(shots[it.shot], TX);
  const int x0 = (it.tile % txs) * TX, y0 = (it.tile / txs) * TY;
  if constexpr (LOAD == LOAD_CP_ASYNC) {
    const ShotDesc<T> &sd = shots[it.shot];
    copy_box_async<T, TX + H, TY + 1>(st + G::S_VX, sd.f[0], sd, x0, y0, k, lane);
    copy_box_async<T, TX + H, TY + 1>(st + G::S_VY, sd.f[1], sd, x0 - H, y0 - 1, k, lane);
    copy_box_async<T, TX + H, TY + 1>(st + G::S_VZ, sd.f[2], sd, x0 - H, y0, k, lane);
    copy_box_async<T, TX + H, TY + 1>(st + G::S_CS, sd.cs, sd, x0 - H, y0, k, lane);
    copy_box_async<T, TX + H, TY + 1>(st + G::S_RHO, sd.rho, sd, x0 - H, y0, k, lane);
    copy_box_async<T, TX, TY>(st + G::S_CP, sd.cp, sd, x0, y0, k, lane);
#pragma unroll
    for (int c = 0; c < 6; ++c) copy_box_async<T, TX, TY>(st + G::S_SIG + c * G::SC, sd.f[3 + c], sd, x0, y0, k, lane);
    cp_async_arrive_noinc(bar);
    return;
  }
  const CUtensorMap *m = maps[it.shot].stress;
  mbar_arrive_expect_tx(bar, G::S_TX);
  tma_load_3d(st + G::S_VX, &m[0], x0, y0, k, bar);
  tma_load_3d(st + G::S_VY, &m[1], x0 - H, y0 - 1, k, bar);
  tma_load_3d(st + G::S_VZ, &m[2], x0 - H, y0, k, bar);
  tma_load_3d(st + G::S_CS, &m[3], x0 - H, y0, k, bar);
  tma_load_3d(st + G::S_RHO, &m[4], x0 - H, y0, k, bar);
  tma_load_3d(st + G::S_CP, &m[5], x0, y0, k, bar);
#pragma unroll
  for (int c = 0; c < 6; ++c) tma_load_3d(st + G::S_SIG + c * G::SC, &m[6 + c], x0, y0, k, bar);
}

// One velocity plane: the six stresses with the halos the divergence needs,
// rho with its halo, and vx vy vz of the tile.
template <typename T, int TX, int TY, int NS, int CPT, int MB, int LOAD>
__device__ __forceinline__ void velocity_issue(const ShotDesc<T> *__restrict__ shots,
                                               const ShotMaps *__restrict__ maps, const Item &it, int k,
                                               unsigned char *st, uint64_t *bar, int lane) {
  using G = Geo<T, TX, TY, NS, CPT, MB>;
  constexpr int H = G::H;
  const int txs = tiles_x_of(shots[it.shot], TX);
  const int x0 = (it.tile % txs) * TX, y0 = (it.tile / txs) * TY;
  if constexpr (LOAD == LOAD_CP_ASYNC) {
    const ShotDesc<T> &sd = shots[it.shot];
    copy_box_async<T, TX + H, TY>(st + G::V_SXX, sd.f[3], sd, x0 - H, y0, k, lane);
    copy_box_async<T, TX, TY + 1>(st + G::V_SYY, sd.f[4], sd, x0, y0, k, lane);
    copy_box_async<T, TX, TY>(st + G::V_SZZ, sd.f[5], sd, x0, y0, k, lane);
    copy_box_async<T, TX + H, TY + 1>(st + G::V_SXY, sd.f[6], sd, x0, y0 - 1, k, lane);
    copy_box_async<T, TX + H, TY>(st + G::V_SXZ, sd.f[7], sd, x0, y0, k, lane);
    copy_box_async<T, TX, TY + 1>(st + G::V_SYZ, sd.f[8], sd, x0, y0 - 1, k, lane);
    copy_box_async<T, TX + H, TY + 1>(st + G::V_RHO, sd.rho, sd, x0 - H, y0, k, lane);
#pragma unroll
    for (int c = 0; c < 3; ++c) copy_box_async<T, TX, TY>(st + G::V_V + c * G::SC, sd.f[c], sd, x0, y0, k, lane);
    cp_async_arrive_noinc(bar);
    return;
  }
  const CUtensorMap *m = maps[it.shot].vel;
  mbar_arrive_expect_tx(bar, G::V_TX);
  tma_load_3d(st + G::V_SXX, &m[0], x0 - H, y0, k, bar);
  tma_load_3d(st + G::V_SYY, &m[1], x0, y0, k, bar);
  tma_load_3d(st + G::V_SZZ, &m[2], x0, y0, k, bar);
  tma_load_3d(st + G::V_SXY, &m[3], x0, y0 - 1, k, bar);
  tma_load_3d(st + G::V_SXZ, &m[4], x0, y0, k, bar);
  tma_load_3d(st + G::V_SYZ, &m[5], x0, y0 - 1, k, bar);
  tma_load_3d(st + G::V_RHO, &m[6], x0 - H, y0, k, bar);
#pragma unroll
  for (int c = 0; c < 3; ++c) tma_load_3d(st + G::V_V + c * G::SC, &m[7 + c], x0, y0, k, bar);
}

// Waits for the stages of loads n and n+1 (planes k and k+1); load n was
// already waited for as the previous plane's k+1 unless k is the first plane
// of its work item.  False when a wait passed its limit; the caller records
// the timeout and returns.
template <int NS>
__device__ __forceinline__ bool wait_planes(uint64_t *full, unsigned n, bool first, unsigned long long wait_ns,
                                            unsigned *err, int lane) {
  const int s0 = (int)(n % NS), s1 = (int)((n + 1) % NS);
  bool ok = !first || mbar_wait_bounded(&full[s0], (uint32_t)((n / NS) & 1), wait_ns);
  ok = ok && mbar_wait_bounded(&full[s1], (uint32_t)(((n + 1) / NS) & 1), wait_ns);
  if (__any_sync(0xffffffffu, !ok)) {
    if (lane == 0) atomicOr(err, DEV_ERR_TIMEOUT);
    return false;
  }
  return true;
}

// Load that bypasses L1, for values another block wrote during this launch
// (the dataflow kernel's z-1 planes at the start of an item).
template <typename T, int N>
__device__ __forceinline__ void ld_vec_l2(const T *p, T (&o)[N]) {
  unpack<T, N>(__ldcg(reinterpret_cast<const typename VType<T, N>::V *>(p)), o);
}

// Consumers of the dataflow kernel: waits (bounded) until the producer has
// acquired the item's dependencies and arrived on its ready barrier.
__device__ __forceinline__ bool flow_ready(uint64_t *ready, uint32_t parity, unsigned long long wait_ns,
                                           unsigned *err, int lane) {
  const bool ok = mbar_wait_bounded(ready, parity, wait_ns);
  if (__any_sync(0xffffffffu, !ok)) {
    if (lane == 0) atomicOr(err, DEV_ERR_TIMEOUT);
    return false;
  }
  return true;
}

// ----------------------------------------------------------- stress ----
// The stress half-step over one work item (the block's consumer warps).
// STAGE is the byte stride of the ring's stages.  FLOW (the dataflow
// kernel): the item's inputs were written by other blocks of the same
// launch; nothing global is read before the producer has acquired the
// item's dependencies and arrived on `ready` (phase parity ready_parity),
// and the z-1 plane, written during this launch, bypasses L1.
template <typename T, int TX, int TY, int NS, int CPT, int MB, int STAGE, bool FLOW>
__device__ __forceinline__ bool stress_item(const ShotDesc<T> &sd, const Item &item, const unsigned char *smem,
                                            uint64_t *full, uint64_t *empty, unsigned &n, unsigned *__restrict__ err,
                                            unsigned long long wait_ns, int tid, uint64_t *ready = nullptr,
                                            uint32_t ready_parity = 0) {
  using G = Geo<T, TX, TY, NS, CPT, MB>;
  constexpr int V = G::VEC, H = G::H, WW = G::WW;
  const int lane = tid & 31;
  const int tx = tid % G::NTX, ty = tid / G::NTX;
  const int nx = sd.nx, ny = sd.ny, nz = sd.nz, px = sd.px;
  const int txs = (nx + TX - 1) / TX;
  const int x0 = (item.tile % txs) * TX, y0 = (item.tile / txs) * TY;
  const int xg = x0 + tx * V, y = y0 + ty;
  const bool live = (xg < nx) && (y < ny);
  const T dt = sd.dt, idx = sd.idx, idy = sd.idy, idz = sd.idz;
  const long long plane = (long long)ny * px;
  const long long rowoff = (long long)y * px + xg;
  T *const f3 = sd.f[3], *const f4 = sd.f[4], *const f5 = sd.f[5];
  T *const f6 = sd.f[6], *const f7 = sd.f[7], *const f8 = sd.f[8];
  const int zl = sd.zl, zr = sd.zr;
  const T *const prof_z = sd.prof_z;
  T *const psi_x = sd.psi_x, *const psi_y = sd.psi_y, *const psi_z = sd.psi_z;
  const long long psx = sd.psx, psy = sd.psy, psz = sd.psz;
  const int xw = sd.xw, yw = sd.yw;

  // FLOW: the producer has acquired the item's dependencies
  if (FLOW && !flow_ready(ready, ready_parity, wait_ns, err, lane)) return false;

  // z-1 neighbour of vz for the first plane of the run
  T vz_zm[V];
#pragma unroll
  for (int e = 0; e < V; ++e) vz_zm[e] = T(0);
  if (live && item.k0 > 0) {
    if constexpr (FLOW) ld_vec_l2(sd.f[2] + (long long)(item.k0 - 1) * plane + rowoff, vz_zm);
    else ld_vec_rw(sd.f[2] + (long long)(item.k0 - 1) * plane + rowoff, vz_zm);
  }

  // x-slab profile and placement (fixed over the run)
  const bool in_x = live && (xg < sd.xl || xg >= sd.xr);
  const int xs = xg < sd.xl ? xg : sd.xl + (xg - sd.xr);
  T ax[V], bx[V], ikx[V], axh[V], bxh[V], ikxh[V];
  if (in_x) {
    ld_vec_global(sd.prof_x + PR_A * px + xg, ax);
    ld_vec_global(sd.prof_x + PR_B * px + xg, bx);
    ld_vec_global(sd.prof_x + PR_IK * px + xg, ikx);
    ld_vec_global(sd.prof_x + PR_AH * px + xg, axh);
    ld_vec_global(sd.prof_x + PR_BH * px + xg, bxh);
    ld_vec_global(sd.prof_x + PR_IKH * px + xg, ikxh);
  } else {
#pragma unroll
    for (int e = 0; e < V; ++e) { ax[e] = axh[e] = T(0); bx[e] = bxh[e] = ikx[e] = ikxh[e] = T(1); }
  }
  const bool row_y = y < sd.yl || y >= sd.yr;   // the row lies in the y slab
  const bool in_y = live && row_y;
  const int ys = y < sd.yl ? y : sd.yl + (y - sd.yr);
  T ay = 0, by = 1, iky = 1, ayh = 0, byh = 1, ikyh = 1;
  if (in_y) {
    ay = sd.prof_y[PR_A * ny + y]; by = sd.prof_y[PR_B * ny + y]; iky = sd.prof_y[PR_IK * ny + y];
    ayh = sd.prof_y[PR_AH * ny + y]; byh = sd.prof_y[PR_BH * ny + y]; ikyh = sd.prof_y[PR_IKH * ny + y];
  }
  const int sb = (ty * WW + tx * V);       // vx box (origin x0, y0)
  const int sl = (ty * WW + H + tx * V);   // vz/cs/rho boxes (origin x0-H, y0)
  const int syl = sl + WW;                 // vy box (origin x0-H, y0-1): own row is ty+1
  const int sc = ty * TX + tx * V;         // centre boxes

  // the update ranges (simpelmodel.cpp:378-498) as per-cell bits, set once
  // per work item; the normal stresses also need k >= 1 (applied per plane)
  unsigned mbits = 0;
#pragma unroll
  for (int e = 0; e < V; ++e) {
    const int x = xg + e;
    mbits |= ((y >= 1) && (x <= nx - 2) ? 1u : 0u) << e;                   // normal: j >= 2, i <= NX-1
    mbits |= ((y <= ny - 2) && (x >= 1) && (x <= nx - 1) ? 1u : 0u) << (8 + e);   // sigma_xy
    mbits |= ((x >= 1) && (x <= nx - 1) ? 1u : 0u) << (16 + e);            // sigma_xz
    mbits |= ((y <= ny - 2) && (x <= nx - 1) ? 1u : 0u) << (24 + e);       // sigma_yz
  }
  T *gx = psi_x + ((long long)item.k0 * ny + y) * xw + xs;
  T *gy = psi_y + ((long long)item.k0 * yw + ys) * px + xg;
  const long long dgx = (long long)ny * xw, dgy = (long long)yw * px;
  long long g = (long long)item.k0 * plane + rowoff;
  for (int k = item.k0; k < item.k1; ++k, gx += dgx, gy += dgy, g += plane) {
    // memory variables and z profile first: their latency overlaps the wait
    const bool plane_z = k < zl || k >= zr;       // the plane lies in the z slab
    const bool in_z = live && plane_z;
    const int zs = k < zl ? k : zl + (k - zr);
    T az = 0, bz = 1, ikz = 1, azh = 0, bzh = 1, ikzh = 1;
    if (in_z) {
      az = prof_z[PR_A * nz + k]; bz = prof_z[PR_B * nz + k]; ikz = prof_z[PR_IK * nz + k];
      azh = prof_z[PR_AH * nz + k]; bzh = prof_z[PR_BH * nz + k]; ikzh = prof_z[PR_IKH * nz + k];
    }
    T px0[V], px1[V], px2[V], py0[V], py1[V], py2[V], pz0[V], pz1[V], pz2[V];
    T *gz = psi_z + ((long long)zs * ny + y) * px + xg;
    if (in_x) {
      ld_vec_rw(gx + PSI_S0 * psx, px0);
      ld_vec_rw(gx + PSI_S1 * psx, px1);
      ld_vec_rw(gx + PSI_S2 * psx, px2);
    } else {
#pragma unroll
      for (int e = 0; e < V; ++e) px0[e] = px1[e] = px2[e] = T(0);
    }
    if (in_y) {
      ld_vec_rw(gy + PSI_S0 * psy, py0);
      ld_vec_rw(gy + PSI_S1 * psy, py1);
      ld_vec_rw(gy + PSI_S2 * psy, py2);
    } else {
#pragma unroll
      for (int e = 0; e < V; ++e) py0[e] = py1[e] = py2[e] = T(0);
    }
    if (in_z) {
      ld_vec_rw(gz + PSI_S0 * psz, pz0);
      ld_vec_rw(gz + PSI_S1 * psz, pz1);
      ld_vec_rw(gz + PSI_S2 * psz, pz2);
    } else {
#pragma unroll
      for (int e = 0; e < V; ++e) pz0[e] = pz1[e] = pz2[e] = T(0);
    }

    if (!wait_planes<NS>(full, n, k == item.k0, wait_ns, err, lane)) return false;
    const int s0 = (int)(n % NS), s1 = (int)((n + 1) % NS);
    const unsigned char *cur = smem + s0 * STAGE;
    const unsigned char *nxt = smem + s1 * STAGE;
    const T *bvx = reinterpret_cast<const T *>(cur + G::S_VX);
    const T *bvy = reinterpret_cast<const T *>(cur + G::S_VY);
    const T *bvz = reinterpret_cast<const T *>(cur + G::S_VZ);
    const T *bcs = reinterpret_cast<const T *>(cur + G::S_CS);
    const T *brho = reinterpret_cast<const T *>(cur + G::S_RHO);
    const T *bcp = reinterpret_cast<const T *>(cur + G::S_CP);
    const T *bsig = reinterpret_cast<const T *>(cur + G::S_SIG);
    constexpr int CS = G::SC / (int)sizeof(T);

    T vx_c[V], vx_yp[V], vx_zp[V], vy_c[V], vy_ym[V], vy_zp[V], vz_c[V], vz_yp[V];
    T cs_c[V], cs_yp[V], cs_zp[V], rho_c[V], rho_yp[V], rho_zp[V], cp_c[V];
    ld_vec(bvx + sb, vx_c);
    ld_vec(bvx + sb + WW, vx_yp);
    const T vx_e = bvx[sb + V];
    ld_vec(reinterpret_cast<const T *>(nxt + G::S_VX) + sb, vx_zp);
    ld_vec(bvy + syl, vy_c);
    ld_vec(bvy + syl - WW, vy_ym);
    const T vy_w = bvy[syl - 1];
    ld_vec(reinterpret_cast<const T *>(nxt + G::S_VY) + syl, vy_zp);
    ld_vec(bvz + sl, vz_c);
    ld_vec(bvz + sl + WW, vz_yp);
    const T vz_w = bvz[sl - 1];
    ld_vec(bcs + sl, cs_c);
    ld_vec(bcs + sl + WW, cs_yp);
    const T cs_w = bcs[sl - 1];
    ld_vec(reinterpret_cast<const T *>(nxt + G::S_CS) + sl, cs_zp);
    ld_vec(brho + sl, rho_c);
    ld_vec(brho + sl + WW, rho_yp);
    const T rho_w = brho[sl - 1];
    ld_vec(reinterpret_cast<const T *>(nxt + G::S_RHO) + sl, rho_zp);
    ld_vec(bcp + sc, cp_c);
    T sxx[V], syy[V], szz[V], sxy[V], sxz[V], syz[V];
    ld_vec(bsig + 0 * CS + sc, sxx);
    ld_vec(bsig + 1 * CS + sc, syy);
    ld_vec(bsig + 2 * CS + sc, szz);
    ld_vec(bsig + 3 * CS + sc, sxy);
    ld_vec(bsig + 4 * CS + sc, sxz);
    ld_vec(bsig + 5 * CS + sc, syz);

    // stage s0 is no longer read by this warp (s1 still is, as the next plane)
    const bool last = (k == item.k1 - 1);
    __syncwarp();
    if (lane == 0) {
      mbar_arrive(&empty[s0]);
      if (last) mbar_arrive(&empty[s1]);
    }

    // this plane's update masks: bit e of byte c = component c of cell e
    const unsigned mk = k >= 1 ? mbits : (mbits & 0xffffff00u);
    // The y- and z-direction C-PML terms are evaluated only for rows /
    // planes inside the slabs (elsewhere a = 0 and 1/K = 1 and the terms
    // are exact no-ops).  Memory variables are updated whether or not the
    // cell's stress is: a cell outside the update ranges never uses them.
    auto compute = [&](auto PY, auto PZ) {
      constexpr bool pyo = decltype(PY)::value, pzo = decltype(PZ)::value;
#pragma unroll
      for (int e = 0; e < V; ++e) {
        const int x = xg + e;
        const T vx_xp = (e < V - 1) ? vx_c[e + 1] : vx_e;
        const T vy_xm = (e > 0) ? vy_c[e - 1] : vy_w;
        const T vz_xm = (e > 0) ? vz_c[e - 1] : vz_w;
        const T cs_xm = (e > 0) ? cs_c[e - 1] : cs_w;
        const T rho_xm = (e > 0) ? rho_c[e - 1] : rho_w;

        // normal stresses, simpelmodel.cpp:378-413
        {
          const bool m = (mk >> (0 + e)) & 1u;
          const T vp = cp_c[e], vs = cs_c[e], rhos = rho_c[e];
          const T lambda = rhos * (vp * vp - T(2) * vs * vs);
          const T l2m = rhos * vp * vp;
          const T DT_l2m = dt * l2m, DT_l = dt * lambda;
          T dvx_dx = (vx_xp - vx_c[e]) * idx;
          T dvy_dy = (vy_c[e] - vy_ym[e]) * idy;
          T dvz_dz = (vz_c[e] - vz_zm[e]) * idz;
          const T qx = bxh[e] * px0[e] + axh[e] * dvx_dx;
          dvx_dx = dvx_dx * ikxh[e] + qx;
          px0[e] = qx;
          if constexpr (pyo) {
            const T qy = by * py0[e] + ay * dvy_dy;
            dvy_dy = dvy_dy * iky + qy;
            py0[e] = qy;
          }
          if constexpr (pzo) {
            const T qz = bz * pz0[e] + az * dvz_dz;
            dvz_dz = dvz_dz * ikz + qz;
            pz0[e] = qz;
          }
          if (m) {
            sxx[e] = DT_l2m * dvx_dx + DT_l * (dvy_dy + dvz_dz) + sxx[e];
            syy[e] = DT_l * (dvx_dx + dvz_dz) + DT_l2m * dvy_dy + syy[e];
            szz[e] = DT_l * (dvx_dx + dvy_dy) + DT_l2m * dvz_dz + szz[e];
          }
        }
        // sigma_xy, :416-442
        {
          const bool m = (mk >> (8 + e)) & 1u;
          const T vs = (cs_xm + cs_yp[e]) / T(2);
          const T rhos = (rho_xm + rho_yp[e]) / T(2);
          const T DT_mu = dt * (rhos * vs * vs);
          T dvy_dx = (vy_c[e] - vy_xm) * idx;
          T dvx_dy = (vx_yp[e] - vx_c[e]) * idy;
          const T qx = bx[e] * px1[e] + ax[e] * dvy_dx;
          dvy_dx = dvy_dx * ikx[e] + qx;
          px1[e] = qx;
          if constexpr (pyo) {
            const T qy = byh * py1[e] + ayh * dvx_dy;
            dvx_dy = dvx_dy * ikyh + qy;
            py1[e] = qy;
          }
          if (m) sxy[e] = DT_mu * (dvy_dx + dvx_dy) + sxy[e];
        }
        // sigma_xz, :445-471 (z+1 of plane nz-1 is the zero plane)
        {
          const bool m = (mk >> (16 + e)) & 1u;
          const T vs = (cs_xm + cs_zp[e]) / T(2);
          const T rhos = (rho_xm + rho_zp[e]) / T(2);
          const T DT_mu = dt * (rhos * vs * vs);
          T dvz_dx = (vz_c[e] - vz_xm) * idx;
          T dvx_dz = (vx_zp[e] - vx_c[e]) * idz;
          const T qx = bx[e] * px2[e] + ax[e] * dvz_dx;
          dvz_dx = dvz_dx * ikx[e] + qx;
          px2[e] = qx;
          if constexpr (pzo) {
            const T qz = bzh * pz1[e] + azh * dvx_dz;
            dvx_dz = dvx_dz * ikzh + qz;
            pz1[e] = qz;
          }
          if (m) sxz[e] = DT_mu * (dvz_dx + dvx_dz) + sxz[e];
        }
        // sigma_yz, :473-498
        {
          const bool m = (mk >> (24 + e)) & 1u;
          const T vs = (cs_yp[e] + cs_zp[e]) / T(2);
          const T rhos = (rho_yp[e] + rho_zp[e]) / T(2);
          const T DT_mu = dt * (rhos * vs * vs);
          T dvz_dy = (vz_yp[e] - vz_c[e]) * idy;
          T dvy_dz = (vy_zp[e] - vy_c[e]) * idz;
          if constexpr (pyo) {
            const T qy = byh * py2[e] + ayh * dvz_dy;
            dvz_dy = dvz_dy * ikyh + qy;
            py2[e] = qy;
          }
          if constexpr (pzo) {
            const T qz = bzh * pz2[e] + azh * dvy_dz;
            dvy_dz = dvy_dz * ikzh + qz;
            pz2[e] = qz;
          }
          if (m) syz[e] = DT_mu * (dvz_dy + dvy_dz) + syz[e];
        }
        vz_zm[e] = vz_c[e];
      }
    };
    if (row_y) {
      if (plane_z) compute(std::true_type{}, std::true_type{});
      else compute(std::true_type{}, std::false_type{});
    } else {
      if (plane_z) compute(std::false_type{}, std::true_type{});
      else compute(std::false_type{}, std::false_type{});
    }

    if (live) {
      st_vec(f3 + g, sxx);
      st_vec(f4 + g, syy);
      st_vec(f5 + g, szz);
      st_vec(f6 + g, sxy);
      st_vec(f7 + g, sxz);
      st_vec(f8 + g, syz);
      if (in_x) {
        st_vec(gx + PSI_S0 * psx, px0);
        st_vec(gx + PSI_S1 * psx, px1);
        st_vec(gx + PSI_S2 * psx, px2);
      }
      if (in_y) {
        st_vec(gy + PSI_S0 * psy, py0);
        st_vec(gy + PSI_S1 * psy, py1);
        st_vec(gy + PSI_S2 * psy, py2);
      }
      if (in_z) {
        st_vec(gz + PSI_S0 * psz, pz0);
        st_vec(gz + PSI_S1 * psz, pz1);
        st_vec(gz + PSI_S2 * psz, pz2);
      }
    }
    n += last ? 2 : 1;
  }
  return true;
}

// --------------------------------------------------------- velocity ----
// The velocity half-step over one work item at step `tick` (see
// stress_item for STAGE and FLOW), with the receivers and the force source.
template <typename T, int TX, int TY, int NS, int CPT, int MB, int STAGE, bool FLOW>
__device__ __forceinline__ bool velocity_item(const ShotDesc<T> &sd, const Item &item, int tick,
                                              const unsigned char *smem, uint64_t *full, uint64_t *empty,
                                              unsigned &n, unsigned *__restrict__ err, unsigned long long wait_ns,
                                              int tid, uint64_t *ready = nullptr, uint32_t ready_parity = 0) {
  using G = Geo<T, TX, TY, NS, CPT, MB>;
  constexpr int V = G::VEC, H = G::H, WW = G::WW;
  constexpr int CS = G::SC / (int)sizeof(T);
  const int lane = tid & 31;
  const int tx = tid % G::NTX, ty = tid / G::NTX;
  const int nx = sd.nx, ny = sd.ny, nz = sd.nz, px = sd.px;
  const int txs = (nx + TX - 1) / TX;
  const int x0 = (item.tile % txs) * TX, y0 = (item.tile / txs) * TY;
  const int xg = x0 + tx * V, y = y0 + ty;
  const bool live = (xg < nx) && (y < ny);
  const T dt = sd.dt, idx = sd.idx, idy = sd.idy, idz = sd.idz;
  const long long plane = (long long)ny * px;
  const long long rowoff = (long long)y * px + xg;
  T *const f0 = sd.f[0], *const f1 = sd.f[1], *const f2 = sd.f[2];
  const int zl = sd.zl, zr = sd.zr;
  const T *const prof_z = sd.prof_z;
  T *const psi_x = sd.psi_x, *const psi_y = sd.psi_y, *const psi_z = sd.psi_z;
  const long long psx = sd.psx, psy = sd.psy, psz = sd.psz;
  const int xw = sd.xw, yw = sd.yw;
  const int it_step = tick - sd.tick0;
  const bool sample = (it_step % sd.sampgat == 0) && (it_step / sd.sampgat <= sd.nsamp) && it_step > 0;
  const int samp = it_step / sd.sampgat - 1;
  const int *const rec_plane = sd.rec_plane;
  // receivers exist in this item's planes at all (most items have none)
  const bool item_rec = sample && rec_plane[item.k1] > rec_plane[item.k0];
  const bool src_row = sd.src_kind == 0 && y == sd.src_j && sd.src_i >= xg && sd.src_i < xg + V &&
                       it_step >= 1 && it_step <= sd.nstep;

  if (FLOW && !flow_ready(ready, ready_parity, wait_ns, err, lane)) return false;

  T sxz_zm[V], syz_zm[V];
#pragma unroll
  for (int e = 0; e < V; ++e) sxz_zm[e] = syz_zm[e] = T(0);
  if (live && item.k0 > 0) {
    const long long g = (long long)(item.k0 - 1) * plane + rowoff;
    if constexpr (FLOW) {
      ld_vec_l2(sd.f[7] + g, sxz_zm);
      ld_vec_l2(sd.f[8] + g, syz_zm);
    } else {
      ld_vec_rw(sd.f[7] + g, sxz_zm);
      ld_vec_rw(sd.f[8] + g, syz_zm);
    }
  }

  const bool in_x = live && (xg < sd.xl || xg >= sd.xr);
  const int xs = xg < sd.xl ? xg : sd.xl + (xg - sd.xr);
  T ax[V], bx[V], ikx[V], axh[V], bxh[V], ikxh[V];
  if (in_x) {
    ld_vec_global(sd.prof_x + PR_A * px + xg, ax);
    ld_vec_global(sd.prof_x + PR_B * px + xg, bx);
    ld_vec_global(sd.prof_x + PR_IK * px + xg, ikx);
    ld_vec_global(sd.prof_x + PR_AH * px + xg, axh);
    ld_vec_global(sd.prof_x + PR_BH * px + xg, bxh);
    ld_vec_global(sd.prof_x + PR_IKH * px + xg, ikxh);
  } else {
#pragma unroll
    for (int e = 0; e < V; ++e) { ax[e] = axh[e] = T(0); bx[e] = bxh[e] = ikx[e] = ikxh[e] = T(1); }
  }
  const bool row_y = y < sd.yl || y >= sd.yr;   // the row lies in the y slab
  const bool in_y = live && row_y;
  const int ys = y < sd.yl ? y : sd.yl + (y - sd.yr);
  T ay = 0, by = 1, iky = 1, ayh = 0, byh = 1, ikyh = 1;
  if (in_y) {
    ay = sd.prof_y[PR_A * ny + y]; by = sd.prof_y[PR_B * ny + y]; iky = sd.prof_y[PR_IK * ny + y];
    ayh = sd.prof_y[PR_AH * ny + y]; byh = sd.prof_y[PR_BH * ny + y]; ikyh = sd.prof_y[PR_IKH * ny + y];
  }
  const int sl0 = ty * WW + H + tx * V;     // sxx box (origin x0-H, y0)
  const int sr0 = ty * WW + tx * V;         // sxz box (origin x0, y0)
  const int sr1 = (ty + 1) * WW + tx * V;   // sxy box (origin x0, y0-1): own row ty+1
  const int sc = ty * TX + tx * V;          // syy box (origin x0, y0) / centre boxes
  const int sc1 = (ty + 1) * TX + tx * V;   // syz box (origin x0, y0-1)

  // the update ranges (simpelmodel.cpp:502-590) as per-cell bits, set once
  // per work item; the plane conditions are applied per plane
  unsigned mbits = 0;
#pragma unroll
  for (int e = 0; e < V; ++e) {
    const int x = xg + e;
    mbits |= ((y >= 1) && (x >= 1) && (x <= nx - 1) ? 1u : 0u) << e;        // vx (with k >= 1)
    mbits |= ((y <= ny - 2) && (x <= nx - 2) ? 1u : 0u) << (8 + e);         // vy (with k >= 1)
    mbits |= ((y >= 1) && (x <= nx - 2) ? 1u : 0u) << (16 + e);             // vz (with k <= nz-2)
  }
  T *gx = psi_x + ((long long)item.k0 * ny + y) * xw + xs;
  T *gy = psi_y + ((long long)item.k0 * yw + ys) * px + xg;
  const long long dgx = (long long)ny * xw, dgy = (long long)yw * px;
  long long g = (long long)item.k0 * plane + rowoff;
  for (int k = item.k0; k < item.k1; ++k, gx += dgx, gy += dgy, g += plane) {
    const bool plane_z = k < zl || k >= zr;       // the plane lies in the z slab
    const bool in_z = live && plane_z;
    const int zs = k < zl ? k : zl + (k - zr);
    T az = 0, bz = 1, ikz = 1, azh = 0, bzh = 1, ikzh = 1;
    if (in_z) {
      az = prof_z[PR_A * nz + k]; bz = prof_z[PR_B * nz + k]; ikz = prof_z[PR_IK * nz + k];
      azh = prof_z[PR_AH * nz + k]; bzh = prof_z[PR_BH * nz + k]; ikzh = prof_z[PR_IKH * nz + k];
    }
    T px0[V], px1[V], px2[V], py0[V], py1[V], py2[V], pz0[V], pz1[V], pz2[V];
    T *gz = psi_z + ((long long)zs * ny + y) * px + xg;
    if (in_x) {
      ld_vec_rw(gx + PSI_V0 * psx, px0);
      ld_vec_rw(gx + PSI_V1 * psx, px1);
      ld_vec_rw(gx + PSI_V2 * psx, px2);
    } else {
#pragma unroll
      for (int e = 0; e < V; ++e) px0[e] = px1[e] = px2[e] = T(0);
    }
    if (in_y) {
      ld_vec_rw(gy + PSI_V0 * psy, py0);
      ld_vec_rw(gy + PSI_V1 * psy, py1);
      ld_vec_rw(gy + PSI_V2 * psy, py2);
    } else {
#pragma unroll
      for (int e = 0; e < V; ++e) py0[e] = py1[e] = py2[e] = T(0);
    }
    if (in_z) {
      ld_vec_rw(gz + PSI_V0 * psz, pz0);
      ld_vec_rw(gz + PSI_V1 * psz, pz1);
      ld_vec_rw(gz + PSI_V2 * psz, pz2);
    } else {
#pragma unroll
      for (int e = 0; e < V; ++e) pz0[e] = pz1[e] = pz2[e] = T(0);
    }

    int rlo = 0, rhi = 0;   // receivers of this plane
    if (item_rec) {
      rlo = rec_plane[k];
      rhi = rec_plane[k + 1];
    }

    if (!wait_planes<NS>(full, n, k == item.k0, wait_ns, err, lane)) return false;
    const int s0 = (int)(n % NS), s1 = (int)((n + 1) % NS);
    const unsigned char *cur = smem + s0 * STAGE;
    const unsigned char *nxt = smem + s1 * STAGE;
    const T *bsxx = reinterpret_cast<const T *>(cur + G::V_SXX);
    const T *bsyy = reinterpret_cast<const T *>(cur + G::V_SYY);
    const T *bszz = reinterpret_cast<const T *>(cur + G::V_SZZ);
    const T *bsxy = reinterpret_cast<const T *>(cur + G::V_SXY);
    const T *bsxz = reinterpret_cast<const T *>(cur + G::V_SXZ);
    const T *bsyz = reinterpret_cast<const T *>(cur + G::V_SYZ);
    const T *brho = reinterpret_cast<const T *>(cur + G::V_RHO);
    const T *bv = reinterpret_cast<const T *>(cur + G::V_V);

    T sxx_c[V], syy_c[V], syy_yp[V], szz_c[V], szz_zp[V], sxy_c[V], sxy_ym[V], sxz_c[V];
    T syz_c[V], syz_ym[V], rho_c[V], rho_yp[V], rho_zp[V], vx[V], vy[V], vz[V];
    ld_vec(bsxx + sl0, sxx_c);
    const T sxx_w = bsxx[sl0 - 1];
    ld_vec(bsyy + sc, syy_c);
    ld_vec(bsyy + sc + TX, syy_yp);
    ld_vec(bszz + sc, szz_c);
    ld_vec(reinterpret_cast<const T *>(nxt + G::V_SZZ) + sc, szz_zp);
    ld_vec(bsxy + sr1, sxy_c);
    ld_vec(bsxy + sr1 - WW, sxy_ym);
    const T sxy_e = bsxy[sr1 + V];
    ld_vec(bsxz + sr0, sxz_c);
    const T sxz_e = bsxz[sr0 + V];
    ld_vec(bsyz + sc1, syz_c);
    ld_vec(bsyz + sc1 - TX, syz_ym);
    ld_vec(brho + sl0, rho_c);
    ld_vec(brho + sl0 + WW, rho_yp);
    const T rho_w = brho[sl0 - 1];
    ld_vec(reinterpret_cast<const T *>(nxt + G::V_RHO) + sl0, rho_zp);
    ld_vec(bv + 0 * CS + sc, vx);
    ld_vec(bv + 1 * CS + sc, vy);
    ld_vec(bv + 2 * CS + sc, vz);

    const bool last = (k == item.k1 - 1);
    __syncwarp();
    if (lane == 0) {
      mbar_arrive(&empty[s0]);
      if (last) mbar_arrive(&empty[s1]);
    }

    // this plane's update masks: bit e of byte c = component c of cell e
    const unsigned mk = (k >= 1 ? (mbits & 0x00ffffu) : 0u) | (k <= nz - 2 ? (mbits & 0xff0000u) : 0u);
    // y/z C-PML terms only inside the slabs; memory variables updated
    // whether or not the cell's velocity is (as in the stress half-step)
    auto compute = [&](auto PY, auto PZ) {
      constexpr bool pyo = decltype(PY)::value, pzo = decltype(PZ)::value;
#pragma unroll
      for (int e = 0; e < V; ++e) {
        const int x = xg + e;
        const T sxx_xm = (e > 0) ? sxx_c[e - 1] : sxx_w;
        const T rho_xm = (e > 0) ? rho_c[e - 1] : rho_w;
        const T sxy_xp = (e < V - 1) ? sxy_c[e + 1] : sxy_e;
        const T sxz_xp = (e < V - 1) ? sxz_c[e + 1] : sxz_e;
        // vx, simpelmodel.cpp:502-530
        {
          const bool m = (mk >> (0 + e)) & 1u;
          const T rhos = (rho_c[e] + rho_xm) / T(2);
          const T DT_over_rho = div_fast(dt, rhos);
          T d1 = (sxx_c[e] - sxx_xm) * idx;
          T d2 = (sxy_c[e] - sxy_ym[e]) * idy;
          T d3 = (sxz_c[e] - sxz_zm[e]) * idz;
          const T qx = bx[e] * px0[e] + ax[e] * d1;
          d1 = d1 * ikx[e] + qx;
          px0[e] = qx;
          if constexpr (pyo) {
            const T qy = by * py0[e] + ay * d2;
            d2 = d2 * iky + qy;
            py0[e] = qy;
          }
          if constexpr (pzo) {
            const T qz = bz * pz0[e] + az * d3;
            d3 = d3 * ikz + qz;
            pz0[e] = qz;
          }
          if (m) vx[e] = DT_over_rho * (d1 + d2 + d3) + vx[e];
        }
        // vy, :532-559
        {
          const bool m = (mk >> (8 + e)) & 1u;
          const T rhos = (rho_c[e] + rho_yp[e]) / T(2);
          const T DT_over_rho = div_fast(dt, rhos);
          T d1 = (sxy_xp - sxy_c[e]) * idx;
          T d2 = (syy_yp[e] - syy_c[e]) * idy;
          T d3 = (syz_c[e] - syz_zm[e]) * idz;
          const T qx = bxh[e] * px1[e] + axh[e] * d1;
          d1 = d1 * ikxh[e] + qx;
          px1[e] = qx;
          if constexpr (pyo) {
            const T qy = byh * py1[e] + ayh * d2;
            d2 = d2 * ikyh + qy;
            py1[e] = qy;
          }
          if constexpr (pzo) {
            const T qz = bz * pz1[e] + az * d3;
            d3 = d3 * ikz + qz;
            pz1[e] = qz;
          }
          if (m) vy[e] = DT_over_rho * (d1 + d2 + d3) + vy[e];
        }
        // vz, :563-590
        {
          const bool m = (mk >> (16 + e)) & 1u;
          const T rhos = (rho_c[e] + rho_zp[e]) / T(2);
          const T DT_over_rho = div_fast(dt, rhos);
          T d1 = (sxz_xp - sxz_c[e]) * idx;
          T d2 = (syz_c[e] - syz_ym[e]) * idy;
          T d3 = (szz_zp[e] - szz_c[e]) * idz;
          const T qx = bxh[e] * px2[e] + axh[e] * d1;
          d1 = d1 * ikxh[e] + qx;
          px2[e] = qx;
          if constexpr (pyo) {
            const T qy = by * py2[e] + ay * d2;
            d2 = d2 * iky + qy;
            py2[e] = qy;
          }
          if constexpr (pzo) {
            const T qz = bzh * pz2[e] + azh * d3;
            d3 = d3 * ikzh + qz;
            pz2[e] = qz;
          }
          if (m) vz[e] = DT_over_rho * (d1 + d2 + d3) + vz[e];
        }
        sxz_zm[e] = sxz_c[e];
        syz_zm[e] = syz_c[e];
      }
    };
    if (row_y) {
      if (plane_z) compute(std::true_type{}, std::true_type{});
      else compute(std::true_type{}, std::false_type{});
    } else {
      if (plane_z) compute(std::false_type{}, std::true_type{});
      else compute(std::false_type{}, std::false_type{});
    }

    if (live) {
      // receivers in this row segment (velocity after the update, :593-602)
      if (rlo < rhi) {
        int lo = rlo, hi = rhi;
        {
          const int end = hi;
          while (lo < hi) {   // first receiver with (j, i) >= (y, xg)
            const int mid = (lo + hi) >> 1;
            const int4 r = sd.rec_sorted[mid];
            if (r.y < y || (r.y == y && r.x < xg)) lo = mid + 1; else hi = mid;
          }
          for (int q = lo; q < end; ++q) {
            const int4 r = sd.rec_sorted[q];
            if (r.y != y || r.x >= xg + V) break;
            const int e = r.x - xg;
            T rvx = vx[0], rvy = vy[0], rvz = vz[0];
#pragma unroll
            for (int c = 1; c < V; ++c) {
              rvx = (c == e) ? vx[c] : rvx;
              rvy = (c == e) ? vy[c] : rvy;
              rvz = (c == e) ? vz[c] : rvz;
            }
            T *out = sd.seis + (long long)r.w * 3 * sd.nsamp + samp;
            out[0] = rvx;
            out[sd.nsamp] = rvy;
            out[2 * sd.nsamp] = rvz;
          }
        }
      }
      // force source after the update (cudazerocopy.cu:451-453)
      if (src_row && k == sd.src_k) {
        const T s = sd.stf[it_step - 1];
        const int se = sd.src_i - xg;
        // the averaged densities at the source cell, from the model itself
        // (out-of-grid neighbours are zero, as in the stage boxes)
        const long long gs = (long long)k * plane + rowoff + se;
        const T r0 = sd.rho[gs];
        const T rxs = (r0 + (sd.src_i >= 1 ? sd.rho[gs - 1] : T(0))) / T(2);
        const T rys = (r0 + (y + 1 < ny ? sd.rho[gs + px] : T(0))) / T(2);
        const T rzs = (r0 + (k + 1 < nz ? sd.rho[gs + plane] : T(0))) / T(2);
        const bool wx = sd.src_w[0] != T(0), wy = sd.src_w[1] != T(0), wz = sd.src_w[2] != T(0);
        const T fx = sd.src_w[0] * s, fy = sd.src_w[1] * s, fz = sd.src_w[2] * s;
        T tvx = vx[0], tvy = vy[0], tvz = vz[0];
#pragma unroll
        for (int c = 0; c < V; ++c) {
          const bool hit = (c == se);
          vx[c] = (hit && wx) ? vx[c] + fx * dt / rxs : vx[c];
          vy[c] = (hit && wy) ? vy[c] + fy * dt / rys : vy[c];
          vz[c] = (hit && wz) ? vz[c] + fz * dt / rzs : vz[c];
          tvx = hit ? vx[c] : tvx;
          tvy = hit ? vy[c] : tvy;
          tvz = hit ? vz[c] : tvz;
        }
        // source-point trace: the velocity after the injection
        const int ns = sd.nstep + 1;
        sd.src_trace[it_step] = tvx;
        sd.src_trace[ns + it_step] = tvy;
        sd.src_trace[2 * ns + it_step] = tvz;
      }
      st_vec(f0 + g, vx);
      st_vec(f1 + g, vy);
      st_vec(f2 + g, vz);
      if (in_x) {
        st_vec(gx + PSI_V0 * psx, px0);
        st_vec(gx + PSI_V1 * psx, px1);
        st_vec(gx + PSI_V2 * psx, px2);
      }
      if (in_y) {
        st_vec(gy + PSI_V0 * psy, py0);
        st_vec(gy + PSI_V1 * psy, py1);
        st_vec(gy + PSI_V2 * psy, py2);
      }
      if (in_z) {
        st_vec(gz + PSI_V0 * psz, pz0);
        st_vec(gz + PSI_V1 * psz, pz1);
        st_vec(gz + PSI_V2 * psz, pz2);
      }
    }
    n += last ? 2 : 1;
  }
  return true;
}

// ------------------------------------------------- half-step kernels ----
// Barrier set-up shared by the kernels: full[s] expects the producer's one
// arrival plus the stage's bytes (TMA) or one arrival per lane (cp.async);
// empty[s] one arrival per consumer warp.
template <int NS, int NCW, int LOAD>
__device__ __forceinline__ void init_ring(uint64_t *full, uint64_t *empty) {
  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(&full[s], LOAD == LOAD_TMA ? 1 : 32);
      mbar_init(&empty[s], NCW);
    }
    fence_mbar_init();
  }
  __syncthreads();
}

// (tick and dtick are unused by the stress half-step; the parameter list is
// shared with the velocity kernel so both launch from one argument array)
template <typename T, int TX, int TY, int NS, int CPT, int MB, int LOAD>
__global__ void __launch_bounds__(Geo<T, TX, TY, NS, CPT, MB>::THREADS, Geo<T, TX, TY, NS, CPT, MB>::MINB)
    stress_kernel(const ShotDesc<T> *__restrict__ shots, const ShotMaps *__restrict__ maps,
                  const Item *__restrict__ items, const int2 *__restrict__ ranges, int tick,
                  const int *__restrict__ dtick, unsigned *__restrict__ err, int ctl) {
  using G = Geo<T, TX, TY, NS, CPT, MB>;
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + NS * G::S_STAGE);
  uint64_t *empty = full + NS;

  const int tid = threadIdx.x;
  const int2 range = ranges[blockIdx.x];
  if (range.x >= range.y) return;
  init_ring<NS, G::NCW, LOAD>(full, empty);

  if (tid >= G::NT) {  // producer warp
    auto issue = [&](const Item &it, int k, int slot, uint64_t *bar, int lane) {
      stress_issue<T, TX, TY, NS, CPT, MB, LOAD>(shots, maps, it, k, smem + slot * G::S_STAGE, bar, lane);
    };
    ItemPrefetch<T, TX, TY> prefetch{{}, shots, tid - G::NT, ctl, PSI_S0};
    produce<NS, LOAD == LOAD_CP_ASYNC>(items, range, full, empty, issue, prefetch, err, ctl, tid - G::NT);
    return;
  }

  const unsigned long long wait_ns = (ctl & CTL_WITHHOLD_LOADS) ? kTestWaitLimitNs : kWaitLimitNs;
  unsigned n = 0;  // index of the load holding the current plane
  for (int ii = range.x; ii < range.y; ++ii) {
    const Item item = items[ii];
    if (!stress_item<T, TX, TY, NS, CPT, MB, G::S_STAGE, false>(shots[item.shot], item, smem, full, empty, n, err,
                                                                 wait_ns, tid))
      return;
  }
}

template <typename T, int TX, int TY, int NS, int CPT, int MB, int LOAD>
__global__ void __launch_bounds__(Geo<T, TX, TY, NS, CPT, MB>::THREADS, Geo<T, TX, TY, NS, CPT, MB>::MINB)
    velocity_kernel(const ShotDesc<T> *__restrict__ shots, const ShotMaps *__restrict__ maps,
                    const Item *__restrict__ items, const int2 *__restrict__ ranges, int tick,
                    const int *__restrict__ dtick, unsigned *__restrict__ err, int ctl) {
  using G = Geo<T, TX, TY, NS, CPT, MB>;
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + NS * G::V_STAGE);
  uint64_t *empty = full + NS;

  const int tid = threadIdx.x;
  const int2 range = ranges[blockIdx.x];
  if (range.x >= range.y) return;
  init_ring<NS, G::NCW, LOAD>(full, empty);

  if (tid >= G::NT) {  // producer warp
    auto issue = [&](const Item &it, int k, int slot, uint64_t *bar, int lane) {
      velocity_issue<T, TX, TY, NS, CPT, MB, LOAD>(shots, maps, it, k, smem + slot * G::V_STAGE, bar, lane);
    };
    ItemPrefetch<T, TX, TY> prefetch{{}, shots, tid - G::NT, ctl, PSI_V0};
    produce<NS, LOAD == LOAD_CP_ASYNC>(items, range, full, empty, issue, prefetch, err, ctl, tid - G::NT);
    return;
  }

  const unsigned long long wait_ns = (ctl & CTL_WITHHOLD_LOADS) ? kTestWaitLimitNs : kWaitLimitNs;
  // step counter: an argument for direct launches, device memory plus an
  // offset inside a replayable CUDA graph
  if (dtick) tick += *dtick;
  unsigned n = 0;
  for (int ii = range.x; ii < range.y; ++ii) {
    const Item item = items[ii];
    if (!velocity_item<T, TX, TY, NS, CPT, MB, G::V_STAGE, false>(shots[item.shot], item, tick, smem, full, empty,
                                                                   n, err, wait_ns, tid))
      return;
  }
}

// ------------------------------------------------- dataflow kernel ----
// Many time steps in one persistent launch.  The work is a list of items,
// each the stress or the velocity half-step of one (shot, x-y tile,
// z-chunk) at one of list_steps steps; a launch of nsteps steps walks the
// list again for every further list_steps steps (the item of list step s
// in pass p runs step p * list_steps + s; items of steps >= nsteps are
// skipped, so one list serves shorter launches); block b takes items
// b, b + G, ... of every pass
// (G blocks, all resident: the launch is cooperative).  Chunk j of a shot
// covers planes [jC, (j+1)C) for stress and the same range shifted down by
// one plane for velocity, so that
//   stress (j, tile, step r)   reads v written by velocity (j and j+1) of
//                              step r-1 on the tile and its four
//                              neighbours, and overwrites the stresses
//                              those items read;
//   velocity (j, tile, step r) reads the stresses of stress (j-1 and j) of
//                              step r on the tile and its neighbours.
// Each item, before its loads, waits for those items' completion counters
// (flags[kind][chunk][tile], NCW added once an item is written: NCW (r + 1)
// once step r is done); the host orders the list so that every dependency
// comes earlier (checked there), so the waits always end.  The host places
// each item soon after the items it waits for (and, with overlapping
// steps, lets a step start where the previous one is done): a velocity
// chunk runs right after the stresses it reads were
// written, while they are still in L2.  Results are bit-identical to the
// two half-step kernels.  Memory ordering: consumer warps write, fence the
// async proxy (the TMA of the reading block), __syncwarp, and arrive (CTA
// scope) on a shared per-item count; the last warp releases the item's
// counter at gpu scope; the producer acquires the counters (relaxed
// loads + fence.acq_rel.gpu), fences the async proxy, arrives on the
// item's ready barrier and then issues its loads; consumers read global
// memory for the item only after that barrier.  Every wait is bounded: a wait that passes its limit
// sets DEV_ERR_TIMEOUT and the block stops.
// RB ready barriers: the producer is at most NS loads ahead of the slowest
// consumer warp and every item takes at least two loads, so it never gets
// RB items ahead (a barrier is re-armed only after every warp passed it).
template <typename T, int TX, int TY, int NS, int CPT, int MB>
struct Flow {
  using G = Geo<T, TX, TY, NS, CPT, MB>;
  static constexpr int STAGE = G::S_STAGE > G::V_STAGE ? G::S_STAGE : G::V_STAGE;
  static constexpr int RB = 8;
  static_assert(RB >= NS / 2 + 2, "ready barriers for the items in flight");
  static constexpr int SMEM = NS * STAGE + 16 * NS + 8 * RB + 4 * RB;
};

__device__ __forceinline__ int ld_relaxed_gpu(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }
__device__ __forceinline__ void red_release_gpu_add(int *p, int v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// CTA-scope acquire-release add on a shared-memory counter; returns the old value.
__device__ __forceinline__ int atom_acq_rel_cta_add(int *p, int v) {
  int old;
  asm volatile("atom.acq_rel.cta.shared::cta.add.s32 %0, [%1], %2;" : "=r"(old) : "r"(smem_u32(p)), "r"(v) : "memory");
  return old;
}

// Lane 0 of the producer: waits until every counter this item depends on
// has reached its target.  The (up to ten) counters are read together, so
// a satisfied item costs one L2 round trip.
template <typename T>
__device__ __forceinline__ bool flow_wait_deps(const ShotDesc<T> &sd, const FlowItem &fi, int txs, int tys, int ncw,
                                               unsigned long long wait_ns) {
  const int ntiles = txs * tys;
  const int tile = fi.it.tile, tx = tile % txs, ty = tile / txs;
  const int *base;
  int c0, c1, target;
  if (fi.kind == 0) {   // stress: velocity of the previous step, chunks j and j+1
    base = sd.flow_flags + (size_t)sd.flow_chunks * ntiles;
    c0 = fi.chunk;
    c1 = fi.chunk + 1 < sd.flow_chunks ? fi.chunk + 1 : -1;
    target = ncw * fi.step;
  } else {              // velocity: stress of this step, chunks j-1 and j
    base = sd.flow_flags;
    c0 = fi.chunk;
    c1 = fi.chunk > 0 ? fi.chunk - 1 : -1;
    target = ncw * (fi.step + 1);
  }
  if (target <= 0) return true;
  const int *p[10];
  int np = 0;
  const int nb[5][2] = {{tx, ty}, {tx - 1, ty}, {tx + 1, ty}, {tx, ty - 1}, {tx, ty + 1}};
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    const int x = nb[q][0], y = nb[q][1];
    if (x < 0 || x >= txs || y < 0 || y >= tys) continue;
    p[np++] = base + (size_t)c0 * ntiles + y * txs + x;
    if (c1 >= 0) p[np++] = base + (size_t)c1 * ntiles + y * txs + x;
  }
  unsigned long long t0 = 0;
  for (;;) {
    int v[10];
#pragma unroll
    for (int q = 0; q < 10; ++q) v[q] = q < np ? ld_relaxed_gpu(p[q]) : target;
    bool ok = true;
#pragma unroll
    for (int q = 0; q < 10; ++q) ok = ok && v[q] >= target;
    if (ok) break;
    const unsigned long long t = globaltimer_ns();
    if (t0 == 0) t0 = t;
    else if (t - t0 > wait_ns) return false;
    __nanosleep(64);
  }
  fence_acq_rel_gpu();
  fence_proxy_async_global();
  return true;
}

template <typename T, int TX, int TY, int NS, int CPT, int MB>
__global__ void __launch_bounds__(Geo<T, TX, TY, NS, CPT, MB>::THREADS, Geo<T, TX, TY, NS, CPT, MB>::MINB)
    flow_kernel(const ShotDesc<T> *__restrict__ shots, const ShotMaps *__restrict__ maps,
                const FlowItem *__restrict__ items, int nitems, int list_steps, int nsteps, int tick,
                const int *__restrict__ dtick, unsigned *__restrict__ err, int ctl) {
  using G = Geo<T, TX, TY, NS, CPT, MB>;
  using F = Flow<T, TX, TY, NS, CPT, MB>;
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + NS * F::STAGE);
  uint64_t *empty = full + NS;
  uint64_t *ready = empty + NS;   // F::RB barriers, one per item in flight
  int *arrived = reinterpret_cast<int *>(ready + F::RB);   // F::RB consumer-warp counters
  const int tid = threadIdx.x;
  if (tid == 0)
    for (int r = 0; r < F::RB; ++r) {
      mbar_init(&ready[r], 1);
      arrived[r] = 0;
    }
  init_ring<NS, G::NCW, LOAD_TMA>(full, empty);
  const unsigned long long wait_ns = (ctl & CTL_WITHHOLD_LOADS) ? kTestWaitLimitNs : kWaitLimitNs;
  const int pass_steps = list_steps > 0 ? list_steps : nsteps;   // (one pass if the list's length is unset)

  if (tid >= G::NT) {  // producer warp
    const int lane = tid - G::NT;
    if (ctl & CTL_WITHHOLD_LOADS) return;  // test mode: no stage is ever filled
    ItemPrefetch<T, TX, TY> pf_s{{}, shots, lane, ctl, PSI_S0};
    ItemPrefetch<T, TX, TY> pf_v{{}, shots, lane, ctl, PSI_V0};
    unsigned n = 0, idx = 0;
    bool ok = true;
    for (int rep = 0; rep < nsteps && ok; rep += pass_steps)
    for (int q = blockIdx.x; q < nitems && ok; q += gridDim.x) {
      FlowItem fi = items[q];
      // the block's next work item into L1: its consumers read it at their
      // next item's start, and so does this warp (101^3: +0.4%)
      if (lane == 0) {
        const int qn = q + (int)gridDim.x < nitems ? q + (int)gridDim.x : (int)blockIdx.x;
        asm volatile("prefetch.global.L1 [%0];" ::"l"(items + qn));
      }
      fi.step += rep;
      if (fi.step >= nsteps) continue;   // a list of more steps than this launch runs
      const ShotDesc<T> &sd = shots[fi.it.shot];
      int good = 1;
      if (lane == 0) {
        const int txs = (sd.nx + TX - 1) / TX, tys = (sd.ny + TY - 1) / TY;
        good = flow_wait_deps(sd, fi, txs, tys, G::NCW, wait_ns);
        if (good) mbar_arrive(&ready[idx % F::RB]);   // release the consumers' global reads
      }
      ++idx;
      if (!__shfl_sync(0xffffffffu, good, 0)) {
        ok = false;
        break;
      }
      if (fi.kind == 0) {
        auto issue = [&](const Item &it, int k, int slot, uint64_t *bar, int l) {
          stress_issue<T, TX, TY, NS, CPT, MB, LOAD_TMA>(shots, maps, it, k, smem + slot * F::STAGE, bar, l);
        };
        ok = produce_item<NS, false>(fi.it, n, full, empty, issue, pf_s, lane);
      } else {
        auto issue = [&](const Item &it, int k, int slot, uint64_t *bar, int l) {
          velocity_issue<T, TX, TY, NS, CPT, MB, LOAD_TMA>(shots, maps, it, k, smem + slot * F::STAGE, bar, l);
        };
        ok = produce_item<NS, false>(fi.it, n, full, empty, issue, pf_v, lane);
      }
    }
    produce_drain<NS, false>(n, ok, full, err, lane);
    return;
  }

  const int lane = tid & 31, warp = tid >> 5;
  if (dtick) tick += *dtick;
  unsigned n = 0, idx = 0;
  for (int rep = 0; rep < nsteps; rep += pass_steps)
  for (int q = blockIdx.x; q < nitems; q += gridDim.x) {
    FlowItem fi = items[q];
    fi.step += rep;
    if (fi.step >= nsteps) continue;
    const ShotDesc<T> &sd = shots[fi.it.shot];
    uint64_t *rb = &ready[idx % F::RB];
    int *arr = &arrived[idx % F::RB];
    const uint32_t rp = (idx / F::RB) & 1;
    ++idx;
    bool ok;
    if (fi.kind == 0)
      ok = stress_item<T, TX, TY, NS, CPT, MB, F::STAGE, true>(sd, fi.it, smem, full, empty, n, err, wait_ns, tid,
                                                                rb, rp);
    else
      ok = velocity_item<T, TX, TY, NS, CPT, MB, F::STAGE, true>(sd, fi.it, tick + fi.step, smem, full, empty, n,
                                                                  err, wait_ns, tid, rb, rp);
    if (!ok) return;
    // this warp's share of the item is written: it arrives (CTA scope) on
    // the item's counter, and the last warp to arrive releases the whole
    // item at gpu scope -- cumulative over the other warps' writes it has
    // acquired -- so one gpu-scope fence per item instead of one per warp
    fence_proxy_async_global();
    __syncwarp();
    if (lane == 0 && atom_acq_rel_cta_add(arr, 1) == G::NCW - 1) {
      *arr = 0;   // re-armed for item idx + RB (no warp is that far ahead)
      const int txs = (sd.nx + TX - 1) / TX, tys = (sd.ny + TY - 1) / TY;
      int *flag = sd.flow_flags + ((size_t)fi.kind * sd.flow_chunks + fi.chunk) * (txs * tys) + fi.it.tile;
      red_release_gpu_add(flag, G::NCW);
    }
    (void)warp;
  }
}

}  // namespace ela3d
