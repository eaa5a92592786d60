// ela3d_stencil.cu -- compiled instances of the stress and velocity kernels.
// Each instance fixes the real type, the x-y tile (TX x TY cells) and the
// number of shared-memory stages NS; the engine's autotuner picks one per
// grid size.
#include "ela3d_internal.h"
#include "ela3d_stencil.cuh"

namespace ela3d {

// NSV: stages of the velocity kernel's ring (its stage is smaller than the
// stress kernel's, so it can hold more of them); the dataflow kernel runs
// both half-steps in one ring of NS stages.
template <typename T, int TX, int TY, int NS, int CPT = Vec<T>::N, int MB = 0, int LOAD = LOAD_TMA, int NSV = NS>
static Variant make_variant() {
  using G = Geo<T, TX, TY, NS, CPT, MB>;
  using GV = Geo<T, TX, TY, NSV, CPT, MB>;
  Variant v;
  v.fp64 = sizeof(T) == 8;
  v.tx = TX;
  v.ty = TY;
  v.ns = NS;
  v.ns_vel = NSV;
  v.threads = G::THREADS;
  v.stress_smem = G::S_SMEM;
  v.vel_smem = GV::V_SMEM;
  v.halo = G::H;
  v.loads = LOAD;
  v.stress = reinterpret_cast<const void *>(&stress_kernel<T, TX, TY, NS, CPT, MB, LOAD>);
  v.velocity = reinterpret_cast<const void *>(&velocity_kernel<T, TX, TY, NSV, CPT, MB, LOAD>);
  v.flow = nullptr;
  v.flow_smem = 0;
  if constexpr (LOAD == LOAD_TMA) {
    v.flow = reinterpret_cast<const void *>(&flow_kernel<T, TX, TY, NS, CPT, MB>);
    v.flow_smem = Flow<T, TX, TY, NS, CPT, MB>::SMEM;
  }
  return v;
}

static const Variant kVariants[] = {
    // velocity ring of 5 stages (5 x 38 KB; the stress ring's 4 x 46 KB):
    // more bytes in flight per SM, 1.2% less velocity time at 256^3
    make_variant<float, 128, 7, 4, 4, 0, LOAD_TMA, 5>(),
    make_variant<float, 128, 6, 5>(),
    make_variant<float, 128, 5, 6>(),
    make_variant<float, 64, 14, 4>(),
    make_variant<float, 128, 3, 4>(),
    make_variant<float, 64, 6, 4>(),
    // 28 threads per row, so a warp spans two rows: covers rows of ~100
    // cells with less waste than the 128-wide tile (101: 90% against 79%)
    make_variant<float, 112, 8, 4>(),
    // the 128x7 tile with its stages filled by cp.async instead of TMA (the
    // measured alternative to the tensor-memory-accelerator loads)
    make_variant<float, 128, 7, 4, 4, 0, LOAD_CP_ASYNC>(),
    // FP64 (the accuracy build; its rate on GB300 makes it compute-bound):
    // one cell per thread keeps it free of register spills
    make_variant<double, 32, 7, 4, 1>(),
    make_variant<double, 32, 3, 4, 1, 2>(),
    make_variant<double, 32, 6, 3>(),
    make_variant<double, 64, 3, 4>(),
};

const Variant *variants(int *count) {
  *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
  return kVariants;
}

}  // namespace ela3d
