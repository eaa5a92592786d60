// ela3d_stencil.cu -- compiled instances of the stress and velocity kernels.
// Each instance fixes the real type, the x-y tile (TX x TY cells) and the
// number of shared-memory stages NS; the engine's autotuner picks one per
// grid size.
#include "ela3d_internal.h"
#include "ela3d_stencil.cuh"

namespace ela3d {

template <typename T, int TX, int TY, int NS>
static Variant make_variant() {
  using G = Geo<T, TX, TY, NS>;
  Variant v;
  v.fp64 = sizeof(T) == 8;
  v.tx = TX;
  v.ty = TY;
  v.ns = NS;
  v.threads = G::NT;
  v.stress_smem = G::S_SMEM;
  v.vel_smem = G::V_SMEM;
  v.halo = G::H;
  v.stress = reinterpret_cast<const void *>(&stress_kernel<T, TX, TY, NS>);
  v.velocity = reinterpret_cast<const void *>(&velocity_kernel<T, TX, TY, NS>);
  return v;
}

static const Variant kVariants[] = {
    make_variant<float, 64, 8, 4>(),
    make_variant<float, 64, 4, 4>(),
    make_variant<float, 128, 4, 3>(),
    make_variant<float, 32, 8, 4>(),
    make_variant<float, 64, 16, 3>(),
    make_variant<double, 32, 8, 3>(),
    make_variant<double, 64, 4, 3>(),
};

const Variant *variants(int *count) {
  *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
  return kVariants;
}

}  // namespace ela3d
