// ela3d_media.cu -- earth models generated on the GPU straight into a
// shot's padded model arrays (no host arrays, no upload).
//  - homogeneous: constant cp, cs, rho (simpelmodel.cpp:45-59);
//  - layered dome: interfaces z_i(x, y) = depth_i - A exp(-r^2 / (2 s^2))
//    (cells); layer L = number of interfaces at or above the cell, capped at
//    nlayers-1; cs = cp / ratio_L, rho = coef * cp^pow; then cp and rho get
//    independent uniform relative noise of +-perturb from a counter-based
//    hash of (seed, cell) (SplitMix64), so any cell's value is reproducible
//    without a sequential generator;
//  - the five-medium anticline of generate_3d_model_anticline.m: dome
//    Z = ((sin X + sin Y)/2 - 0.5)/0.5 clipped at 0 on X, Y in [0, pi]
//    (:2-13), interfaces h - 100 Z with h = 121/161/201 (:17-30), the k < 80
//    pocket inside medium 3 (:50-55) and the media table (:71-76); depths
//    scale with nz / 201 (exactly the MATLAB model at 201 cells).
// Values are computed in double and rounded to float32, the precision the
// model is defined in, before being stored in the plan's type.
#include <math.h>
#include <stdint.h>

#include "ela3d_internal.h"

namespace ela3d {

__device__ __forceinline__ double hash_uniform(uint64_t seed, uint64_t cell, uint64_t stream) {
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (cell * 2 + stream + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);  // [0, 1)
}

template <typename T>
__global__ void model_kernel(ModelSpec s, int nx, int ny, int nz, int px, T *cp, T *cs, T *rho) {
  const long long n = (long long)px * ny * nz;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(q % px);
    const long long r = q / px;
    const int y = (int)(r % ny), k = (int)(r / ny);
    if (x >= nx) {
      cp[q] = T(0); cs[q] = T(0); rho[q] = T(0);
      continue;
    }
    double vp, vs, dn;
    if (s.kind == MODEL_HOMOGENEOUS) {
      vp = s.cp0; vs = s.cs0; dn = s.rho0;
    } else if (s.kind == MODEL_LAYERED_DOME) {
      const double dx = x - s.dome_xc, dy = y - s.dome_yc;
      const double dome = s.dome_amp * exp(-(dx * dx + dy * dy) / (2.0 * s.dome_sigma * s.dome_sigma));
      int L = 0;
      for (int i = 0; i < s.nlayers && i < kMaxLayers; ++i) L += (k >= s.depth[i] - dome) ? 1 : 0;
      if (L > s.nlayers - 1) L = s.nlayers - 1;
      const double cpl = s.cp[L];
      vs = cpl / s.cs_ratio[L];
      dn = s.rho_coef * pow(cpl, s.rho_pow);
      vp = cpl;
      if (s.perturb > 0) {
        const uint64_t cell = ((uint64_t)k * ny + y) * nx + x;
        vp *= 1.0 + s.perturb * (2.0 * hash_uniform(s.seed, cell, 0) - 1.0);
        dn *= 1.0 + s.perturb * (2.0 * hash_uniform(s.seed, cell, 1) - 1.0);
      }
    } else {  // MODEL_MATLAB_ANTICLINE
      const double PI = 3.141592653589793238462643;
      const double X = PI * x / (nx - 1), Y = PI * y / (ny - 1);
      double Z = ((sin(X) + sin(Y)) / 2.0 - 0.5) / 0.5;
      if (Z < 0) Z = 0;
      const double sc = nz / 201.0;
      const double kk = k + 1;   // 1-based depth index of the MATLAB loop
      const double s1 = 121 * sc - 100 * sc * Z, s2 = 161 * sc - 100 * sc * Z, s3 = 201 * sc - 100 * sc * Z;
      int m = 1;
      if (kk > s1) m = 2;
      if (kk > s2) { m = 3; if (kk < 80 * sc) m = 4; }
      if (kk > s3) m = 5;
      const double media[6][3] = {{0, 0, 0}, {3000, 1700, 2800}, {3600, 1400, 2300}, {3000, 1700, 2800},
                                  {3600, 1700, 2800}, {3650, 1500, 2450}};
      vp = media[m][0]; vs = media[m][1]; dn = media[m][2];
    }
    cp[q] = (T)(float)vp;
    cs[q] = (T)(float)vs;
    rho[q] = (T)(float)dn;
  }
}

cudaError_t launch_model_f32(const ModelSpec &s, int nx, int ny, int nz, int px, float *cp, float *cs, float *rho,
                             cudaStream_t st) {
  model_kernel<float><<<1216, 256, 0, st>>>(s, nx, ny, nz, px, cp, cs, rho);
  return cudaGetLastError();
}
cudaError_t launch_model_f64(const ModelSpec &s, int nx, int ny, int nz, int px, double *cp, double *cs, double *rho,
                             cudaStream_t st) {
  model_kernel<double><<<1216, 256, 0, st>>>(s, nx, ny, nz, px, cp, cs, rho);
  return cudaGetLastError();
}

}  // namespace ela3d
