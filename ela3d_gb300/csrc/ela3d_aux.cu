// ela3d_aux.cu -- set-up and monitoring kernels around the time loop:
// C-PML profiles and source time function (computed in FP64 on the GPU and
// rounded to the plan's type), model staging, the explosive source, and the
// FP64 total-energy reduction used by the stability monitor.
#include <math.h>

#include "ela3d_internal.h"

namespace ela3d {

// C-PML profiles of one axis in FP64, simpelmodel.cpp:142-361.
// d0 = -(NPOWER+1) vpml ln(R) / (2 L); inside the layer, with x the
// normalised depth into it: d = d0 x^N, K = 1 + (Kmax-1) x^N,
// alpha = amax (1 - x) + 0.1 amax, b = exp(-(d/K + alpha) dt),
// a = d (b - 1) / (K (d + K alpha)) where |d| > 1e-6.  Full nodes sit at
// i*d, half nodes at (i + 1/2)*d.  The compat variant keeps the CPU
// program's quirks: a_x_half stays 0 (:223), z is normalised by the y
// thickness (:326,:333,:350), the zmin half-node test uses the stale y
// abscissa (:331), and only x clamps alpha (:217-218).
template <typename T>
__global__ void profile_kernel(AxisProfileArgs p, T *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.stride) return;
  T *a_f = out, *b_f = out + p.stride, *ik_f = out + 2 * p.stride;
  T *a_h = out + 3 * p.stride, *b_h = out + 4 * p.stride, *ik_h = out + 5 * p.stride;
  if (i >= p.n) {  // padding columns: identity
    a_f[i] = 0; b_f[i] = 1; ik_f[i] = 1; a_h[i] = 0; b_h[i] = 1; ik_h[i] = 1;
    return;
  }
  const bool compat = p.compat != 0, zc = compat && p.axis == 2;
  const double thick = p.npml * p.d, thick_y = p.npml * p.dy;
  const double d0 = -(p.npower + 1.0) * p.vpml * log(p.rcoef) / (2.0 * thick);
  const double omin = thick, omax = (p.n - 1) * p.d - thick;
  const double val = p.d * i;
  double d = 0, K = 1, al = 0, dh = 0, Kh = 1, alh = 0;
  auto layer = [&](double ab, double nrm, double &dd, double &KK, double &aa) {
    const double xn = ab / nrm;
    const double pw = pow(xn, p.npower);
    dd = d0 * pw;
    KK = 1.0 + (p.k_max - 1.0) * pw;
    aa = p.alpha_max * (1.0 - xn) + 0.1 * p.alpha_max;
  };
  double ab = omin - val;
  if (ab >= 0.0) layer(ab, zc ? thick_y : thick, d, K, al);
  ab = zc ? thick_y - (p.dy * (p.ny - 1) + p.dy / 2.0) : omin - (val + p.d / 2.0);
  if (ab >= 0.0) layer(ab, zc ? thick_y : thick, dh, Kh, alh);
  ab = val - omax;
  if (ab >= 0.0) layer(ab, thick, d, K, al);
  ab = val + p.d / 2.0 - omax;
  if (ab >= 0.0) layer(ab, zc ? thick_y : thick, dh, Kh, alh);
  if (!compat || p.axis == 0) {
    if (al < 0.0) al = 0.0;
    if (alh < 0.0) alh = 0.0;
  }
  const double b = exp(-(d / K + al) * p.dt);
  const double bh = exp(-(dh / Kh + alh) * p.dt);
  double a = 0, ah = 0;
  if (fabs(d) > 1e-6) a = d * (b - 1.0) / (K * (d + K * al));
  if (fabs(dh) > 1e-6 && !(compat && p.axis == 0)) ah = dh * (bh - 1.0) / (Kh * (dh + Kh * alh));
  a_f[i] = (T)a; b_f[i] = (T)b; ik_f[i] = (T)(1.0 / K);
  a_h[i] = (T)ah; b_h[i] = (T)bh; ik_h[i] = (T)(1.0 / Kh);
}

// Source time function per step it = 1..nstep at t = (it-1) dt:
// Ricker f (1 - 2a tau^2) e^{-a tau^2} (elatic_3d_unified_cuda_memory.cu:441),
// Gaussian derivative -2 f a tau e^{-a tau^2} (simpelmodel.cpp:610),
// Gaussian f e^{-a tau^2}; a = pi^2 f0^2, tau = t - t0.
template <typename T>
__global__ void stf_kernel(StfArgs p, T *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.nstep) return;
  const double PI = 3.141592653589793238462643;
  const double a = PI * PI * p.f0 * p.f0;
  const double tau = i * p.dt - p.t0;
  const double g = exp(-a * tau * tau);
  double s;
  if (p.stf == 1) s = -p.factor * 2.0 * a * tau * g;
  else if (p.stf == 2) s = p.factor * g;
  else s = p.factor * (1.0 - 2.0 * a * tau * tau) * g;
  out[i] = (T)s;
}

template <typename T>
__global__ void pad_kernel(const float *__restrict__ src, T *__restrict__ dst, int nx, int ny, int nz,
                           int px) {
  const long long n = (long long)px * ny * nz;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(q % px);
    const long long r = q / px;  // row index = k*ny + j
    dst[q] = x < nx ? (T)src[r * nx + x] : T(0);
  }
}

// Explosive source after the velocity half-step, simpelmodel.cpp:607-622:
// sigma_nn += w_nn s dt (lambda + 2 mu) with (w) = (sin a, sin a, cos a).
template <typename T>
__global__ void explosive_kernel(const ShotDesc<T> *shots, int nshots, int tick, const int *dtick) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nshots) return;
  if (dtick) tick += *dtick;
  const ShotDesc<T> &sd = shots[q];
  if (sd.src_kind != 1) return;
  const int it = tick - sd.tick0;
  if (it < 1 || it > sd.nstep) return;
  const long long o = ((long long)sd.src_k * sd.ny + sd.src_j) * sd.px + sd.src_i;
  const T l2m = sd.rho[o] * sd.cp[o] * sd.cp[o];
  const T s = sd.stf[it - 1];
  const T fx = sd.expl_w[0] * s, fy = sd.expl_w[1] * s, fz = sd.expl_w[2] * s;
  const T sxx = sd.f[3][o] + fx * sd.dt * l2m;
  const T syy = sd.f[4][o] + fy * sd.dt * l2m;
  const T szz = sd.f[5][o] + fz * sd.dt * l2m;
  sd.f[3][o] = sxx;
  sd.f[4][o] = syy;
  sd.f[5][o] = szz;
  // source-point trace (elatic_3d_unified_cuda_memory.cu:463-465)
  const int ns = sd.nstep + 1;
  sd.src_trace[it] = sxx;
  sd.src_trace[ns + it] = syy;
  sd.src_trace[2 * ns + it] = szz;
}

// Kinetic 1/2 rho |v|^2 plus isotropic strain energy
// (1/(4mu)) sigma:sigma - lambda / (4mu(3lambda+2mu)) tr(sigma)^2, cell-local,
// accumulated in FP64 (no counterpart in the reference; the stability monitor).
// Two passes in a fixed order, so repeated calls on one state agree to the
// bit: one block per z-plane writes the plane's sum to part[k], then one
// block adds the planes in order (energy_sum_kernel).
__device__ __forceinline__ double block_sum_f64(double v) {
  __shared__ double part[32];
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  v = 0.0;
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.0;
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  }
  return v;  // valid in thread 0
}

template <typename T>
__global__ void energy_plane_kernel(const ShotDesc<T> *shot, int nx, int ny, double *part) {
  const ShotDesc<T> &sd = *shot;
  const int k = blockIdx.x;
  const long long cells = (long long)nx * ny;
  double acc = 0.0;
  for (long long q = threadIdx.x; q < cells; q += blockDim.x) {
    const long long y = q / nx, x = q - y * nx;
    const long long o = ((long long)k * ny + y) * sd.px + x;
    const double rho = sd.rho[o], cp = sd.cp[o], cs = sd.cs[o];
    const double mu = rho * cs * cs, lam = rho * (cp * cp - 2.0 * cs * cs);
    const double vx = sd.f[0][o], vy = sd.f[1][o], vz = sd.f[2][o];
    const double sxx = sd.f[3][o], syy = sd.f[4][o], szz = sd.f[5][o];
    const double sxy = sd.f[6][o], sxz = sd.f[7][o], syz = sd.f[8][o];
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
  acc = block_sum_f64(acc);
  if (threadIdx.x == 0) part[k] = acc;
}

template <typename T>
__global__ void energy_sum_kernel(const ShotDesc<T> *shot, const double *part, int nz, double *out) {
  const ShotDesc<T> &sd = *shot;
  double acc = 0.0;
  for (int k = threadIdx.x; k < nz; k += blockDim.x) acc += part[k];
  acc = block_sum_f64(acc);
  if (threadIdx.x == 0) *out = acc * (double)(1.0 / sd.idx) * (double)(1.0 / sd.idy) * (double)(1.0 / sd.idz);
}

// Device step counter for replayable CUDA graphs.
__global__ void tick_set_kernel(int *dtick, int value) { *dtick = value; }
__global__ void tick_add_kernel(int *dtick, int delta) { *dtick += delta; }

cudaError_t launch_tick_set(int *dtick, int value, cudaStream_t s) {
  tick_set_kernel<<<1, 1, 0, s>>>(dtick, value);
  return cudaGetLastError();
}
cudaError_t launch_tick_add(int *dtick, int delta, cudaStream_t s) {
  tick_add_kernel<<<1, 1, 0, s>>>(dtick, delta);
  return cudaGetLastError();
}

static int blocks_for(long long n, int threads, int cap) {
  long long b = (n + threads - 1) / threads;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

cudaError_t launch_profile_f32(const AxisProfileArgs &a, float *out, cudaStream_t s) {
  profile_kernel<float><<<(a.stride + 127) / 128, 128, 0, s>>>(a, out);
  return cudaGetLastError();
}
cudaError_t launch_profile_f64(const AxisProfileArgs &a, double *out, cudaStream_t s) {
  profile_kernel<double><<<(a.stride + 127) / 128, 128, 0, s>>>(a, out);
  return cudaGetLastError();
}
cudaError_t launch_stf_f32(const StfArgs &a, float *out, cudaStream_t s) {
  stf_kernel<float><<<(a.nstep + 255) / 256, 256, 0, s>>>(a, out);
  return cudaGetLastError();
}
cudaError_t launch_stf_f64(const StfArgs &a, double *out, cudaStream_t s) {
  stf_kernel<double><<<(a.nstep + 255) / 256, 256, 0, s>>>(a, out);
  return cudaGetLastError();
}
cudaError_t launch_pad_f32(const float *src, float *dst, int nx, int ny, int nz, int px, cudaStream_t s) {
  pad_kernel<float><<<blocks_for((long long)px * ny * nz, 256, 4096), 256, 0, s>>>(src, dst, nx, ny, nz, px);
  return cudaGetLastError();
}
cudaError_t launch_pad_f64(const float *src, double *dst, int nx, int ny, int nz, int px, cudaStream_t s) {
  pad_kernel<double><<<blocks_for((long long)px * ny * nz, 256, 4096), 256, 0, s>>>(src, dst, nx, ny, nz, px);
  return cudaGetLastError();
}
cudaError_t launch_explosive_f32(const ShotDesc<float> *shots, int nshots, int tick, const int *dtick,
                                 cudaStream_t s) {
  explosive_kernel<float><<<(nshots + 63) / 64, 64, 0, s>>>(shots, nshots, tick, dtick);
  return cudaGetLastError();
}
cudaError_t launch_explosive_f64(const ShotDesc<double> *shots, int nshots, int tick, const int *dtick,
                                 cudaStream_t s) {
  explosive_kernel<double><<<(nshots + 63) / 64, 64, 0, s>>>(shots, nshots, tick, dtick);
  return cudaGetLastError();
}
// out[0] = the energy; out[1 .. nz] = the per-plane sums (scratch)
template <typename T>
static cudaError_t launch_energy(const ShotDesc<T> *shot, int nx, int ny, int nz, double *out, cudaStream_t s) {
  energy_plane_kernel<T><<<nz, 256, 0, s>>>(shot, nx, ny, out + 1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  energy_sum_kernel<T><<<1, 256, 0, s>>>(shot, out + 1, nz, out);
  return cudaGetLastError();
}
cudaError_t launch_energy_f32(const ShotDesc<float> *shot, int nx, int ny, int nz, double *out, cudaStream_t s) {
  return launch_energy(shot, nx, ny, nz, out, s);
}
cudaError_t launch_energy_f64(const ShotDesc<double> *shot, int nx, int ny, int nz, double *out, cudaStream_t s) {
  return launch_energy(shot, nx, ny, nz, out, s);
}

}  // namespace ela3d
