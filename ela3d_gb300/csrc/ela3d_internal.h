// ela3d_internal.h -- declarations shared between the host engine
// (ela3d_engine.cu) and the kernel translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ela3d_device.cuh"

namespace ela3d {

// One compiled instance of the two stencil kernels.
struct Variant {
  int fp64;             // 0 float, 1 double
  int tx, ty, ns;       // tile and pipeline depth (stress kernel, dataflow kernel)
  int ns_vel;           // pipeline depth of the velocity kernel
  int threads;          // threads per block
  int stress_smem, vel_smem;  // dynamic shared memory bytes
  int halo;             // x halo (elements) of the wide boxes
  int loads;            // LOAD_TMA or LOAD_CP_ASYNC (how stages are filled)
  const void *stress;   // __global__ entry points
  const void *velocity;
  const void *flow;     // dataflow kernel (many steps per launch); null if not compiled
  int flow_smem;
};

// All compiled variants (ela3d_stencil.cu).
const Variant *variants(int *count);

// Inputs of the FP64 profile kernel for one axis (ela3d_aux.cu).
struct AxisProfileArgs {
  int n;          // cells on this axis
  int stride;     // length of each of the six output arrays (>= n)
  int axis;       // 0 x, 1 y, 2 z
  int compat;     // reproduce the reference CPU profile code
  int npml;
  int ny;         // for the compat zmin half-node test
  double d, dy;   // spacing of this axis and of y
  double npower, k_max, alpha_max, rcoef, vpml, dt;
};

struct StfArgs {
  int nstep, stf;
  double f0, t0, factor, dt;
};

// Launchers (return the launch error).
cudaError_t launch_profile_f32(const AxisProfileArgs &a, float *out, cudaStream_t s);
cudaError_t launch_profile_f64(const AxisProfileArgs &a, double *out, cudaStream_t s);
cudaError_t launch_stf_f32(const StfArgs &a, float *out, cudaStream_t s);
cudaError_t launch_stf_f64(const StfArgs &a, double *out, cudaStream_t s);
// Copies a compact float nx*ny*nz array into a padded [nz][ny][px] array.
cudaError_t launch_pad_f32(const float *src, float *dst, int nx, int ny, int nz, int px, cudaStream_t s);
cudaError_t launch_pad_f64(const float *src, double *dst, int nx, int ny, int nz, int px, cudaStream_t s);
// Explosive source after the velocity half-step, one thread per shot.
cudaError_t launch_explosive_f32(const ShotDesc<float> *shots, int nshots, int tick, const int *dtick,
                                 cudaStream_t s);
cudaError_t launch_explosive_f64(const ShotDesc<double> *shots, int nshots, int tick, const int *dtick,
                                 cudaStream_t s);
// Device step counter of replayable graphs: *dtick = value / *dtick += delta.
cudaError_t launch_tick_set(int *dtick, int value, cudaStream_t s);
cudaError_t launch_tick_add(int *dtick, int delta, cudaStream_t s);
// Total energy of one shot, accumulated into *out (double, device).
cudaError_t launch_energy_f32(const ShotDesc<float> *shot, int nx, int ny, int nz, double *out, cudaStream_t s);
cudaError_t launch_energy_f64(const ShotDesc<double> *shot, int nx, int ny, int nz, double *out, cudaStream_t s);

// Model generated on the device (ela3d_media.cu); mirrors ela3d_model_spec.
enum { MODEL_HOMOGENEOUS = 0, MODEL_LAYERED_DOME = 1, MODEL_MATLAB_ANTICLINE = 2 };
constexpr int kMaxLayers = 8;
struct ModelSpec {
  int kind, nlayers;
  double cp[kMaxLayers], cs_ratio[kMaxLayers], depth[kMaxLayers];
  double dome_amp, dome_sigma, dome_xc, dome_yc;
  double rho_coef, rho_pow, perturb;
  unsigned long long seed;
  double cp0, cs0, rho0;
};
cudaError_t launch_model_f32(const ModelSpec &s, int nx, int ny, int nz, int px, float *cp, float *cs, float *rho,
                             cudaStream_t st);
cudaError_t launch_model_f64(const ModelSpec &s, int nx, int ny, int nz, int px, double *cp, double *cs,
                             double *rho, cudaStream_t st);

}  // namespace ela3d
