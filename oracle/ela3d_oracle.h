/*
 * ela3d_oracle.h -- CPU restatement of the reference's SEISMIC_CPML time loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: tests/, the smoke entry and
 * bench.py's cpu_baseline leg may call it; the product library never does.
 *
 * It restates, in plain C, the single-threaded float32 program
 * seismicCPML_3d_isotropic_simpelmodel.cpp (loops :376-590, profiles
 * :142-361, gather :593-602, source :605-622), with its hard-coded locals
 * turned into a parameter struct.  Storage is 0-based and x-fastest with one
 * extra zero z-plane (see the reference's read of k = NIMZ+1 at :450/:477).
 * Cell (i, j, k) here is the reference's 1-based cell (i+1, j+1, k+1).
 *
 * Parity is pinned by comparing this restatement with the reference program
 * itself, compiled by oracle/make_ref.py from the unmodified source plus a
 * mechanical parameter patch, on the same inputs (tests/golden/).
 */
#ifndef ELA3D_ORACLE_H
#define ELA3D_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Source time functions (reference: Gaussian derivative at
 * seismicCPML_3d_isotropic_simpelmodel.cpp:610, Ricker at
 * elatic_3d_unified_cuda_memory.cu:441, Gaussian commented at :438). */
enum { ORACLE_STF_RICKER = 0, ORACLE_STF_GAUSS_DERIV = 1, ORACLE_STF_GAUSS = 2 };
/* Injection: force into velocity (seismicCPML_3d_isotropic_cudazerocopy.cu:451-453)
 * or explosive into the normal stresses (simpelmodel.cpp:620-622). */
enum { ORACLE_SRC_FORCE = 0, ORACLE_SRC_EXPLOSIVE = 1 };
/* PML profile variant: reproduce the CPU program's profile code as written,
 * or the textbook C-PML (per-axis thickness, a_x_half set, zmin half active). */
enum { ORACLE_PML_COMPAT = 0, ORACLE_PML_CLEAN = 1 };

typedef struct {
    int nx, ny, nz;
    double dx, dy, dz;
    double dt;
    int npml;
    double npower, k_max;
    double alpha_max;     /* < 0: 2*PI*(f0/2) as the reference computes it */
    double rcoef, vpml;
    double f0, t0, factor;
    int src_i, src_j, src_k;   /* 0-based */
    int src_kind, stf;
    double src_w[3];           /* force weights (vx, vy, vz) */
    double angle_force;        /* degrees, explosive source */
    int nrec;
    const int *rec;            /* nrec x (i, j, k), 0-based */
    int sampgat;
    int pml_mode;
} oracle_params;

/* Runs nsteps time steps from a zero state.
 * seis: nrec x 3 x (nsteps / sampgat), may be NULL.
 * fields: 9 x nx*ny*nz (vx vy vz sxx syy szz sxy sxz syz), may be NULL.
 * Returns 0, or -1 on bad arguments / allocation failure. */
int oracle_run_f32(const oracle_params *p, const float *cp, const float *cs,
                   const float *rho, int nsteps, float *seis, float *fields);
int oracle_run_f64(const oracle_params *p, const double *cp, const double *cs,
                   const double *rho, int nsteps, double *seis, double *fields);

/* The 18 profile arrays the time loop consumes, in this order:
 * a_x, b_x, K_x, a_x_half, b_x_half, K_x_half, then the same for y and z.
 * out holds 6*nx + 6*ny + 6*nz values. */
int oracle_profiles_f32(const oracle_params *p, float *out);
int oracle_profiles_f64(const oracle_params *p, double *out);

#ifdef __cplusplus
}
#endif
#endif
