/*
 * ela3d_oracle_impl.h -- body of the CPU restatement, included twice by
 * ela3d_oracle.c with REAL = float and REAL = double.  TEST INFRASTRUCTURE.
 *
 * Every expression keeps the operand order and the float/double promotions
 * of seismicCPML_3d_isotropic_simpelmodel.cpp so that, built with
 * -ffp-contract=off, the float instance reproduces that program bit for bit.
 * Requires: REAL, SFX (name suffix), POWR, EXPR, LOGR, SINR, COSR.
 */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)

/* One axis of the C-PML profiles.
 * Follows simpelmodel.cpp:142-361: x at :158-224, y at :226-291, z at :293-361.
 * The compat variant keeps three quirks of that code:
 *   - x: the half-node 'a' is written into alpha_x_half instead (:223), so
 *     a_x_half stays 0;
 *   - z: both z profiles are normalised by the y thickness (:326,:333,:350)
 *     and the zmin half-node test reads the stale y abscissa left by the y
 *     loop (:331);
 *   - only the x loop clamps alpha at 0 (:217-218).
 * out: a, b, K, a_half, b_half, K_half, each n long. */
static void FN(axis_profile)(const oracle_params *p, int axis, REAL *out)
{
    const int compat = (p->pml_mode == ORACLE_PML_COMPAT);
    const int n = axis == 0 ? p->nx : (axis == 1 ? p->ny : p->nz);
    const double dd = axis == 0 ? p->dx : (axis == 1 ? p->dy : p->dz);
    REAL *ca = out, *cb = out + n, *cK = out + 2 * n;
    REAL *ca_h = out + 3 * n, *cb_h = out + 4 * n, *cK_h = out + 5 * n;

    const REAL NPOWER = (REAL)p->npower;
    const REAL K_MAX_PML = (REAL)p->k_max;
    const REAL DELTATT = (REAL)p->dt;
    const REAL PI = (REAL)3.141592653589793238462643;
    const REAL f0 = (REAL)p->f0;
    const REAL ALPHA_MAX_PML = p->alpha_max < 0 ? 2 * PI * (f0 / 2) : (REAL)p->alpha_max;
    const REAL Rcoef = (REAL)p->rcoef;
    const REAL vpml = (REAL)p->vpml;

    /* thickness_PML_* = NPOINTS_PML * DELTA* (int product, :148-150) */
    const REAL thick = (REAL)(p->npml * dd);
    const REAL thick_y = (REAL)(p->npml * p->dy);
    const REAL d0 = (REAL)((double)(-(NPOWER + 1) * vpml * LOGR(Rcoef)) / (2.0 * (double)thick));
    const REAL origin_min = thick;
    const REAL origin_max = (REAL)((n - 1) * dd) - thick;
    /* normalisation thickness per test (compat z uses thickness_PML_y) */
    const REAL nrm_full_min = (compat && axis == 2) ? thick_y : thick;
    const REAL nrm_half_min = (compat && axis == 2) ? thick_y : thick;
    const REAL nrm_full_max = thick;
    const REAL nrm_half_max = (compat && axis == 2) ? thick_y : thick;
    /* stale yval after the y loop (:253), read by the zmin half test (:331) */
    const REAL yval_stale = (REAL)p->dy * (REAL)(p->ny - 1);
    const REAL yorigin_min = thick_y;

    if (p->npml == 0) {
        /* the reference divides by a zero thickness here (d0 = x/0); a
         * layer of zero cells is taken to mean no layer: a = 0, b = K = 1 */
        for (int i = 0; i < n; i++) {
            ca[i] = 0; cb[i] = 1; cK[i] = 1;
            ca_h[i] = 0; cb_h[i] = 1; cK_h[i] = 1;
        }
        return;
    }
    for (int i = 0; i < n; i++) {
        REAL d = 0, K = 1, alpha = 0, d_h = 0, K_h = 1, alpha_h = 0;
        REAL a = 0, a_h = 0, xn, ab;
        const REAL val = (REAL)dd * (REAL)i;

        ab = origin_min - val;
        if (ab >= 0.0) {
            xn = ab / nrm_full_min;
            d = d0 * POWR(xn, NPOWER);
            K = (REAL)(1.0 + (K_MAX_PML - 1.0) * POWR(xn, NPOWER));
            alpha = (REAL)(ALPHA_MAX_PML * (1.0 - xn) + 0.1 * ALPHA_MAX_PML);
        }
        if (compat && axis == 2)
            ab = (REAL)(yorigin_min - (yval_stale + p->dy / 2.0));
        else
            ab = (REAL)(origin_min - (val + dd / 2.0));
        if (ab >= 0.0) {
            xn = ab / nrm_half_min;
            d_h = d0 * POWR(xn, NPOWER);
            K_h = (REAL)(1.0 + (K_MAX_PML - 1.0) * POWR(xn, NPOWER));
            alpha_h = (REAL)(ALPHA_MAX_PML * (1.0 - xn) + 0.1 * ALPHA_MAX_PML);
        }
        ab = val - origin_max;
        if (ab >= 0.0) {
            xn = ab / nrm_full_max;
            d = d0 * POWR(xn, NPOWER);
            K = (REAL)(1.0 + (K_MAX_PML - 1.0) * POWR(xn, NPOWER));
            alpha = (REAL)(ALPHA_MAX_PML * (1.0 - xn) + 0.1 * ALPHA_MAX_PML);
        }
        ab = (REAL)(val + dd / 2.0 - origin_max);
        if (ab >= 0.0) {
            xn = ab / nrm_half_max;
            d_h = d0 * POWR(xn, NPOWER);
            K_h = (REAL)(1.0 + (K_MAX_PML - 1.0) * POWR(xn, NPOWER));
            alpha_h = (REAL)(ALPHA_MAX_PML * (1.0 - xn) + 0.1 * ALPHA_MAX_PML);
        }
        if (!compat || axis == 0) {
            if (alpha < 0.0) alpha = 0.0;
            if (alpha_h < 0.0) alpha_h = 0.0;
        }
        const REAL b = EXPR(-(d / K + alpha) * DELTATT);
        const REAL b_h = EXPR(-(d_h / K_h + alpha_h) * DELTATT);
        if (fabs(d) > 1e-6) a = (REAL)(d * (b - 1.0) / (K * (d + K * alpha)));
        if (fabs(d_h) > 1e-6) {
            const REAL v = (REAL)(d_h * (b_h - 1.0) / (K_h * (d_h + K_h * alpha_h)));
            if (!(compat && axis == 0)) a_h = v; /* compat x: lands in alpha_x_half */
        }
        ca[i] = a; cb[i] = b; cK[i] = K;
        ca_h[i] = a_h; cb_h[i] = b_h; cK_h[i] = K_h;
    }
}

int FN(oracle_profiles_)(const oracle_params *p, REAL *out)
{
    if (!p || !out || p->nx < 2 || p->ny < 2 || p->nz < 2) return -1;
    FN(axis_profile)(p, 0, out);
    FN(axis_profile)(p, 1, out + 6 * p->nx);
    FN(axis_profile)(p, 2, out + 6 * p->nx + 6 * p->ny);
    return 0;
}

/* Source time function at step it (1-based), simpelmodel.cpp:608-610 for the
 * Gaussian derivative; the Ricker follows elatic_3d_unified_cuda_memory.cu:441
 * written with the float program's types. */
static REAL FN(source_term)(const oracle_params *p, int it)
{
    const REAL PI = (REAL)3.141592653589793238462643;
    const REAL f0 = (REAL)p->f0, t0 = (REAL)p->t0, factor = (REAL)p->factor;
    const REAL DELTATT = (REAL)p->dt;
    const REAL a = PI * PI * f0 * f0;
    const REAL t = (REAL)(it - 1) * DELTATT;
    if (p->stf == ORACLE_STF_GAUSS_DERIV)
        return (REAL)(-factor * 2.0 * a * (t - t0) * EXPR(-a * POWR((t - t0), 2)));
    if (p->stf == ORACLE_STF_GAUSS)
        return (REAL)(factor * EXPR(-a * POWR((t - t0), 2)));
    return (REAL)(factor * (1.0 - 2.0 * a * POWR((t - t0), 2)) * EXPR(-a * POWR(t - t0, 2)));
}

int FN(oracle_run_)(const oracle_params *p, const REAL *ccp, const REAL *ccs,
                    const REAL *crho_in, int nsteps, REAL *seis, REAL *fields)
{
    if (!p || !ccp || !ccs || !crho_in || nsteps < 0) return -1;
    const int NX = p->nx, NY = p->ny, NZ = p->nz;
    if (NX < 2 || NY < 2 || NZ < 2 || p->sampgat < 1) return -1;
    if (p->src_i < 0 || p->src_i >= NX || p->src_j < 0 || p->src_j >= NY ||
        p->src_k < 0 || p->src_k >= NZ) return -1;
    const long PL = (long)NX * NY;
    const long NC = PL * NZ;
    const long NA = PL * (NZ + 1); /* one zero plane above k = NZ-1 */
    const int nsamp = nsteps / p->sampgat;

    REAL *pool = (REAL *)calloc((size_t)NA * 30 + 18 * (size_t)(NX + NY + NZ), sizeof(REAL));
    if (!pool) return -1;
    REAL *cp = pool, *cs = cp + NA, *rho = cs + NA;
    REAL *vx = rho + NA, *vy = vx + NA, *vz = vy + NA;
    REAL *sxx = vz + NA, *syy = sxx + NA, *szz = syy + NA;
    REAL *sxy = szz + NA, *sxz = sxy + NA, *syz = sxz + NA;
    REAL *m_dvx_dx = syz + NA, *m_dvy_dy = m_dvx_dx + NA, *m_dvz_dz = m_dvy_dy + NA;
    REAL *m_dvy_dx = m_dvz_dz + NA, *m_dvx_dy = m_dvy_dx + NA;
    REAL *m_dvz_dx = m_dvx_dy + NA, *m_dvx_dz = m_dvz_dx + NA;
    REAL *m_dvz_dy = m_dvx_dz + NA, *m_dvy_dz = m_dvz_dy + NA;
    REAL *m_dsxx_dx = m_dvy_dz + NA, *m_dsxy_dy = m_dsxx_dx + NA, *m_dsxz_dz = m_dsxy_dy + NA;
    REAL *m_dsxy_dx = m_dsxz_dz + NA, *m_dsyy_dy = m_dsxy_dx + NA, *m_dsyz_dz = m_dsyy_dy + NA;
    REAL *m_dsxz_dx = m_dsyz_dz + NA, *m_dsyz_dy = m_dsxz_dx + NA, *m_dszz_dz = m_dsyz_dy + NA;
    REAL *prof = m_dszz_dz + NA;
    for (long c = 0; c < NC; c++) { cp[c] = ccp[c]; cs[c] = ccs[c]; rho[c] = crho_in[c]; }

    FN(oracle_profiles_)(p, prof);
    const REAL *a_x = prof, *b_x = a_x + NX, *K_x = b_x + NX;
    const REAL *a_x_half = K_x + NX, *b_x_half = a_x_half + NX, *K_x_half = b_x_half + NX;
    const REAL *a_y = prof + 6 * NX, *b_y = a_y + NY, *K_y = b_y + NY;
    const REAL *a_y_half = K_y + NY, *b_y_half = a_y_half + NY, *K_y_half = b_y_half + NY;
    const REAL *a_z = prof + 6 * NX + 6 * NY, *b_z = a_z + NZ, *K_z = b_z + NZ;
    const REAL *a_z_half = K_z + NZ, *b_z_half = a_z_half + NZ, *K_z_half = b_z_half + NZ;

    const REAL DELTATT = (REAL)p->dt;
    const REAL ONE_OVER_DELTAXX = 1 / (REAL)p->dx;
    const REAL ONE_OVER_DELTAYY = 1 / (REAL)p->dy;
    const REAL ONE_OVER_DELTAZZ = 1 / (REAL)p->dz;
    const REAL PI = (REAL)3.141592653589793238462643;
    const REAL DEGREES_TO_RADIANSS = PI / 180;
    const REAL ANGLE_FORCEE = (REAL)p->angle_force;
    const long lesource = p->src_i + (long)p->src_j * NX + (long)p->src_k * PL;

#define IDX(i, j, k) ((long)(i) + (long)(j) * NX + (long)(k) * PL)
    for (int it = 1; it <= nsteps; it++) {
        /* normal stresses, simpelmodel.cpp:378-413 */
        for (int k = 1; k <= NZ - 1; k++)
            for (int j = 1; j <= NY - 1; j++)
                for (int i = 0; i <= NX - 2; i++) {
                    const long o = IDX(i, j, k), right = o + 1, yb = o - NX, zb = o - PL;
                    REAL vp = cp[o], vs = cs[o], rhos = rho[o];
                    REAL lambda = rhos * (vp * vp - 2 * vs * vs);
                    REAL lambdaplus2mu = rhos * vp * vp;
                    REAL DT_l2m = DELTATT * lambdaplus2mu;
                    REAL DT_l = DELTATT * lambda;
                    REAL dvx_dx = (vx[right] - vx[o]) * ONE_OVER_DELTAXX;
                    REAL dvy_dy = (vy[o] - vy[yb]) * ONE_OVER_DELTAYY;
                    REAL dvz_dz = (vz[o] - vz[zb]) * ONE_OVER_DELTAZZ;
                    m_dvx_dx[o] = b_x_half[i] * m_dvx_dx[o] + a_x_half[i] * dvx_dx;
                    m_dvy_dy[o] = b_y[j] * m_dvy_dy[o] + a_y[j] * dvy_dy;
                    m_dvz_dz[o] = b_z[k] * m_dvz_dz[o] + a_z[k] * dvz_dz;
                    dvx_dx = dvx_dx / K_x_half[i] + m_dvx_dx[o];
                    dvy_dy = dvy_dy / K_y[j] + m_dvy_dy[o];
                    dvz_dz = dvz_dz / K_z[k] + m_dvz_dz[o];
                    sxx[o] = DT_l2m * dvx_dx + DT_l * (dvy_dy + dvz_dz) + sxx[o];
                    syy[o] = DT_l * (dvx_dx + dvz_dz) + DT_l2m * dvy_dy + syy[o];
                    szz[o] = DT_l * (dvx_dx + dvy_dy) + DT_l2m * dvz_dz + szz[o];
                }
        /* sigma_xy, :416-442 */
        for (int k = 0; k <= NZ - 1; k++)
            for (int j = 0; j <= NY - 2; j++)
                for (int i = 1; i <= NX - 1; i++) {
                    const long o = IDX(i, j, k), left = o - 1, yt = o + NX;
                    REAL vs = (cs[left] + cs[yt]) / 2;
                    REAL rhos = (rho[left] + rho[yt]) / 2;
                    REAL mu = rhos * vs * vs;
                    REAL DT_mu = DELTATT * mu;
                    REAL dvy_dx = (vy[o] - vy[left]) * ONE_OVER_DELTAXX;
                    REAL dvx_dy = (vx[yt] - vx[o]) * ONE_OVER_DELTAYY;
                    m_dvy_dx[o] = b_x[i] * m_dvy_dx[o] + a_x[i] * dvy_dx;
                    m_dvx_dy[o] = b_y_half[j] * m_dvx_dy[o] + a_y_half[j] * dvx_dy;
                    dvy_dx = dvy_dx / K_x[i] + m_dvy_dx[o];
                    dvx_dy = dvx_dy / K_y_half[j] + m_dvx_dy[o];
                    sxy[o] = DT_mu * (dvy_dx + dvx_dy) + sxy[o];
                }
        /* sigma_xz and sigma_yz, :445-499 (k = NZ-1 reads the zero plane) */
        for (int k = 0; k <= NZ - 1; k++) {
            for (int j = 0; j <= NY - 1; j++)
                for (int i = 1; i <= NX - 1; i++) {
                    const long o = IDX(i, j, k), left = o - 1, zt = o + PL;
                    REAL vs = (cs[left] + cs[zt]) / 2;
                    REAL rhos = (rho[left] + rho[zt]) / 2;
                    REAL mu = rhos * vs * vs;
                    REAL DT_mu = DELTATT * mu;
                    REAL dvz_dx = (vz[o] - vz[left]) * ONE_OVER_DELTAXX;
                    REAL dvx_dz = (vx[zt] - vx[o]) * ONE_OVER_DELTAZZ;
                    m_dvz_dx[o] = b_x[i] * m_dvz_dx[o] + a_x[i] * dvz_dx;
                    m_dvx_dz[o] = b_z_half[k] * m_dvx_dz[o] + a_z_half[k] * dvx_dz;
                    dvz_dx = dvz_dx / K_x[i] + m_dvz_dx[o];
                    dvx_dz = dvx_dz / K_z_half[k] + m_dvx_dz[o];
                    sxz[o] = DT_mu * (dvz_dx + dvx_dz) + sxz[o];
                }
            for (int j = 0; j <= NY - 2; j++)
                for (int i = 0; i <= NX - 1; i++) {
                    const long o = IDX(i, j, k), zt = o + PL, yt = o + NX;
                    REAL vs = (cs[yt] + cs[zt]) / 2;
                    REAL rhos = (rho[yt] + rho[zt]) / 2;
                    REAL mu = rhos * vs * vs;
                    REAL DT_mu = DELTATT * mu;
                    REAL dvz_dy = (vz[yt] - vz[o]) * ONE_OVER_DELTAYY;
                    REAL dvy_dz = (vy[zt] - vy[o]) * ONE_OVER_DELTAZZ;
                    m_dvz_dy[o] = b_y_half[j] * m_dvz_dy[o] + a_y_half[j] * dvz_dy;
                    m_dvy_dz[o] = b_z_half[k] * m_dvy_dz[o] + a_z_half[k] * dvy_dz;
                    dvz_dy = dvz_dy / K_y_half[j] + m_dvz_dy[o];
                    dvy_dz = dvy_dz / K_z_half[k] + m_dvy_dz[o];
                    syz[o] = DT_mu * (dvz_dy + dvy_dz) + syz[o];
                }
        }
        /* vx and vy, :502-560 */
        for (int k = 1; k <= NZ - 1; k++) {
            for (int j = 1; j <= NY - 1; j++)
                for (int i = 1; i <= NX - 1; i++) {
                    const long o = IDX(i, j, k), left = o - 1, yb = o - NX, zb = o - PL;
                    REAL rhos = (rho[o] + rho[left]) / 2;
                    REAL DT_over_rho = DELTATT / rhos;
                    REAL dsxx_dx = (sxx[o] - sxx[left]) * ONE_OVER_DELTAXX;
                    REAL dsxy_dy = (sxy[o] - sxy[yb]) * ONE_OVER_DELTAYY;
                    REAL dsxz_dz = (sxz[o] - sxz[zb]) * ONE_OVER_DELTAZZ;
                    m_dsxx_dx[o] = b_x[i] * m_dsxx_dx[o] + a_x[i] * dsxx_dx;
                    m_dsxy_dy[o] = b_y[j] * m_dsxy_dy[o] + a_y[j] * dsxy_dy;
                    m_dsxz_dz[o] = b_z[k] * m_dsxz_dz[o] + a_z[k] * dsxz_dz;
                    dsxx_dx = dsxx_dx / K_x[i] + m_dsxx_dx[o];
                    dsxy_dy = dsxy_dy / K_y[j] + m_dsxy_dy[o];
                    dsxz_dz = dsxz_dz / K_z[k] + m_dsxz_dz[o];
                    vx[o] = DT_over_rho * (dsxx_dx + dsxy_dy + dsxz_dz) + vx[o];
                }
            for (int j = 0; j <= NY - 2; j++)
                for (int i = 0; i <= NX - 2; i++) {
                    const long o = IDX(i, j, k), right = o + 1, zb = o - PL, yt = o + NX;
                    REAL rhos = (rho[o] + rho[yt]) / 2;
                    REAL DT_over_rho = DELTATT / rhos;
                    REAL dsxy_dx = (sxy[right] - sxy[o]) * ONE_OVER_DELTAXX;
                    REAL dsyy_dy = (syy[yt] - syy[o]) * ONE_OVER_DELTAYY;
                    REAL dsyz_dz = (syz[o] - syz[zb]) * ONE_OVER_DELTAZZ;
                    m_dsxy_dx[o] = b_x_half[i] * m_dsxy_dx[o] + a_x_half[i] * dsxy_dx;
                    m_dsyy_dy[o] = b_y_half[j] * m_dsyy_dy[o] + a_y_half[j] * dsyy_dy;
                    m_dsyz_dz[o] = b_z[k] * m_dsyz_dz[o] + a_z[k] * dsyz_dz;
                    dsxy_dx = dsxy_dx / K_x_half[i] + m_dsxy_dx[o];
                    dsyy_dy = dsyy_dy / K_y_half[j] + m_dsyy_dy[o];
                    dsyz_dz = dsyz_dz / K_z[k] + m_dsyz_dz[o];
                    vy[o] = DT_over_rho * (dsxy_dx + dsyy_dy + dsyz_dz) + vy[o];
                }
        }
        /* vz, :563-590 */
        for (int k = 0; k <= NZ - 2; k++)
            for (int j = 1; j <= NY - 1; j++)
                for (int i = 0; i <= NX - 2; i++) {
                    const long o = IDX(i, j, k), right = o + 1, yb = o - NX, zt = o + PL;
                    REAL rhos = (rho[o] + rho[zt]) / 2;
                    REAL DT_over_rho = DELTATT / rhos;
                    REAL dsxz_dx = (sxz[right] - sxz[o]) * ONE_OVER_DELTAXX;
                    REAL dsyz_dy = (syz[o] - syz[yb]) * ONE_OVER_DELTAYY;
                    REAL dszz_dz = (szz[zt] - szz[o]) * ONE_OVER_DELTAZZ;
                    m_dsxz_dx[o] = b_x_half[i] * m_dsxz_dx[o] + a_x_half[i] * dsxz_dx;
                    m_dsyz_dy[o] = b_y[j] * m_dsyz_dy[o] + a_y[j] * dsyz_dy;
                    m_dszz_dz[o] = b_z_half[k] * m_dszz_dz[o] + a_z_half[k] * dszz_dz;
                    dsxz_dx = dsxz_dx / K_x_half[i] + m_dsxz_dx[o];
                    dsyz_dy = dsyz_dy / K_y[j] + m_dsyz_dy[o];
                    dszz_dz = dszz_dz / K_z_half[k] + m_dszz_dz[o];
                    vz[o] = DT_over_rho * (dsxz_dx + dsyz_dy + dszz_dz) + vz[o];
                }
        /* receivers: velocity after this step's update, before the source
         * (the gather at :593-602 precedes the injection at :605-622) */
        if (seis && it % p->sampgat == 0 && it / p->sampgat <= nsamp) {
            const int s = it / p->sampgat - 1;
            for (int r = 0; r < p->nrec; r++) {
                const int *q = p->rec + 3 * r;
                const long o = IDX(q[0], q[1], q[2]);
                seis[((long)r * 3 + 0) * nsamp + s] = vx[o];
                seis[((long)r * 3 + 1) * nsamp + s] = vy[o];
                seis[((long)r * 3 + 2) * nsamp + s] = vz[o];
            }
        }
        /* source */
        {
            const REAL source_term = FN(source_term)(p, it);
            if (p->src_kind == ORACLE_SRC_EXPLOSIVE) {
                /* :607,:611-612,:620-622 */
                REAL lambdaplus2mu = rho[lesource] * cp[lesource] * cp[lesource];
                REAL force_x = SINR(ANGLE_FORCEE * DEGREES_TO_RADIANSS) * source_term;
                REAL force_y = COSR(ANGLE_FORCEE * DEGREES_TO_RADIANSS) * source_term;
                sxx[lesource] = sxx[lesource] + force_x * DELTATT * lambdaplus2mu;
                syy[lesource] = syy[lesource] + force_x * DELTATT * lambdaplus2mu;
                szz[lesource] = szz[lesource] + force_y * DELTATT * lambdaplus2mu;
            } else {
                /* seismicCPML_3d_isotropic_cudazerocopy.cu:451-453, per-component weight */
                const long o = lesource;
                if (p->src_w[0] != 0.0) {
                    REAL f = (REAL)p->src_w[0] * source_term;
                    vx[o] = vx[o] + f * DELTATT / ((rho[o] + rho[o - 1]) / 2);
                }
                if (p->src_w[1] != 0.0) {
                    REAL f = (REAL)p->src_w[1] * source_term;
                    vy[o] = vy[o] + f * DELTATT / ((rho[o] + rho[o + NX]) / 2);
                }
                if (p->src_w[2] != 0.0) {
                    REAL f = (REAL)p->src_w[2] * source_term;
                    vz[o] = vz[o] + f * DELTATT / ((rho[o] + rho[o + PL]) / 2);
                }
            }
        }
    }
#undef IDX
    if (fields) {
        REAL *fl[9] = {vx, vy, vz, sxx, syy, szz, sxy, sxz, syz};
        for (int f = 0; f < 9; f++)
            for (long c = 0; c < NC; c++) fields[(long)f * NC + c] = fl[f][c];
    }
    free(pool);
    return 0;
}

#undef FN
#undef CAT
#undef CAT_
