/*
 * ref_harness.h -- hooks included by the patched reference CPU program that
 * oracle/make_ref.py generates under oracle/_ref/.  TEST INFRASTRUCTURE.
 *
 * The reference program (seismicCPML_3d_isotropic_simpelmodel.cpp) hard-codes
 * every parameter in main().  The patch replaces those literals with fields
 * of g_cfg, read here from a "key value" text file (argv[1]), and calls:
 *   ref_load_model  after the constant model fill   (reference :45-59)
 *   ref_record      between the gather and the source (:592-604)
 *   ref_step_hook   at the top of each time step and after the loop (:376)
 *   ref_finish      before the frees                (:728)
 * Files written to the working directory:
 *   seis.bin   nrec x 3 x (nstep/sampgat) values (the program's real type)
 *   fields.bin 9 compact NX*NY*NZ fields: vx vy vz sxx syy szz sxy sxz syz
 *   steps.txt  "t_first t_last steps" wall-clock seconds of the timed steps
 * Cell (i, j, k) in the config is 0-based; the program stores the 1-based
 * cell (i+1, j+1, k+1) at address (i+1) + (j+1)*NX + (k+1)*NX*NY.
 */
#ifndef ELA3D_REF_HARNESS_H
#define ELA3D_REF_HARNESS_H

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <fstream>
#include <sstream>
#include <time.h>

struct ref_cfg_t {
    int nx = 32, ny = 32, nz = 32;
    int dx = 10;
    double dt = 1e-3;
    int nstep = 10, sampgat = 1, it_output = 1 << 30;
    int ngatx = 1, ngaty = 1;
    int npml = 10;
    double npower = 2, k_max = 1, alpha_max = -1, rcoef = 1e-3, vpml = 3000;
    double f0 = 7, t0 = 1.2 / 7, factor = 1e7, angle = 0;
    int src_i = 16, src_j = 16, src_k = 16;
    int src_kind = 0, stf = 0;
    double w[3] = {0, 0, 1};
    int clean = 0;
    int time_from = 1;   /* first timed step (inclusive) */
    std::string model_prefix; /* <prefix>cp.bin, cs.bin, rho.bin; empty = keep fill */
    std::vector<int> rec;     /* 0-based i j k triples */
};

static ref_cfg_t g_cfg;
static std::vector<double> g_seis;
static double g_t_first = 0, g_t_last = 0;

static double ref_now()
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static void ref_load_cfg(int argc, char **argv)
{
    if (argc < 2) { fprintf(stderr, "usage: %s config.txt\n", argv[0]); exit(2); }
    std::ifstream in(argv[1]);
    if (!in) { fprintf(stderr, "cannot open %s\n", argv[1]); exit(2); }
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream ss(line);
        std::string k;
        if (!(ss >> k) || k[0] == '#') continue;
        ref_cfg_t &c = g_cfg;
        if (k == "nx") ss >> c.nx; else if (k == "ny") ss >> c.ny; else if (k == "nz") ss >> c.nz;
        else if (k == "dx") ss >> c.dx; else if (k == "dt") ss >> c.dt;
        else if (k == "nstep") ss >> c.nstep; else if (k == "sampgat") ss >> c.sampgat;
        else if (k == "it_output") ss >> c.it_output;
        else if (k == "ngatx") ss >> c.ngatx; else if (k == "ngaty") ss >> c.ngaty;
        else if (k == "npml") ss >> c.npml; else if (k == "npower") ss >> c.npower;
        else if (k == "k_max") ss >> c.k_max; else if (k == "alpha_max") ss >> c.alpha_max;
        else if (k == "rcoef") ss >> c.rcoef; else if (k == "vpml") ss >> c.vpml;
        else if (k == "f0") ss >> c.f0; else if (k == "t0") ss >> c.t0;
        else if (k == "factor") ss >> c.factor; else if (k == "angle") ss >> c.angle;
        else if (k == "src") ss >> c.src_i >> c.src_j >> c.src_k;
        else if (k == "src_kind") ss >> c.src_kind; else if (k == "stf") ss >> c.stf;
        else if (k == "w") ss >> c.w[0] >> c.w[1] >> c.w[2];
        else if (k == "clean") ss >> c.clean;
        else if (k == "time_from") ss >> c.time_from;
        else if (k == "model") ss >> c.model_prefix;
        else if (k == "rec") { int i, j, kk; ss >> i >> j >> kk; c.rec.push_back(i); c.rec.push_back(j); c.rec.push_back(kk); }
        else { fprintf(stderr, "unknown key %s\n", k.c_str()); exit(2); }
    }
    const int nrec = (int)g_cfg.rec.size() / 3;
    const int nsamp = g_cfg.nstep / g_cfg.sampgat;
    g_seis.assign((size_t)nrec * 3 * (nsamp > 0 ? nsamp : 0), 0.0);
}

template <class R>
static void ref_load_one(R *dst, const std::string &path, int NX, int NY, int NZ)
{
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) { fprintf(stderr, "cannot open %s\n", path.c_str()); exit(2); }
    std::vector<R> buf((size_t)NX * NY * NZ);
    if (fread(buf.data(), sizeof(R), buf.size(), f) != buf.size()) {
        fprintf(stderr, "short model file %s\n", path.c_str()); exit(2);
    }
    fclose(f);
    for (int k = 0; k < NZ; k++)
        for (int j = 0; j < NY; j++)
            for (int i = 0; i < NX; i++)
                dst[(i + 1) + (size_t)(j + 1) * NX + (size_t)(k + 1) * NX * NY] =
                    buf[i + (size_t)j * NX + (size_t)k * NX * NY];
}

template <class R>
static void ref_load_model(R *ccp, R *ccs, R *crho, int NX, int NY, int NZ)
{
    if (g_cfg.model_prefix.empty()) return;
    ref_load_one(ccp, g_cfg.model_prefix + "cp.bin", NX, NY, NZ);
    ref_load_one(ccs, g_cfg.model_prefix + "cs.bin", NX, NY, NZ);
    ref_load_one(crho, g_cfg.model_prefix + "rho.bin", NX, NY, NZ);
}

template <class R>
static void ref_record(int it, const R *vx, const R *vy, const R *vz, int NX, int NY)
{
    if (it % g_cfg.sampgat) return;
    const int nrec = (int)g_cfg.rec.size() / 3;
    const int nsamp = g_cfg.nstep / g_cfg.sampgat;
    const int s = it / g_cfg.sampgat - 1;
    if (s >= nsamp) return;
    for (int r = 0; r < nrec; r++) {
        const int *q = &g_cfg.rec[3 * r];
        size_t o = (q[0] + 1) + (size_t)(q[1] + 1) * NX + (size_t)(q[2] + 1) * NX * NY;
        g_seis[((size_t)r * 3 + 0) * nsamp + s] = vx[o];
        g_seis[((size_t)r * 3 + 1) * nsamp + s] = vy[o];
        g_seis[((size_t)r * 3 + 2) * nsamp + s] = vz[o];
    }
}

static void ref_step_hook(int it)
{
    if (it == g_cfg.time_from) g_t_first = ref_now();
    if (it == g_cfg.nstep + 1) g_t_last = ref_now();
}

template <class R>
static void ref_finish(R *vx, R *vy, R *vz, R *sxx, R *syy, R *szz, R *sxy, R *sxz,
                       R *syz, int NX, int NY, int NZ)
{
    {
        std::vector<R> s(g_seis.begin(), g_seis.end());
        FILE *f = fopen("seis.bin", "wb");
        if (f) { fwrite(s.data(), sizeof(R), s.size(), f); fclose(f); }
    }
    FILE *f = fopen("fields.bin", "wb");
    if (f) {
        R *fl[9] = {vx, vy, vz, sxx, syy, szz, sxy, sxz, syz};
        std::vector<R> buf((size_t)NX * NY * NZ);
        for (int c = 0; c < 9; c++) {
            for (int k = 0; k < NZ; k++)
                for (int j = 0; j < NY; j++)
                    for (int i = 0; i < NX; i++)
                        buf[i + (size_t)j * NX + (size_t)k * NX * NY] =
                            fl[c][(i + 1) + (size_t)(j + 1) * NX + (size_t)(k + 1) * NX * NY];
            fwrite(buf.data(), sizeof(R), buf.size(), f);
        }
        fclose(f);
    }
    FILE *t = fopen("steps.txt", "w");
    if (t) {
        fprintf(t, "%.9f %.9f %d\n", g_t_first, g_t_last, g_cfg.nstep - g_cfg.time_from + 1);
        fclose(t);
    }
}

#endif
