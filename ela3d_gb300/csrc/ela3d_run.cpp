// ela3d_run -- the drop-in for the reference program's main(): runs one shot
// on the GPU through the C ABI (include/ela3d.h) from a parameter file and
// writes the reference program's own output files.  Host code only; links
// against libela3d.so.
//
//   ela3d_run params.txt [--outdir DIR] [--fp64]
//
// params.txt holds "key value" lines with the reference's parameter names
// (the locals of seismicCPML_3d_isotropic_simpelmodel.cpp:19-78): nx ny nz,
// dx (one spacing, DELTAX), dt, nstep, sampgat, it_output, ngatx ngaty
// (receiver text layout), npml, npower, k_max, alpha_max, rcoef, vpml, f0,
// t0, factor, angle, "src i j k" (0-based), src_kind (0 force, 1
// explosive), stf (0 Ricker, 1 Gaussian derivative, 2 Gaussian),
// "w wx wy wz", clean (0/1 profile variant), energy_every, model PREFIX
// (PREFIXcp.bin, PREFIXcs.bin, PREFIXrh.bin, float32 x fastest; without it
// the reference's constant medium cp 3300, cs 3300/1.732, rho 3000), and
// optional "rec i j k" lines; any other key is an error.  Keys and defaults
// are those of the Python runner (python -m ela3d_gb300 run), so both read
// the same file alike.
//
// Outputs, in the layouts of the reference's programs:
//   rechorvx.txt rechorvy.txt rechorvz.txt  when ngatx and ngaty are given:
//       plane KSOURCE+1 (1-based) subsampled as the program prints it
//       (simpelmodel.cpp:593-602,625-671), values as iostream prints them
//       (6 significant digits), each followed by a space, one line per sample;
//   vz%05i.bin vy%05i.bin vx%05i.bin  every it_output steps (:673-725): the
//       program's (NIMX+1)(NIMY+1)(NIMZ+1) values read with pitch NIMX, each
//       address mapped to its cell or to a never-written zero; float64 with
//       --fp64;
//   recsrcx.txt recsrcy.txt recsrcz.txt  the source-point trace of the FP64
//       GPU program (elatic_3d_unified_cuda_memory.cu:1202-1223);
//   seis.bin  the "rec" receivers, float32 [nrec][3][nstep/sampgat].
// Exit status 0 on success, 1 on bad input, 2 when the library reports an
// error (its message on stderr).
#include <algorithm>
#include <iterator>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/ela3d.h"

namespace {

struct Args {
  std::string params, outdir = ".";
  bool fp64 = false;
};

struct Input {
  ela3d_params p{};
  std::vector<int32_t> rec;
  int ngatx = 0, ngaty = 0;
  std::string model;
};

bool fail(const std::string &msg) {
  std::fprintf(stderr, "ela3d_run: %s\n", msg.c_str());
  return false;
}

bool parse(const std::string &path, Input *in) {
  std::ifstream f(path);
  if (!f) return fail("cannot open " + path);
  std::map<std::string, std::vector<std::string>> kv;
  std::vector<int32_t> rec;
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream ss(line);
    std::string k;
    if (!(ss >> k) || k[0] == '#') continue;
    std::vector<std::string> v;
    for (std::string t; ss >> t;) v.push_back(t);
    static const char *const kKeys[] = {"nx", "ny", "nz", "dx", "dt", "nstep", "sampgat", "it_output", "ngatx",
                                        "ngaty", "npml", "npower", "k_max", "alpha_max", "rcoef", "vpml", "f0",
                                        "t0", "factor", "angle", "src", "src_kind", "stf", "w", "clean",
                                        "energy_every", "model", "rec"};
    if (std::none_of(std::begin(kKeys), std::end(kKeys), [&](const char *q) { return k == q; }))
      return fail(path + ": unknown key " + k);
    if (k == "rec") {
      if (v.size() < 3) return fail("rec needs i j k");
      for (int q = 0; q < 3; ++q) rec.push_back(std::atoi(v[q].c_str()));
    } else {
      kv[k] = v;
    }
  }
  auto num = [&](const char *k, double d) { return kv.count(k) && !kv[k].empty() ? std::atof(kv[k][0].c_str()) : d; };
  auto integer = [&](const char *k, int d) { return kv.count(k) && !kv[k].empty() ? std::atoi(kv[k][0].c_str()) : d; };
  ela3d_params &p = in->p;
  std::memset(&p, 0, sizeof p);
  p.nx = integer("nx", 32);
  p.ny = integer("ny", 32);
  p.nz = integer("nz", 32);
  p.nstep = integer("nstep", 10);
  p.dx = p.dy = p.dz = num("dx", 10.0);
  p.dt = num("dt", 1e-3);
  p.npml = integer("npml", 10);
  p.pml_mode = integer("clean", 0);
  p.npower = num("npower", 2.0);
  p.k_max = num("k_max", 1.0);
  p.alpha_max = num("alpha_max", -1.0);
  p.rcoef = num("rcoef", 1e-3);
  p.vpml = num("vpml", 3000.0);
  p.f0 = num("f0", 7.0);
  p.t0 = num("t0", 1.2 / 7.0);
  p.factor = num("factor", 1e7);
  p.stf = integer("stf", 0);
  p.src_kind = integer("src_kind", 0);
  p.src_i = p.src_j = p.src_k = 16;
  if (kv.count("src")) {
    if (kv["src"].size() < 3) return fail("src needs i j k");
    p.src_i = std::atoi(kv["src"][0].c_str());
    p.src_j = std::atoi(kv["src"][1].c_str());
    p.src_k = std::atoi(kv["src"][2].c_str());
  }
  p.sampgat = integer("sampgat", 1);
  p.src_w[0] = 0.0;
  p.src_w[1] = 0.0;
  p.src_w[2] = 1.0;
  if (kv.count("w")) {
    if (kv["w"].size() < 3) return fail("w needs wx wy wz");
    for (int q = 0; q < 3; ++q) p.src_w[q] = std::atof(kv["w"][q].c_str());
  }
  p.angle_force = num("angle", 0.0);
  p.it_output = integer("it_output", 0);
  p.energy_every = integer("energy_every", 0);
  in->ngatx = integer("ngatx", 0);
  in->ngaty = integer("ngaty", 0);
  if (kv.count("model") && !kv["model"].empty()) in->model = kv["model"][0];
  in->rec = rec;
  if (p.nx < 1 || p.ny < 1 || p.nz < 1) return fail("nx, ny, nz must be positive");
  return true;
}

bool read_model(const std::string &prefix, size_t n, std::vector<float> *m) {
  static const char *kNames[3] = {"cp", "cs", "rh"};
  for (int c = 0; c < 3; ++c) {
    const std::string path = prefix + kNames[c] + ".bin";
    FILE *fp = std::fopen(path.c_str(), "rb");
    if (!fp) return fail("cannot open " + path);
    m[c].resize(n);
    const size_t got = std::fread(m[c].data(), sizeof(float), n, fp);
    std::fclose(fp);
    if (got != n) return fail("short model file " + path);
  }
  return true;
}

// Cells of the receiver text (simpelmodel.cpp:593-602,629-670): the program
// prints buffer entries kk = i + j*NIMX for i = 0, xlen, ... <= NIMX and
// j = 0, ylen, ... <= NIMY (xlen = NIMX/Ngatx, ylen = (NIMY - 2 NPOINTS_PML)
// / Ngaty); entry kk is 1-based cell ((kk-1) % NIMX + 1, (kk-1) / NIMX) of
// plane KSOURCE+1 when that row lies in [1, NIMY], else a never-written 0.
// Returns the distinct cells (0-based i j k triples) and, per printed value,
// the index of its cell or -1.
bool gather_layout(const ela3d_params &p, int ngatx, int ngaty, std::vector<int32_t> *cells,
                   std::vector<int> *slots) {
  const int xlen = p.nx / ngatx, ylen = (p.ny - 2 * p.npml) / ngaty;
  if (xlen <= 0 || ylen <= 0) return fail("more receivers than grid cells (the reference program stops here)");
  const int k = p.src_k + 1;
  std::map<std::pair<int, int>, int> index;
  for (int j = 0; j <= p.ny; j += ylen)
    for (int i = 0; i <= p.nx; i += xlen) {
      const long long kk = i + (long long)j * p.nx;
      if (kk >= 1) {
        const int i1 = (int)((kk - 1) % p.nx) + 1, j1 = (int)((kk - 1) / p.nx);
        if (j1 >= 1 && j1 <= p.ny) {
          const std::pair<int, int> key(i1 - 1, j1 - 1);
          auto it = index.find(key);
          if (it == index.end()) {
            it = index.emplace(key, (int)(cells->size() / 3)).first;
            cells->push_back(i1 - 1);
            cells->push_back(j1 - 1);
            cells->push_back(k);
          }
          slots->push_back(it->second);
          continue;
        }
      }
      slots->push_back(-1);
    }
  return true;
}

// A value as C++ iostreams print a float or double by default (%g, 6 digits).
void put(FILE *fp, double v) { std::fprintf(fp, "%g ", v); }

bool write_rechor(const std::string &dir, const std::vector<float> &seis, int ncells, int nsamp,
                  const std::vector<int> &slots) {
  static const char *kNames[3] = {"rechorvx.txt", "rechorvy.txt", "rechorvz.txt"};
  for (int c = 0; c < 3; ++c) {
    const std::string path = dir + "/" + kNames[c];
    FILE *fp = std::fopen(path.c_str(), "w");
    if (!fp) return fail("cannot write " + path);
    for (int s = 0; s < nsamp; ++s) {
      for (int q : slots) {
        if (q < 0) std::fputs("0 ", fp);
        else put(fp, seis[((size_t)q * 3 + c) * nsamp + s]);
      }
      std::fputc('\n', fp);
    }
    std::fclose(fp);
  }
  (void)ncells;
  return true;
}

template <typename T>
bool write_recsrc(const std::string &dir, const std::vector<T> &trace, int nstep) {
  static const char *kNames[3] = {"recsrcx.txt", "recsrcy.txt", "recsrcz.txt"};
  for (int c = 0; c < 3; ++c) {
    const std::string path = dir + "/" + kNames[c];
    FILE *fp = std::fopen(path.c_str(), "w");
    if (!fp) return fail("cannot write " + path);
    for (int s = 0; s <= nstep; ++s) put(fp, (double)trace[(size_t)c * (nstep + 1) + s]);
    std::fclose(fp);
  }
  return true;
}

// v?%05i.bin (simpelmodel.cpp:685-722): the program writes (NIMX+1)(NIMY+1)
// (NIMZ+1) values at addresses ii + jj*NIMX + kk*NIMX*NIMY of arrays that
// hold 1-based cell (i, j, k) at i + j*NIMX + k*NIMX*NIMY; an address maps to
// the cell ((a-1) % NIMX + 1, ...) where row 0 of a plane is row NIMY of the
// plane below, or to a never-written zero.
template <typename T>
bool write_snapshot(const std::string &path, const std::vector<T> &field, int nx, int ny, int nz) {
  FILE *fp = std::fopen(path.c_str(), "wb");
  if (!fp) return fail("cannot write " + path);
  std::vector<T> row((size_t)nx + 1);
  for (long long kk = 0; kk <= nz; ++kk)
    for (long long jj = 0; jj <= ny; ++jj) {
      for (long long ii = 0; ii <= nx; ++ii) {
        const long long a = ii + jj * nx + kk * (long long)nx * ny;
        T v = T(0);
        if (a >= 1) {
          const long long b = a - 1;
          const long long i1 = b % nx + 1, q = b / nx;
          long long j1 = q % ny, k1 = q / ny;
          if (j1 == 0) { j1 = ny; k1 -= 1; }
          if (k1 >= 1 && k1 <= nz) v = field[((k1 - 1) * ny + (j1 - 1)) * nx + (i1 - 1)];
        }
        row[(size_t)ii] = v;
      }
      if (std::fwrite(row.data(), sizeof(T), row.size(), fp) != row.size()) {
        std::fclose(fp);
        return fail("short write " + path);
      }
    }
  std::fclose(fp);
  return true;
}

template <typename T>
bool snapshots(ela3d_plan *plan, const std::string &dir, int it, const ela3d_params &p) {
  static const int kComps[3] = {ELA3D_VZ, ELA3D_VY, ELA3D_VX};
  static const char *kNames[3] = {"vz", "vy", "vx"};
  std::vector<T> f((size_t)p.nx * p.ny * p.nz);
  for (int c = 0; c < 3; ++c) {
    ela3d_status st;
    if constexpr (sizeof(T) == 8) st = ela3d_get_field_f64(plan, kComps[c], f.data());
    else st = ela3d_get_field(plan, kComps[c], f.data());
    if (st != ELA3D_OK) return fail(std::string("ela3d_get_field: ") + ela3d_last_error());
    char name[32];
    std::snprintf(name, sizeof name, "%s%05i.bin", kNames[c], it);
    if (!write_snapshot(dir + "/" + name, f, p.nx, p.ny, p.nz)) return false;
  }
  return true;
}

int run(const Args &a) {
  Input in;
  if (!parse(a.params, &in)) return 1;
  ela3d_params p = in.p;
  p.precision = a.fp64 ? ELA3D_FP64 : ELA3D_FP32;
  const size_t n = (size_t)p.nx * p.ny * p.nz;
  std::vector<float> m[3];
  if (!in.model.empty()) {
    if (!read_model(in.model, n, m)) return 1;
  } else {
    m[0].assign(n, 3300.0f);
    m[1].assign(n, (float)(3300.0 / 1.732));
    m[2].assign(n, 3000.0f);
  }
  std::vector<int32_t> cells;
  std::vector<int> slots;
  const bool text = in.ngatx > 0 && in.ngaty > 0;
  if (text && !gather_layout(p, in.ngatx, in.ngaty, &cells, &slots)) return 1;
  const int ncells = (int)(cells.size() / 3);
  std::vector<int32_t> rec = cells;
  rec.insert(rec.end(), in.rec.begin(), in.rec.end());
  p.rec = rec.empty() ? nullptr : rec.data();
  p.nrec = (int32_t)(rec.size() / 3);

  ela3d_plan *plan = nullptr;
  ela3d_status st = ela3d_plan_create(&p, m[0].data(), m[1].data(), m[2].data(), &plan);
  if (st != ELA3D_OK) {
    std::fprintf(stderr, "ela3d_run: ela3d_plan_create: %s (%s)\n", ela3d_status_string(st), ela3d_last_error());
    return st == ELA3D_ERR_INVALID_ARG ? 1 : 2;
  }
  int rc = 0;
  const int chunk = p.it_output > 0 ? p.it_output : p.nstep;
  for (int done = 0; done < p.nstep && rc == 0;) {
    const int steps = std::min(chunk, p.nstep - done);
    st = ela3d_run(plan, steps);
    if (st != ELA3D_OK) {
      std::fprintf(stderr, "ela3d_run: ela3d_run: %s (%s)\n", ela3d_status_string(st), ela3d_last_error());
      rc = 2;
      break;
    }
    done += steps;
    if (p.it_output > 0 && done % p.it_output == 0) {
      const bool ok = a.fp64 ? snapshots<double>(plan, a.outdir, done, p) : snapshots<float>(plan, a.outdir, done, p);
      if (!ok) rc = 2;
    }
  }
  const int nsamp = p.nstep / p.sampgat;
  if (rc == 0) {
    std::vector<float> seis((size_t)p.nrec * 3 * nsamp);
    if (!seis.empty() && (st = ela3d_get_seismograms(plan, seis.data())) != ELA3D_OK) {
      std::fprintf(stderr, "ela3d_run: ela3d_get_seismograms: %s\n", ela3d_last_error());
      rc = 2;
    }
    bool ok = rc == 0;
    if (ok && a.fp64) {
      std::vector<double> trace((size_t)3 * (p.nstep + 1));
      ok = ela3d_get_source_trace_f64(plan, trace.data()) == ELA3D_OK && write_recsrc(a.outdir, trace, p.nstep);
    } else if (ok) {
      std::vector<float> trace((size_t)3 * (p.nstep + 1));
      ok = ela3d_get_source_trace(plan, trace.data()) == ELA3D_OK && write_recsrc(a.outdir, trace, p.nstep);
    }
    if (ok && text) ok = write_rechor(a.outdir, seis, ncells, nsamp, slots);
    if (ok && !in.rec.empty()) {
      const std::string path = a.outdir + "/seis.bin";
      FILE *fp = std::fopen(path.c_str(), "wb");
      const size_t off = (size_t)ncells * 3 * nsamp, cnt = seis.size() - off;
      ok = fp && std::fwrite(seis.data() + off, sizeof(float), cnt, fp) == cnt;
      if (fp) std::fclose(fp);
    }
    if (!ok && rc == 0) rc = 2;
  }
  ela3d_plan_destroy(plan);
  return rc;
}

}  // namespace

int main(int argc, char **argv) {
  Args a;
  for (int q = 1; q < argc; ++q) {
    const std::string s = argv[q];
    if (s == "--outdir" && q + 1 < argc) a.outdir = argv[++q];
    else if (s == "--fp64") a.fp64 = true;
    else if (a.params.empty() && s[0] != '-') a.params = s;
    else {
      std::fprintf(stderr, "usage: ela3d_run params.txt [--outdir DIR] [--fp64]\n");
      return 1;
    }
  }
  if (a.params.empty()) {
    std::fprintf(stderr, "usage: ela3d_run params.txt [--outdir DIR] [--fp64]\n");
    return 1;
  }
  return run(a);
}
