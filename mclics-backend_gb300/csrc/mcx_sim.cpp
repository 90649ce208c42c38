// mcx_sim.cpp -- the simulator driver behind mcx_run_file(): what
// ./mc_sim <paramfile> does in the reference (src/main.cpp:63-83,
// src/simulatorGPU.cpp:24-108, the run loops of src/evolve_{thermal,step,
// quench,electric}.cu), over the GB300 engine.  The loops, their float
// temperature stepping and the po.dat / director_field_*.csv formats follow
// the reference; sweeps, E, Q and S run on the GPU.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/mcx.h"
#include "mcx_host.h"

namespace mcx {
namespace {

std::string g_err;

struct Fail {
  mcx_status st;
};

int anch_code(const std::string &s) {
  static const char *names[] = {"homeotropic", "fg",      "rp",      "strong",
                                "homeotropic_ghrl", "fg_ghrl", "rp_ghrl", "strong_ghrl"};
  for (int i = 0; i < 8; i++)
    if (strcasecmp(s.c_str(), names[i]) == 0) return i;
  return -1;
}

bool ends_with_ci(const std::string &s, const char *suf, std::string &stem) {
  size_t n = strlen(suf);
  if (s.size() >= n && strcasecmp(s.c_str() + s.size() - n, suf) == 0) {
    stem = s.substr(0, s.size() - n);
    return true;
  }
  return false;
}

// print_n (src/io.cpp:50-80): x,y,z,nx,ny,nz,S,pt with S = nan on inactive sites.
// S: the per-site local order parameter computed on the GPU
// (mcx_local_order), or null for the initial-condition file, whose S column
// the reference writes as 1.
bool write_snapshot(const std::string &path, const std::vector<float> &ni, const std::vector<int> &pt,
                    const mcx_replica_desc &d, const float *S) {
  const bool with_S = S != nullptr;
  FILE *f = fopen(path.c_str(), "w");
  if (!f) return false;
  fprintf(f, with_S ? "x,y,z,nx,ny,nz,S,pt\n" : "x,y,z,nx,ny,nz,s,pt\n");
  for (int k = 0; k < d.nz; k++)
    for (int j = 0; j < d.ny; j++)
      for (int i = 0; i < d.nx; i++) {
        const long s = (long)i + (long)d.nx * ((long)j + (long)d.ny * k);
        if (with_S) {
          fprintf(f, "%d,%d,%d,%g,%g,%g,%g,%d\n", i, j, k, ni[3 * s], ni[3 * s + 1], ni[3 * s + 2], S[s], pt[s]);
        } else {
          fprintf(f, "%d,%d,%d,%g,%g,%g,1,%d\n", i, j, k, ni[3 * s], ni[3 * s + 1], ni[3 * s + 2], pt[s]);
        }
      }
  fclose(f);
  return true;
}

// read_ic_file (src/ic.cpp:88-119): header line, then x,y,z,nx,ny,nz rows.
bool read_ic_file(const std::string &path, const mcx_replica_desc &d, std::vector<float> &ni, std::string &err) {
  FILE *f = fopen(path.c_str(), "r");
  if (!f) {
    err = "cannot open ic_file " + path;
    return false;
  }
  char buf[512];
  if (!fgets(buf, sizeof buf, f)) {
    fclose(f);
    err = "empty ic_file";
    return false;
  }
  const long n = (long)d.nx * d.ny * d.nz;
  for (long q = 0; q < n; q++) {
    int x, y, z;
    float a, b, c;
    if (!fgets(buf, sizeof buf, f) || sscanf(buf, "%d,%d,%d,%f,%f,%f", &x, &y, &z, &a, &b, &c) != 6) {
      fclose(f);
      err = "malformed ic_file line " + std::to_string(q + 2);
      return false;
    }
    if (x < 0 || y < 0 || z < 0 || x >= d.nx || y >= d.ny || z >= d.nz) {
      fclose(f);
      err = "ic_file point out of the box at line " + std::to_string(q + 2);
      return false;
    }
    const long s = (long)x + (long)d.nx * ((long)y + (long)d.ny * z);
    ni[3 * s] = a;
    ni[3 * s + 1] = b;
    ni[3 * s + 2] = c;
  }
  fclose(f);
  return true;
}

// Reads and validates a parameter file into replica 0's descriptor, the
// custom mask (if any) and the mode index (0 thermal, 1 step, 2 quench,
// 3 electric).
mcx_status prepare(const char *path, SimParams &P, mcx_replica_desc &d, std::vector<int> &cpt, std::vector<float> &cns,
                   int &im) {
  std::string err;
  int rc = parse_param_file(path, P, err);
  if (rc) {
    g_err = err;
    return (mcx_status)rc;
  }
  memset(&d, 0, sizeof d);
  d.nx = P.Nx;
  d.ny = P.Ny;
  d.nz = P.Nz;
  if (strcasecmp(P.geometry.c_str(), "bulk") == 0) d.geometry = MCX_GEO_BULK;
  else if (strcasecmp(P.geometry.c_str(), "slab") == 0) d.geometry = MCX_GEO_SLAB;
  else if (strcasecmp(P.geometry.c_str(), "sphere") == 0) d.geometry = MCX_GEO_SPHERE;
  else if (strcasecmp(P.geometry.c_str(), "custom") == 0) d.geometry = MCX_GEO_CUSTOM;
  else {
    g_err = "geometry '" + P.geometry + "' not implemented. Options: bulk | slab | sphere | custom";
    return MCX_ERR_PARSE;
  }
  auto bound = [&](const std::string &s, int &out, const char *ax) {
    if (strcasecmp(s.c_str(), "free") == 0) out = MCX_BOUND_FREE;
    else if (strcasecmp(s.c_str(), "periodic") == 0) out = MCX_BOUND_PERIODIC;
    else {
      g_err = std::string(ax) + " boundary '" + s + "' not implemented. Options: free | periodic";
      return false;
    }
    return true;
  };
  if (!bound(P.xbound, d.xbound, "X") || !bound(P.ybound, d.ybound, "Y") || !bound(P.zbound, d.zbound, "Z"))
    return MCX_ERR_PARSE;
  if (strcasecmp(P.potential.c_str(), "ll") == 0 || strcasecmp(P.potential.c_str(), "lebwohl-lahser") == 0)
    d.potential = MCX_POT_LL;
  else if (strcasecmp(P.potential.c_str(), "ghrl") == 0 || strcasecmp(P.potential.c_str(), "grun-hess") == 0)
    d.potential = MCX_POT_GHRL;
  else if (strcasecmp(P.potential.c_str(), "pear") == 0)
    d.potential = MCX_POT_PEAR;
  else {
    g_err = "potential '" + P.potential + "' not implemented. Options: ll | ghrl | pear";
    return MCX_ERR_PARSE;
  }
  d.A = P.A;
  d.B1 = P.B1;
  d.C = P.C;
  d.k11 = P.k11;
  d.k22 = P.k22;
  d.k33 = P.k33;
  d.p0 = P.p0;
  d.elecA = P.elecA;
  d.elecX = P.elecX;
  d.elecY = P.elecY;
  d.elecZ = P.elecZ;
  d.elecE = P.elecE;
  d.T = P.Ti;
  d.ang_var = 0.5f;  // src/evolve_thermal.cpp:36
  d.radius = P.radius;
  int nsurf = d.geometry == MCX_GEO_SLAB ? 2 : d.geometry == MCX_GEO_SPHERE ? 1 : 0;
  if (d.geometry == MCX_GEO_CUSTOM) {
    nsurf = read_custom_geometry(P.bound_file.c_str(), d.nx, d.ny, d.nz, cpt, cns, err);
    if (nsurf < 0) {
      g_err = err;
      return MCX_ERR_PARSE;
    }
  }
  if (nsurf > MCX_MAX_SURFACES) {
    g_err = "more than 16 surfaces";
    return MCX_ERR_UNSUPPORTED;
  }
  d.n_surfaces = nsurf;
  for (int s = 0; s < nsurf; s++) {  // Geometry::Boundary_Init (src/geometry.cpp:73-103)
    if (!P.anchoring_type.count(s)) {
      g_err = "you must define " + std::to_string(nsurf) + " boundaries (anchoring_type " + std::to_string(s) + " missing)";
      return MCX_ERR_PARSE;
    }
    const int a = anch_code(P.anchoring_type[s]);
    if (a < 0) {
      g_err = P.anchoring_type[s] + " boundary condition is not defined";
      return MCX_ERR_PARSE;
    }
    d.anchoring[s] = a;
    if (!P.W.count(s)) {
      g_err = "parameter W not defined for boundary condition #" + std::to_string(s);
      return MCX_ERR_PARSE;
    }
    d.W[s] = P.W[s];
    const bool needs_axis = a == MCX_ANCH_RP || a == MCX_ANCH_STRONG || a == MCX_ANCH_RP_GHRL || a == MCX_ANCH_STRONG_GHRL;
    if (needs_axis && (!P.phi_s.count(s) || !P.theta_s.count(s))) {
      g_err = "parameters phi_s/theta_s not defined for boundary condition #" + std::to_string(s);
      return MCX_ERR_PARSE;
    }
    d.phi_s[s] = P.phi_s.count(s) ? P.phi_s[s] : 0.f;
    d.theta_s[s] = P.theta_s.count(s) ? P.theta_s[s] : 0.f;
  }
  std::string stem, mode = P.evol;
  if (ends_with_ci(mode, "GPU", stem) || ends_with_ci(mode, "GB300", stem)) mode = stem;
  const char *modes[] = {"thermal", "step", "quench", "electric"};
  im = -1;
  for (int q = 0; q < 4; q++)
    if (strcasecmp(mode.c_str(), modes[q]) == 0) im = q;
  if (im < 0) {
    g_err = "evol mode '" + P.evol + "' not implemented. Options: thermal | step | quench | electric (GPU / GB300 suffix accepted)";
    return MCX_ERR_PARSE;
  }
  {
    // bounds as the geometry forces them (src/geometry_slab.cpp:23,
    // src/geometry_sphere.cpp:19-21); red/black sweeps need even lengths on
    // periodic axes, free axes may have any length
    const bool sph = d.geometry == MCX_GEO_SPHERE;
    const int xb = sph ? MCX_BOUND_FREE : d.xbound, yb = sph ? MCX_BOUND_FREE : d.ybound;
    const int zb = sph || d.geometry == MCX_GEO_SLAB ? MCX_BOUND_FREE : d.zbound;
    const char *ax = (xb == MCX_BOUND_PERIODIC && d.nx % 2) ? "Nx"
                     : (yb == MCX_BOUND_PERIODIC && d.ny % 2) ? "Ny"
                     : (zb == MCX_BOUND_PERIODIC && d.nz % 2) ? "Nz"
                                                              : nullptr;
    if (ax) {
      g_err = std::string(ax) + " is odd on a periodic axis (" + std::to_string(d.nx) + "x" + std::to_string(d.ny) +
              "x" + std::to_string(d.nz) + "); red/black sweeps need even lengths on periodic axes";
      return MCX_ERR_UNSUPPORTED;
    }
  }
  if (im == 0 && P.dT == 0) {
    g_err = "dT must be non-zero";
    return MCX_ERR_PARSE;
  }
  if (im == 3 && P.elecdE == 0) {
    g_err = "dE must be non-zero";
    return MCX_ERR_PARSE;
  }
  if (P.replicas < 1) {
    g_err = "replicas must be >= 1";
    return MCX_ERR_PARSE;
  }
  return MCX_OK;
}

mcx_status run(const char *path, const char *out_dir) {
  SimParams P;
  mcx_replica_desc d;
  std::vector<int> cpt;
  std::vector<float> cns;
  int im;
  std::string err;
  if (mcx_status st = prepare(path, P, d, cpt, cns, im)) return st;
  const std::string dir = out_dir ? std::string(out_dir) + "/" : std::string();
  const int R = P.replicas > 0 ? P.replicas : 1;
  std::vector<mcx_replica_desc> descs(R, d);
  for (int r = 0; r < R; r++) {
    descs[r].seed = (unsigned)(P.seed + r);
    descs[r].stream = (unsigned)r;
  }
  mcx_engine *e = nullptr;
  mcx_status st = mcx_create(R, descs.data(), &e);
  if (st) {
    g_err = mcx_last_error(nullptr);
    return st;
  }
  struct Guard {
    mcx_engine *e;
    ~Guard() { mcx_destroy(e); }
  } guard{e};
  auto check = [&](mcx_status s) {
    if (s) {
      g_err = mcx_last_error(e);
      throw Fail{s};
    }
  };
  const long nsites = (long)d.nx * d.ny * d.nz;
  std::vector<float> ni(3 * nsites), S(nsites);
  std::vector<int> pt(nsites);
  std::vector<float> ns(3 * nsites);
  try {
    for (int r = 0; r < R; r++) {
      if (d.geometry == MCX_GEO_CUSTOM) check(mcx_set_mask(e, r, cpt.data(), cns.data()));
      if (strcasecmp(P.ic.c_str(), "random") == 0) {
        check(mcx_init_random(e, r, descs[r].seed));
      } else if (strcasecmp(P.ic.c_str(), "homogeneous") == 0) {
        check(mcx_init_homogeneous(e, r, P.theta_0, P.phi_0));
      } else if (strcasecmp(P.ic.c_str(), "ic_file") == 0) {
        std::fill(ni.begin(), ni.end(), 0.f);
        if (!read_ic_file(P.ic_file, d, ni, err)) {
          g_err = err;
          return MCX_ERR_PARSE;
        }
        check(mcx_set_state(e, r, ni.data()));
      } else if (strcasecmp(P.ic.c_str(), "cholesteric") == 0) {  // src/ic.cpp:121-151
        check(mcx_get_mask(e, r, pt.data(), ns.data()));
        const float theta = P.theta_0;
        const float phi0 = (float)(P.phi_0 * M_PI / 180);
        const float p0 = P.p0_i != 0 ? P.p0_i : P.p0;
        for (int k = 0; k < d.nz; k++)
          for (int j = 0; j < d.ny; j++)
            for (int i = 0; i < d.nx; i++) {
              const long s = (long)i + (long)d.nx * ((long)j + (long)d.ny * k);
              if (pt[s]) {
                const float phi = (float)(phi0 - 2 * M_PI * k / p0);
                ni[3 * s] = (float)(sin(theta * M_PI / 180) * cos(phi));
                ni[3 * s + 1] = (float)(sin(theta * M_PI / 180) * sin(phi));
                ni[3 * s + 2] = (float)cos(theta * M_PI / 180);
              } else {
                ni[3 * s] = 0;
                ni[3 * s + 1] = 0;
                ni[3 * s + 2] = 1;
              }
            }
        check(mcx_set_state(e, r, ni.data()));
      } else {
        g_err = "initial condition '" + P.ic + "' not implemented. Options: random | homogeneous | ic_file | cholesteric";
        return MCX_ERR_PARSE;
      }
    }
    check(mcx_get_mask(e, 0, pt.data(), ns.data()));
    check(mcx_get_state(e, 0, ni.data()));
    write_snapshot(dir + "ic.csv", ni, pt, descs[0], nullptr);
    // po.dat per replica (po_r<r>.dat for r > 0) and, with several replicas,
    // po_avg.dat: their combination by mcx_combine_stats, the table
    // average_replicas.py would write from those files
    const int nfiles = R > 1 ? R + 1 : 1;
    std::vector<FILE *> po(nfiles, nullptr);
    for (int r = 0; r < nfiles; r++) {
      std::string name = r == 0 ? dir + "po.dat"
                         : r == R ? dir + "po_avg.dat"
                                  : dir + "po_r" + std::to_string(r) + ".dat";
      po[r] = fopen(name.c_str(), "a");
      if (!po[r]) {
        g_err = "cannot open " + name;
        for (FILE *f : po)
          if (f) fclose(f);
        return MCX_ERR_IO;
      }
      // Pear runs add the polarization of the block's final state
      // (src/evolve_thermal.cpp:50-53,82-84)
      const char *cols = descs[0].potential == MCX_POT_PEAR ? " S varS E varE P\n" : " S varS E varE\n";
      fprintf(po[r], "%s%s", im == 0 || im == 3 ? "T" : "ii", cols);
      fflush(po[r]);
    }
    struct PoGuard {
      std::vector<FILE *> &v;
      ~PoGuard() {
        for (FILE *f : v)
          if (f) fclose(f);
      }
    } pog{po};
    double stt[MCX_STATS_LEN];
    // one block: MCT thermalisation sweeps, MCS measured sweeps, a po.dat row
    auto block = [&](int n_therm, const char *label_fmt, double label, int ilabel, const std::string &snap) {
      check(mcx_sweep(e, n_therm, 0));
      check(mcx_reset_stats(e, -1));
      check(mcx_sweep(e, P.MCS, 1));
      for (int r = 0; r < R; r++) {
        check(mcx_get_stats(e, r, stt));
        const double n = stt[MCX_ST_N] > 0 ? stt[MCX_ST_N] : 1;
        const double S1 = stt[MCX_ST_S1] / n, S2 = stt[MCX_ST_S2] / n;
        const double E = stt[MCX_ST_E1] / n, E2 = stt[MCX_ST_E2] / n;
        if (label_fmt[1] == 'd')
          fprintf(po[r], "%d %g %g %g %g", ilabel, S1, S2 - S1 * S1, E, E2 - E * E);
        else
          fprintf(po[r], "%g %g %g %g %g", label, S1, S2 - S1 * S1, E, E2 - E * E);
        if (descs[0].potential == MCX_POT_PEAR) {
          double Pz = 0;
          check(mcx_polarization(e, r, &Pz));
          fprintf(po[r], " %g", (float)Pz);
        }
        fprintf(po[r], "\n");
        fflush(po[r]);
      }
      if (R > 1) {
        double cb[MCX_COMBINED_LEN];
        check(mcx_combine_stats(e, 0, nullptr, cb));
        FILE *f = po[R];
        if (label_fmt[1] == 'd')
          fprintf(f, "%d", ilabel);
        else
          fprintf(f, "%g", label);
        fprintf(f, " %g %g %g %g", cb[MCX_CB_S], cb[MCX_CB_VAR_S], cb[MCX_CB_E], cb[MCX_CB_VAR_E]);
        if (descs[0].potential == MCX_POT_PEAR) fprintf(f, " %g", cb[MCX_CB_P]);
        fprintf(f, "\n");
        fflush(f);
      }
      if (!snap.empty()) {
        check(mcx_get_state(e, 0, ni.data()));
        check(mcx_local_order(e, 0, S.data()));
        write_snapshot(snap, ni, pt, descs[0], S.data());
      }
    };
    const bool snapshots = getenv("MCX_NO_SNAPSHOTS") == nullptr;
    if (im == 0) {  // thermal (src/evolve_thermal.cu:79-110)
      if (P.dT == 0) {
        g_err = "dT must be non-zero";
        return MCX_ERR_PARSE;
      }
      const int sign = (int)(-P.dT / fabsf(P.dT));
      for (float T = P.Ti; (int)1e6 * sign * (T - P.Tf) >= 0; T += P.dT) {
        check(mcx_set_temperature(e, -1, T));
        std::string snap = snapshots ? dir + "director_field_" + std::to_string((int)(100 * (T + 1e-7))) + ".csv" : "";
        block(P.MCT, "%g", T, 0, snap);
      }
    } else if (im == 3) {  // electric (src/evolve_electric.cpp:59-90)
      if (P.elecdE == 0) {
        g_err = "dE must be non-zero";
        return MCX_ERR_PARSE;
      }
      check(mcx_set_temperature(e, -1, P.Ti));
      const int sign = (int)(-P.elecdE / fabsf(P.elecdE));
      for (float E = P.elecEi; (int)1e6 * sign * (E - P.elecEf) >= 0; E += P.elecdE) {
        check(mcx_set_field(e, -1, E));
        std::string snap = snapshots ? dir + "director_field_" + std::to_string((int)(100 * (E + 1e-7))) + ".csv" : "";
        block(P.MCT, "%g", E, 0, snap);
      }
    } else {  // step / quench (src/evolve_step.cpp:58-90, src/evolve_quench.cpp:58-94)
      check(mcx_set_temperature(e, -1, P.Ti));
      for (int ii = P.first_file; ii < P.fn + P.first_file; ii++) {
        int n_therm = P.MCT;
        if (im == 2) {
          check(mcx_set_temperature(e, -1, P.Ti));
          check(mcx_sweep(e, P.MCT, 0));
          check(mcx_set_temperature(e, -1, P.Tf));
          n_therm = 0;
          for (int step = 0; step < P.MCT * P.dT; step++) n_therm++;  // MCT*dT sweeps (float bound)
        }
        std::string snap = snapshots ? dir + "director_field_" + std::to_string(ii) + ".csv" : "";
        block(n_therm, "%d", 0, ii, snap);
      }
    }
  } catch (const Fail &f) {
    return f.st;
  }
  return MCX_OK;
}

}  // namespace
}  // namespace mcx

extern "C" mcx_status mcx_run_file(const char *param_file, const char *out_dir) {
  if (!param_file) {
    mcx::set_last_error("mcx_run_file: null parameter file");
    return MCX_ERR_INVALID;
  }
  mcx::g_err.clear();
  mcx_status st = mcx::run(param_file, out_dir);
  if (st) mcx::set_last_error(mcx::g_err.c_str());
  return st;
}

extern "C" mcx_status mcx_check_file(const char *param_file, mcx_replica_desc *desc) {
  if (!param_file) {
    mcx::set_last_error("mcx_check_file: null parameter file");
    return MCX_ERR_INVALID;
  }
  mcx::g_err.clear();
  mcx::SimParams P;
  mcx_replica_desc d;
  std::vector<int> cpt;
  std::vector<float> cns;
  int im;
  mcx_status st = mcx::prepare(param_file, P, d, cpt, cns, im);
  if (st) {
    mcx::set_last_error(mcx::g_err.c_str());
    return st;
  }
  if (desc) *desc = d;
  return MCX_OK;
}

extern "C" mcx_status mcx_print_n(mcx_engine *e, int r, const char *path) {
  if (!e || !path) {
    mcx::set_last_error("mcx_print_n: null engine or path");
    return MCX_ERR_INVALID;
  }
  mcx_replica_desc d;
  if (mcx_status st = mcx_get_desc(e, r, &d, nullptr)) return st;
  const long n = (long)d.nx * d.ny * d.nz;
  std::vector<float> ni(3 * n), ns(3 * n), S(n);
  std::vector<int> pt(n);
  if (mcx_status st = mcx_get_state(e, r, ni.data())) return st;
  if (mcx_status st = mcx_get_mask(e, r, pt.data(), ns.data())) return st;
  if (mcx_status st = mcx_local_order(e, r, S.data())) return st;
  if (!mcx::write_snapshot(path, ni, pt, d, S.data())) {
    mcx::set_engine_error(e, (std::string("mcx_print_n: cannot write ") + path).c_str());
    return MCX_ERR_IO;
  }
  return MCX_OK;
}
