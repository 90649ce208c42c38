// mcx_host.cpp -- host-side setup: GHRL constants, anchoring axes, geometry
// masks, custom geometry files and the parameter-file reader.  Compiled with
// -ffp-contract=off so that the float arithmetic rounds the same way on every
// host.
#include "mcx_host.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include <algorithm>
#include <fstream>
#include <sstream>

namespace mcx {

void ghrl_constants(float k11, float k22, float k33, float p0, float out[5]) {
  // src/io.cpp:281-288
  float Scale = (float)fabs(9.0 / (double)(k11 - 3 * k22 - k33));
  float sigma = p0 != 0 ? (float)((double)(-Scale * k22) * (2 * M_PI / (double)p0)) : 0.0f;
  float lambda = (Scale / 9) * (2 * k11 - 3 * k22 + k33);
  float mu = Scale * (k22 - k11);
  float rho = (Scale / 9) * (k11 - k33);
  float nu = (Scale / 9) * (k11 - 3 * k22 - k33);
  out[0] = lambda;
  out[1] = mu;
  out[2] = nu;
  out[3] = rho;
  out[4] = sigma;
}

void anchoring_axis(float theta_s, float phi_s, float out[3]) {
  const float toPi = (float)(M_PI / 180);
  const double th = (double)(toPi * theta_s), ph = (double)(toPi * phi_s);
  out[0] = (float)(cos(ph) * sin(th));
  out[1] = (float)(sin(ph) * sin(th));
  out[2] = (float)cos(th);
}

bool build_mask(const mcx_replica_desc &d, std::vector<int> &pt, std::vector<float> &ns) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const long n = (long)nx * ny * nz;
  pt.assign(n, 1);
  ns.assign(3 * n, 0.f);
  if (d.geometry == MCX_GEO_BULK) return true;
  if (d.geometry == MCX_GEO_CUSTOM) return false;
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        const long s = (long)i + (long)nx * ((long)j + (long)ny * k);
        if (d.geometry == MCX_GEO_SLAB) {
          if (k == nz - 1) {
            pt[s] = 3;
            ns[3 * s + 2] = 1.f;
          } else if (k == 0) {
            pt[s] = 2;
            ns[3 * s + 2] = -1.f;
          }
        } else {  // sphere
          const float Hx = (float)(nx / 2), Hy = (float)(ny / 2), Hz = (float)(nz / 2);
          const float R = d.radius > 0 ? d.radius : Hz;
          const float Rx = (float)i - Hx, Ry = (float)j - Hy, Rz = (float)k - Hz;
          const float r = sqrtf(Rx * Rx + Ry * Ry + Rz * Rz);
          if (r < R - 1) {
            pt[s] = 1;
          } else if (r < R + 1) {
            pt[s] = 2;
            ns[3 * s] = Rx / r;
            ns[3 * s + 1] = Ry / r;
            ns[3 * s + 2] = Rz / r;
          } else {
            pt[s] = 0;
          }
        }
      }
  return true;
}

static std::vector<std::string> split_csv(const std::string &line) {
  std::vector<std::string> out;
  std::string cur;
  for (char ch : line) {
    if (ch == ',' || ch == '\n' || ch == '\r') {
      out.push_back(cur);
      cur.clear();
    } else if (ch != ' ' && ch != '\t') {
      cur.push_back(ch);
    }
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

int read_custom_geometry(const char *path, int nx, int ny, int nz, std::vector<int> &pt, std::vector<float> &ns,
                         std::string &err) {
  std::ifstream f(path);
  if (!f) {
    err = std::string("cannot open boundary file ") + path;
    return -1;
  }
  std::string line;
  if (!std::getline(f, line)) {
    err = "empty boundary file";
    return -1;
  }
  std::vector<std::string> head = split_csv(line);
  int pnx = -1, pny = -1, pnz = -1, ppt = -1;
  for (size_t c = 0; c < head.size(); c++) {
    if (strcasecmp(head[c].c_str(), "nx") == 0) pnx = (int)c;
    if (strcasecmp(head[c].c_str(), "ny") == 0) pny = (int)c;
    if (strcasecmp(head[c].c_str(), "nz") == 0) pnz = (int)c;
    if (strcasecmp(head[c].c_str(), "pt") == 0) ppt = (int)c;
  }
  if (pnx < 0 || pny < 0 || pnz < 0 || ppt < 0 || head.size() < 4) {
    err = "boundary file header must name nx, ny, nz and pt columns";
    return -1;
  }
  const long n = (long)nx * ny * nz;
  pt.assign(n, 1);
  ns.assign(3 * n, 0.f);
  int maxpt = 0, lineno = 0;
  while (std::getline(f, line)) {
    lineno++;
    std::vector<std::string> v = split_csv(line);
    if (v.empty() || (v.size() == 1 && v[0].empty())) continue;
    if ((int)v.size() <= std::max(std::max(pnx, pny), std::max(pnz, ppt))) {
      err = "malformed boundary file line " + std::to_string(lineno);
      return -1;
    }
    const int i = (int)atof(v[0].c_str()), j = (int)atof(v[1].c_str()), k = (int)atof(v[2].c_str());
    const int p = (int)atof(v[ppt].c_str());
    // src/geometry_custom.cpp:105-115
    if (i >= nx || j >= ny || k >= nz || i < 0 || j < 0 || k < 0) {
      err = "point out of simulation box at line " + std::to_string(lineno);
      return -1;
    }
    if (p < 0) {
      err = "negative point type at line " + std::to_string(lineno);
      return -1;
    }
    const long s = (long)i + (long)nx * ((long)j + (long)ny * k);
    pt[s] = p;
    ns[3 * s] = (float)atof(v[pnx].c_str());
    ns[3 * s + 1] = (float)atof(v[pny].c_str());
    ns[3 * s + 2] = (float)atof(v[pnz].c_str());
    maxpt = std::max(maxpt, p);
  }
  return std::max(0, maxpt - 1);
}

// ---------------------------------------------------------------------------
// Parameter file (src/io.cpp:81-253).
// ---------------------------------------------------------------------------
namespace {
struct Tokens {
  std::vector<std::pair<std::string, int>> tok;  // token, line
  size_t pos = 0;
  bool next(std::string &t, int &line) {
    if (pos >= tok.size()) return false;
    t = tok[pos].first;
    line = tok[pos].second;
    pos++;
    return true;
  }
  void skip_line(int line) {
    while (pos < tok.size() && tok[pos].second == line) pos++;
  }
};

bool to_int(const std::string &s, int &v) {
  char *e = nullptr;
  long x = strtol(s.c_str(), &e, 10);
  if (e == s.c_str()) return false;
  v = (int)x;
  return true;
}
bool to_float(const std::string &s, float &v) {
  char *e = nullptr;
  float x = strtof(s.c_str(), &e);
  if (e == s.c_str()) return false;
  v = x;
  return true;
}
bool is(const std::string &a, const char *b) { return strcasecmp(a.c_str(), b) == 0; }
}  // namespace

int parse_param_file(const char *path, SimParams &p, std::string &err) {
  std::ifstream f(path);
  if (!f) {
    err = std::string("cannot open parameter file ") + path;
    return MCX_ERR_IO;
  }
  Tokens T;
  std::string line;
  int ln = 0;
  while (std::getline(f, line)) {
    ln++;
    std::istringstream is(line);
    std::string t;
    while (is >> t) T.tok.push_back({t, ln});
  }
  std::string key, val;
  int kl, vl;
  auto bad = [&](const std::string &k) {
    err = "invalid value for parameter: " + k;
    return MCX_ERR_PARSE;
  };
  while (T.next(key, kl)) {
    if (key[0] == '#') {
      T.skip_line(kl);
      continue;
    }
    int *ip = nullptr;
    float *fp = nullptr;
    std::string *sp = nullptr;
    std::map<int, float> *mf = nullptr;
    std::map<int, std::string> *ms = nullptr;
    if (is(key, "nx")) ip = &p.Nx;
    else if (is(key, "ny")) ip = &p.Ny;
    else if (is(key, "nz")) ip = &p.Nz;
    else if (is(key, "A")) fp = &p.A;
    else if (is(key, "B1")) fp = &p.B1;
    else if (is(key, "B2")) fp = &p.B2;
    else if (is(key, "C")) fp = &p.C;
    else if (is(key, "Ti")) fp = &p.Ti;
    else if (is(key, "Tf")) fp = &p.Tf;
    else if (is(key, "dT")) fp = &p.dT;
    else if (is(key, "MCS")) ip = &p.MCS;
    else if (is(key, "MCT")) ip = &p.MCT;
    else if (is(key, "seed")) ip = &p.seed;
    else if (is(key, "ic")) sp = &p.ic;
    else if (is(key, "ic_file")) sp = &p.ic_file;
    else if (is(key, "xbound")) sp = &p.xbound;
    else if (is(key, "ybound")) sp = &p.ybound;
    else if (is(key, "zbound")) sp = &p.zbound;
    else if (is(key, "potential")) sp = &p.potential;
    else if (is(key, "evol") || is(key, "mode")) sp = &p.evol;
    else if (is(key, "k11")) fp = &p.k11;
    else if (is(key, "k22")) fp = &p.k22;
    else if (is(key, "k33")) fp = &p.k33;
    else if (is(key, "p0")) fp = &p.p0;
    else if (is(key, "phi_0")) fp = &p.phi_0;
    else if (is(key, "theta_0")) fp = &p.theta_0;
    else if (is(key, "p0_i")) fp = &p.p0_i;
    else if (is(key, "fn")) ip = &p.fn;
    else if (is(key, "first_file_number") || is(key, "initial_output")) ip = &p.first_file;
    else if (is(key, "geometry")) sp = &p.geometry;
    else if (is(key, "boundary_file")) sp = &p.bound_file;
    else if (is(key, "anchoring_type")) ms = &p.anchoring_type;
    else if (is(key, "W")) mf = &p.W;
    else if (is(key, "phi_s")) mf = &p.phi_s;
    else if (is(key, "theta_s")) mf = &p.theta_s;
    else if (is(key, "nk") || is(key, "neighbour_kind") || is(key, "neighbour")) {
      int nk;
      if (!T.next(val, vl) || !to_int(val, nk)) return bad(key);
      T.skip_line(vl);
      if (nk != 1) {  // src/io.cpp:211-223
        err = "neighbour_kind = " + std::to_string(nk) + " is not supported; only nk = 1 (nearest neighbours)";
        return MCX_ERR_PARSE;
      }
      continue;
    } else if (is(key, "elecX") || is(key, "Electric_field_x") || is(key, "EF_x")) fp = &p.elecX;
    else if (is(key, "elecY") || is(key, "Electric_field_y") || is(key, "EF_y")) fp = &p.elecY;
    else if (is(key, "elecZ") || is(key, "Electric_field_z") || is(key, "EF_z")) fp = &p.elecZ;
    else if (is(key, "Ei") || is(key, "initial_E")) fp = &p.elecEi;
    else if (is(key, "Ef") || is(key, "final_E")) fp = &p.elecEf;
    else if (is(key, "dE") || is(key, "E_variation")) fp = &p.elecdE;
    else if (is(key, "elecA") || is(key, "dielectric_anisotropy") || is(key, "Aniso_E")) fp = &p.elecA;
    else if (is(key, "radius")) fp = &p.radius;
    else if (is(key, "replicas")) ip = &p.replicas;
    else {
      err = "unknown parameter: '" + key + "'";
      return MCX_ERR_PARSE;
    }
    if (ms || mf) {
      int id;
      if (!T.next(val, vl) || !to_int(val, id)) return bad(key);
      if (!T.next(val, vl)) return bad(key);
      if (ms) {
        (*ms)[id] = val;
      } else {
        float x;
        if (!to_float(val, x)) return bad(key);
        (*mf)[id] = x;
      }
      T.skip_line(vl);
      continue;
    }
    if (!T.next(val, vl)) return bad(key);
    if (ip && !to_int(val, *ip)) return bad(key);
    if (fp && !to_float(val, *fp)) return bad(key);
    if (sp) *sp = val;
    T.skip_line(vl);
  }
  return MCX_OK;
}

}  // namespace mcx
