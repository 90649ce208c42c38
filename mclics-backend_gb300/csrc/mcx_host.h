// mcx_host.h -- host-side setup shared by the engine and the simulator
// driver: GHRL constants, anchoring axes, geometry masks, parameter file.
#pragma once
#include <map>
#include <string>
#include <vector>

#include "../../include/mcx.h"

namespace mcx {

// setGHRL (src/io.cpp:277-302): lambda, mu, nu, rho, sigma from k11, k22,
// k33, p0 with the reference's float/double rounding.
void ghrl_constants(float k11, float k22, float k33, float p0, float out[5]);

// Easy axis from (theta_s, phi_s) in degrees (src/anchoring_rp.cpp:43-45).
void anchoring_axis(float theta_s, float phi_s, float out[3]);

// Point types and normals of a bulk / slab / sphere lattice in natural AoS
// order (src/geometry_bulk.cpp:57-61, src/geometry_slab.cpp:47-67,
// src/geometry_sphere.cpp:28-54).  Returns false for custom geometry.
bool build_mask(const mcx_replica_desc &d, std::vector<int> &pt, std::vector<float> &ns);

// Custom geometry file (src/geometry_custom.cpp:57-128): CSV with a header
// naming the columns; x, y, z are the first three, nx/ny/nz/pt located by
// name; unlisted sites are bulk (pt = 1).  Returns the surface count
// (max pt - 1) or -1 with a message in err.
int read_custom_geometry(const char *path, int nx, int ny, int nz, std::vector<int> &pt, std::vector<float> &ns,
                         std::string &err);

// The reference's Parameters (include/parameters.h:11-83), as read from a
// parameter file.
struct SimParams {
  std::string geometry = "bulk";
  int Nx = 16, Ny = 16, Nz = 16;
  std::string xbound = "free", ybound = "free", zbound = "free";
  std::string bound_file;
  std::map<int, float> theta_s, phi_s, W;
  std::map<int, std::string> anchoring_type;
  std::string potential = "ll";
  float A = 1.0f, B1 = 0.04f, B2 = 0.4f, C = 0.3f;
  float Ti = 1.2f, Tf = 0.0f, dT = -0.02f;
  std::string evol = "thermal";
  int MCS = 100, MCT = 100, fn = 1, first_file = 0, seed = 1;
  std::string ic = "random", ic_file;
  float phi_0 = 0, theta_0 = 0, p0_i = 0;
  float k11 = 1, k22 = 1, k33 = 1, p0 = 0;
  float elecX = 0, elecY = 0, elecZ = 0, elecA = 0, elecEi = 0, elecEf = 0, elecdE = 0, elecE = 1;
  // extension: sphere radius (0 = Nz/2 as the reference)
  float radius = 0;
  // extension: number of replicas run side by side (seeds seed, seed+1, ...)
  int replicas = 1;
};

// read_input_file (src/io.cpp:81-253): case-insensitive keys, '#' comments,
// unknown keys and bad values are errors.  Returns 0 or an mcx_status with a
// message in err.
int parse_param_file(const char *path, SimParams &p, std::string &err);

// Sets the message mcx_last_error(NULL) returns.
void set_last_error(const char *msg);
// the message mcx_last_error(e) returns
void set_engine_error(mcx_engine *e, const char *msg);

}  // namespace mcx
