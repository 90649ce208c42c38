// mcx_kernels.cuh -- launch interface between the engine (mcx_engine.cu) and
// the kernels (mcx_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "mcx_device.cuh"

namespace mcx {

// Which specialisation of the sweep / measure kernels a batch runs: the pair
// potential, whether any replica has a mask (inactive or surface sites), and
// whether any replica has a field term.  Fixed per engine.
struct Variant {
  int pot;
  bool mask;
  bool field;
};

struct PassArgs {
  const RepDev *reps;
  const int2 *map;  // per CTA: (replica, first float4 group)
  float *dir;
  const uint8_t *pt;
  const float *ns;
  RepState *st;
  int colour;
  // trace outputs (natural site order of one replica), used only by the
  // trace specialisation
  float *tr_dE;
  uint8_t *tr_acc;
  float *tr_prop;
};

struct MeasureArgs {
  const RepDev *reps;
  const int2 *map;
  const float *dir;
  const uint8_t *pt;
  const float *ns;
  double *macc;  // [nrep][kMacc]
};

struct EpilogueArgs {
  const RepDev *reps;
  RepState *st;
  double *macc;
  double *stats;   // [nrep][kStats]
  double *series;  // [nrep][series_cap][2] or null
  int series_cap;
  int nrep;
};

void launch_pass(const Variant &v, const PassArgs &a, int nblocks, bool trace, cudaStream_t st);
void launch_measure(const Variant &v, const MeasureArgs &a, int nblocks, cudaStream_t st);
void launch_epilogue(const EpilogueArgs &a, bool measure, cudaStream_t st);
void launch_measure_out(const EpilogueArgs &a, double *out, cudaStream_t st);
void launch_aos_to_split(const RepDev &R, const float *aos, float *dir, cudaStream_t st);
void launch_split_to_aos(const RepDev &R, const float *dir, float *aos, cudaStream_t st);
void launch_mask_to_split(const RepDev &R, const int *pt_aos, const float *ns_aos, uint8_t *pt, float *ns,
                          cudaStream_t st);
void launch_split_to_mask(const RepDev &R, const uint8_t *pt, const float *ns, int *pt_aos, float *ns_aos,
                          cudaStream_t st);
void launch_init(const RepDev &R, const uint8_t *pt, float *dir, int mode, uint32_t seed, float fx, float fy, float fz,
                 cudaStream_t st);

}  // namespace mcx
