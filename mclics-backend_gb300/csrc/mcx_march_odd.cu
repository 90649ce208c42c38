// mcx_march_odd.cu -- the z-march kernel (mcx_march_kernel.cuh) for masked
// batches that hold a replica with an odd nx: its rows end in phantom slots
// (odd_tail), which the other masked builds leave out of their code.
#include <cuda_runtime.h>

#include "mcx_march_kernel.cuh"

namespace mcx {

template <int POT, bool FIELD, int NT>
static const void *march_fn_odd(int mode) {
  return mode == MODE_SWEEP_MEASURE ? (const void *)k_march<POT, true, FIELD, MODE_SWEEP_MEASURE, NT, false, true>
                                    : (const void *)k_march<POT, true, FIELD, MODE_SWEEP, NT, false, true>;
}

template <int NT>
static const void *march_fn_odd_v(const Variant &v, int mode) {
  if (v.pot == POT_LL) return v.field ? march_fn_odd<POT_LL, true, NT>(mode) : march_fn_odd<POT_LL, false, NT>(mode);
  if (v.pot == POT_PEAR)
    return v.field ? march_fn_odd<POT_PEAR, true, NT>(mode) : march_fn_odd<POT_PEAR, false, NT>(mode);
  return v.field ? march_fn_odd<POT_GHRL, true, NT>(mode) : march_fn_odd<POT_GHRL, false, NT>(mode);
}

const void *march_kernel_odd(const Variant &v, int mode, int nt) {
  switch (nt) {
    case 64: return march_fn_odd_v<64>(v, mode);
    case 256: return march_fn_odd_v<256>(v, mode);
    default: return march_fn_odd_v<128>(v, mode);
  }
}

}  // namespace mcx
