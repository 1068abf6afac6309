// Map-writing instantiations of the TMA CPS kernel (k_cps_tma.cuh): the launchers qmiv_cps_maps
// uses, which also store each pixel's argmin window index.
#include "k_cps_tma.cuh"

namespace qmiv {

#define X(SR, QPW, NWD, KT, T, K64, SB, SUF) \
  QMIV_TMA_MAP_DECL(SR, QPW, NWD, KT, T, K64, SB, SUF) \
  { return launch_tma_as<SR, QPW, NWD, KT, T, true>(d, n, blocks, p, st); }
QMIV_TMA_VARIANTS(X)
#undef X

}  // namespace qmiv
