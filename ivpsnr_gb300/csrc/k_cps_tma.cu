// Argmin-free instantiations of the TMA CPS kernel (k_cps_tma.cuh) and the variant table the
// host picks from; each variant also names its map-writing launcher from k_cps_tma_map.cu.
#include "k_cps_tma.cuh"

namespace qmiv {

#define X(...) QMIV_TMA_MAP_DECL(__VA_ARGS__);
QMIV_TMA_VARIANTS(X)
#undef X

namespace {

#define X(SR, QPW, NWD, KT, T, K64, SB, SUF) \
  { "tma420_sr" #SR "_q" #QPW "_w" #NWD #SUF, launch_tma_as<SR, QPW, NWD, KT, T, false>, \
    QMIV_TMA_MAP_LAUNCHER(SR, QPW, NWD, KT, T, K64, SB, SUF), SR, 2 * QPW * NWD, 64, K64, 2, SB },
const CpsVariant kVariants[] = {
QMIV_TMA_VARIANTS(X)
};
#undef X

}  // namespace

const CpsVariant* cps_variants_tma(int* n)
{
  *n = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
  return kVariants;
}

}  // namespace qmiv
