// Fused eSRRF instantiations for magnification 4, window half-widths J = 1..6,
// tile variant 1 (one producer warp group fewer; chosen per batch by the
// tiling autotuner).
#include "internal.h"

namespace nx {

template <int J>
static FusedEntry entry_m4_alt() {
  return FusedEntry{{&launch_fused<4, J, kModeStack, 1>, &launch_fused<4, J, kModeSum, 1>,
                     &launch_fused<4, J, kModeFull, 1>},
                    {&fused_occupancy<4, J, kModeStack, 1>, &fused_occupancy<4, J, kModeSum, 1>,
                     &fused_occupancy<4, J, kModeFull, 1>},
                    {&fused_smem_bytes<4, J, kModeStack, 1>, &fused_smem_bytes<4, J, kModeSum, 1>,
                     &fused_smem_bytes<4, J, kModeFull, 1>},
                    fused_geometry<4, J, 1>()};
}

const FusedEntry* fused_entry_m4_alt(int J) {
  static const FusedEntry table[6] = {entry_m4_alt<1>(), entry_m4_alt<2>(), entry_m4_alt<3>(),
                                      entry_m4_alt<4>(), entry_m4_alt<5>(), entry_m4_alt<6>()};
  return (J >= 1 && J <= 6) ? &table[J - 1] : nullptr;
}

}  // namespace nx
