// Fused eSRRF instantiations for magnification 5, window half-widths J = 1..6,
// tile variant 1 (one producer warp group fewer; chosen per batch by the
// tiling autotuner).
#include "internal.h"

namespace nx {

template <int J>
static FusedEntry entry_m5_alt() {
  return FusedEntry{{&launch_fused<5, J, kModeStack, 1>, &launch_fused<5, J, kModeSum, 1>,
                     &launch_fused<5, J, kModeFull, 1>},
                    {&fused_occupancy<5, J, kModeStack, 1>, &fused_occupancy<5, J, kModeSum, 1>,
                     &fused_occupancy<5, J, kModeFull, 1>},
                    {&fused_smem_bytes<5, J, kModeStack, 1>, &fused_smem_bytes<5, J, kModeSum, 1>,
                     &fused_smem_bytes<5, J, kModeFull, 1>},
                    fused_geometry<5, J, 1>()};
}

const FusedEntry* fused_entry_m5_alt(int J) {
  static const FusedEntry table[6] = {entry_m5_alt<1>(), entry_m5_alt<2>(), entry_m5_alt<3>(),
                                      entry_m5_alt<4>(), entry_m5_alt<5>(), entry_m5_alt<6>()};
  return (J >= 1 && J <= 6) ? &table[J - 1] : nullptr;
}

}  // namespace nx
