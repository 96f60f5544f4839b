// Fused eSRRF instantiations for magnification 6, window half-widths J = 1..6.
#include "internal.h"

namespace nx {

template <int J>
static FusedEntry entry_m6() {
  return FusedEntry{{&launch_fused<6, J, kModeStack>, &launch_fused<6, J, kModeSum>,
                     &launch_fused<6, J, kModeFull>},
                    {&fused_occupancy<6, J, kModeStack>, &fused_occupancy<6, J, kModeSum>,
                     &fused_occupancy<6, J, kModeFull>},
                    {&fused_smem_bytes<6, J, kModeStack>, &fused_smem_bytes<6, J, kModeSum>,
                     &fused_smem_bytes<6, J, kModeFull>},
                    fused_geometry<6, J>()};
}

const FusedEntry* fused_entry_m6(int J) {
  static const FusedEntry table[6] = {entry_m6<1>(), entry_m6<2>(), entry_m6<3>(),
                                      entry_m6<4>(), entry_m6<5>(), entry_m6<6>()};
  return (J >= 1 && J <= 6) ? &table[J - 1] : nullptr;
}

}  // namespace nx
