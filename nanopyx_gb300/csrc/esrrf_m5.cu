// Fused eSRRF instantiations for magnification 5, window half-widths J = 1..6.
#include "internal.h"

namespace nx {

template <int J>
static FusedEntry entry_m5() {
  return FusedEntry{{&launch_fused<5, J, kModeStack>, &launch_fused<5, J, kModeSum>,
                     &launch_fused<5, J, kModeFull>},
                    {&fused_occupancy<5, J, kModeStack>, &fused_occupancy<5, J, kModeSum>,
                     &fused_occupancy<5, J, kModeFull>},
                    {&fused_smem_bytes<5, J, kModeStack>, &fused_smem_bytes<5, J, kModeSum>,
                     &fused_smem_bytes<5, J, kModeFull>},
                    fused_geometry<5, J>()};
}

const FusedEntry* fused_entry_m5(int J) {
  static const FusedEntry table[6] = {entry_m5<1>(), entry_m5<2>(), entry_m5<3>(),
                                      entry_m5<4>(), entry_m5<5>(), entry_m5<6>()};
  return (J >= 1 && J <= 6) ? &table[J - 1] : nullptr;
}

}  // namespace nx
