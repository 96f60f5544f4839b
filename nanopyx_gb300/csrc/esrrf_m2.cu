// Fused eSRRF instantiations for magnification 2, window half-widths J = 1..6.
#include "internal.h"

namespace nx {

template <int J>
static FusedEntry entry_m2() {
  return FusedEntry{{&launch_fused<2, J, kModeStack>, &launch_fused<2, J, kModeSum>,
                     &launch_fused<2, J, kModeFull>},
                    {&fused_occupancy<2, J, kModeStack>, &fused_occupancy<2, J, kModeSum>,
                     &fused_occupancy<2, J, kModeFull>},
                    {&fused_smem_bytes<2, J, kModeStack>, &fused_smem_bytes<2, J, kModeSum>,
                     &fused_smem_bytes<2, J, kModeFull>},
                    fused_geometry<2, J>()};
}

const FusedEntry* fused_entry_m2(int J) {
  static const FusedEntry table[6] = {entry_m2<1>(), entry_m2<2>(), entry_m2<3>(),
                                      entry_m2<4>(), entry_m2<5>(), entry_m2<6>()};
  return (J >= 1 && J <= 6) ? &table[J - 1] : nullptr;
}

}  // namespace nx
