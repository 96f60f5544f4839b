// Fused eSRRF instantiations for magnification 3, window half-widths J = 1..6.
#include "internal.h"

namespace nx {

template <int J>
static FusedEntry entry_m3() {
  return FusedEntry{{&launch_fused<3, J, kModeStack>, &launch_fused<3, J, kModeSum>,
                     &launch_fused<3, J, kModeFull>},
                    {&fused_occupancy<3, J, kModeStack>, &fused_occupancy<3, J, kModeSum>,
                     &fused_occupancy<3, J, kModeFull>},
                    {&fused_smem_bytes<3, J, kModeStack>, &fused_smem_bytes<3, J, kModeSum>,
                     &fused_smem_bytes<3, J, kModeFull>},
                    fused_geometry<3, J>()};
}

const FusedEntry* fused_entry_m3(int J) {
  static const FusedEntry table[6] = {entry_m3<1>(), entry_m3<2>(), entry_m3<3>(),
                                      entry_m3<4>(), entry_m3<5>(), entry_m3<6>()};
  return (J >= 1 && J <= 6) ? &table[J - 1] : nullptr;
}

}  // namespace nx
