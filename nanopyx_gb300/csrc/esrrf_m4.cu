// Fused eSRRF instantiations for magnification 4, window half-widths J = 1..6.
#include "internal.h"

namespace nx {

template <int J>
static FusedEntry entry_m4() {
  return FusedEntry{{&launch_fused<4, J, kModeStack>, &launch_fused<4, J, kModeSum>,
                     &launch_fused<4, J, kModeFull>},
                    {&fused_occupancy<4, J, kModeStack>, &fused_occupancy<4, J, kModeSum>,
                     &fused_occupancy<4, J, kModeFull>},
                    {&fused_smem_bytes<4, J, kModeStack>, &fused_smem_bytes<4, J, kModeSum>,
                     &fused_smem_bytes<4, J, kModeFull>},
                    fused_geometry<4, J>()};
}

const FusedEntry* fused_entry_m4(int J) {
  static const FusedEntry table[6] = {entry_m4<1>(), entry_m4<2>(), entry_m4<3>(),
                                      entry_m4<4>(), entry_m4<5>(), entry_m4<6>()};
  return (J >= 1 && J <= 6) ? &table[J - 1] : nullptr;
}

}  // namespace nx
