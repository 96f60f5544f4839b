// Fused eSRRF instantiations for magnification 8, window half-widths J = 1..6.
#include "internal.h"

namespace nx {

template <int J>
static FusedEntry entry_m8() {
  return FusedEntry{{&launch_fused<8, J, kModeStack>, &launch_fused<8, J, kModeSum>,
                     &launch_fused<8, J, kModeFull>},
                    {&fused_occupancy<8, J, kModeStack>, &fused_occupancy<8, J, kModeSum>,
                     &fused_occupancy<8, J, kModeFull>},
                    {&fused_smem_bytes<8, J, kModeStack>, &fused_smem_bytes<8, J, kModeSum>,
                     &fused_smem_bytes<8, J, kModeFull>},
                    fused_geometry<8, J>()};
}

const FusedEntry* fused_entry_m8(int J) {
  static const FusedEntry table[6] = {entry_m8<1>(), entry_m8<2>(), entry_m8<3>(),
                                      entry_m8<4>(), entry_m8<5>(), entry_m8<6>()};
  return (J >= 1 && J <= 6) ? &table[J - 1] : nullptr;
}

}  // namespace nx
