// Fused eSRRF instantiations for magnification 1, window half-widths J = 1..6.
#include "internal.h"

namespace nx {

template <int J>
static FusedEntry entry_m1() {
  return FusedEntry{{&launch_fused<1, J, kModeStack>, &launch_fused<1, J, kModeSum>,
                     &launch_fused<1, J, kModeFull>},
                    {&fused_occupancy<1, J, kModeStack>, &fused_occupancy<1, J, kModeSum>,
                     &fused_occupancy<1, J, kModeFull>},
                    {&fused_smem_bytes<1, J, kModeStack>, &fused_smem_bytes<1, J, kModeSum>,
                     &fused_smem_bytes<1, J, kModeFull>},
                    fused_geometry<1, J>()};
}

const FusedEntry* fused_entry_m1(int J) {
  static const FusedEntry table[6] = {entry_m1<1>(), entry_m1<2>(), entry_m1<3>(),
                                      entry_m1<4>(), entry_m1<5>(), entry_m1<6>()};
  return (J >= 1 && J <= 6) ? &table[J - 1] : nullptr;
}

}  // namespace nx
