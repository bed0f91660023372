// FP64 instantiations of the engine's phase-group kernels.
#include "fab_kernel.cuh"

namespace gm {
template <class Pol, int R>
static void* group_ptr(int group) {
  switch (group) {
    case 0: return (void*)fab_kernel<Pol, R, KG_LANCZOS>;
    case 1: return (void*)fab_kernel<Pol, R, KG_SOLVE>;
    case 2: return (void*)fab_kernel<Pol, R, KG_APPLY>;
    case 3: return (void*)fab_kernel<Pol, R, KG_DEFLATE>;
    case 4: return (void*)fab_kernel<Pol, R, KG_LANCZOS | KG_SOLVE | KG_APPLY>;
    case 5: return (void*)fab_kernel<Pol, R, KG_LANCZOS | PH_MPK>;
    case 6: return (void*)fab_kernel<Pol, R, KG_LANCZOS | KG_SOLVE | KG_APPLY | PH_MPK>;
    case 7: return (void*)fab_kernel<Pol, R, KG_LANCZOS | PH_REORTH>;
    case 8: return (void*)fab_kernel<Pol, R, KG_LANCZOS | KG_SOLVE | KG_APPLY | PH_REORTH>;
  }
  return nullptr;
}
void* kernel_fp64(int R, int group) {
  if (R == 1) return group_ptr<PolFP64, 1>(group);
  if (R == 2) return group_ptr<PolFP64, 2>(group);
  if (R == 4) return group_ptr<PolFP64, 4>(group);
  return nullptr;
}
}  // namespace gm
