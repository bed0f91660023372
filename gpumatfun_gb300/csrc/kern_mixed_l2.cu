// One-right-hand-side instantiations of the mixed engine's SpMV phase groups
// at two resident blocks per SM (PolMixedL2), for mixed engines whose matrix
// is held in the L2 persisting window.  Groups without SpMV passes, and the matrix-powers
// and Gram-Schmidt groups (already compiled for two blocks), use the kernels
// of the ordinary policy.
#include "fab_kernel.cuh"

namespace gm {
void* kernel_mixed_l2(int group) {
  switch (group) {
    case 0: return (void*)fab_kernel<PolMixedL2, 1, KG_LANCZOS>;
    case 2: return (void*)fab_kernel<PolMixedL2, 1, KG_APPLY>;
    case 4: return (void*)fab_kernel<PolMixedL2, 1, KG_LANCZOS | KG_SOLVE | KG_APPLY>;
  }
  return nullptr;
}
}  // namespace gm
