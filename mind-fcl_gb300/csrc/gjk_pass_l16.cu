// GJK pass instantiations with 16 and 32 lanes per pair.
#include "gjk_pass.cuh"

namespace fclg {
FCLG_GJK_INSTANTIATE(16)
FCLG_GJK_INSTANTIATE(32)
}  // namespace fclg
