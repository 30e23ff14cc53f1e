// GJK pass instantiations with 4 and 8 lanes per pair.
#include "gjk_pass.cuh"

namespace fclg {
FCLG_GJK_INSTANTIATE(4)
FCLG_GJK_INSTANTIATE(8)
}  // namespace fclg
