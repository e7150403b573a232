// Split-transform variants 0 (NT 256, CH 24), 1 (NT 192, CH 48).
#include "transforms.cuh"

namespace chn {

CHN_SPLIT_VARIANT(0, 256, 24)
CHN_SPLIT_VARIANT(1, 192, 48)

}  // namespace chn
