// Split-transform variants 2 (NT 256, CH 48), 3 (NT 128, CH 24).
#include "transforms.cuh"

namespace chn {

CHN_SPLIT_VARIANT(2, 256, 48)
CHN_SPLIT_VARIANT(3, 128, 24)

}  // namespace chn
