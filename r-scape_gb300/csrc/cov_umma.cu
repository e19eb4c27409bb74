// cov_umma.cu -- tensor-core counting (placeholder until the tcgen05 kernel
// lands): the plan reports the path as unavailable.
#include "cov_umma.h"

namespace covgpu {

struct UmmaPlan { int dummy; };

UmmaPlan* umma_plan_create(int, int, int, int, const TileRC*, int, int) { return nullptr; }
void umma_plan_destroy(UmmaPlan* p) { delete p; }
void umma_set_weights(UmmaPlan*, const double*, int, cudaStream_t) {}
cudaError_t umma_count(UmmaPlan*, const uint8_t*, int64_t, int, bool, float*, cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // namespace covgpu
