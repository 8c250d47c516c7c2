// restart.cu -- placeholder; replaced by the restart kernels.
#include "engine.hpp"
namespace mtc {
int Engine::restart(uint8_t*, uint64_t, const std::vector<const uint8_t*>&, const std::vector<uint64_t>&,
                    const std::vector<HeaderHost>&, uint32_t) {
  return fail(ST_ENOTSUP, "restart not built yet");
}
}
