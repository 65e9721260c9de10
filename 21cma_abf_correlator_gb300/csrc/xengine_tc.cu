// xengine_tc.cu -- tcgen05 tensor-core X-engine (FP16 spectra, FP32 accumulation).

#include "engine.h"

namespace corrgb {

size_t xengine_tc_workspace_bytes(int, int) { return 0; }

corr_status xengine_tc_launch(const XengineArgs &, bool, int, cudaStream_t) {
    return fail(CORR_ERR_NOT_IMPL, "tensor-core X-engine is not built yet");
}

} // namespace corrgb
