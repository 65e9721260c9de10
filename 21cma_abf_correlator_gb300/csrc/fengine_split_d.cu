// fengine_split_d.cu -- F-engine kernels of n_freq 30720 and 32768 (split frames).
// Compiled apart from fengine.cu so that the groups of lengths build in
// parallel; fengine_impl.cuh holds the templates.

#include "fengine_impl.cuh"

namespace corrgb {

corr_status fengine_launch_split_d(int n_freq, const TwiddleTables &tw, const FengineArgs &a,
                                   int num_sms, cudaStream_t stream) {
    switch (n_freq) {
    case 30720: return launch_half<15360>(a, tw, num_sms, stream);
    case 32768: return launch_half<16384>(a, tw, num_sms, stream);
    default: return failf(CORR_ERR_INTERNAL, "fengine_launch_split_d: n_freq=%d", n_freq);
    }
}

} // namespace corrgb
