// fengine_split_b.cu -- F-engine kernels of n_freq 22528 and 24576 (split frames).
// Compiled apart from fengine.cu so that the groups of lengths build in
// parallel; fengine_impl.cuh holds the templates.

#include "fengine_impl.cuh"

namespace corrgb {

corr_status fengine_launch_split_b(int n_freq, const TwiddleTables &tw, const FengineArgs &a,
                                   int num_sms, cudaStream_t stream) {
    switch (n_freq) {
    case 22528: return launch_half<11264>(a, tw, num_sms, stream);
    case 24576: return launch_half<12288>(a, tw, num_sms, stream);
    default: return failf(CORR_ERR_INTERNAL, "fengine_launch_split_b: n_freq=%d", n_freq);
    }
}

} // namespace corrgb
