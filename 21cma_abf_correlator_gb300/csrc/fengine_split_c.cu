// fengine_split_c.cu -- F-engine kernels of n_freq 26624 and 28672 (split frames).
// Compiled apart from fengine.cu so that the groups of lengths build in
// parallel; fengine_impl.cuh holds the templates.

#include "fengine_impl.cuh"

namespace corrgb {

corr_status fengine_launch_split_c(int n_freq, const TwiddleTables &tw, const FengineArgs &a,
                                   int num_sms, cudaStream_t stream) {
    switch (n_freq) {
    case 26624: return launch_half<13312>(a, tw, num_sms, stream);
    case 28672: return launch_half<14336>(a, tw, num_sms, stream);
    default: return failf(CORR_ERR_INTERNAL, "fengine_launch_split_c: n_freq=%d", n_freq);
    }
}

} // namespace corrgb
