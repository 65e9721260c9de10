// fengine_split_a.cu -- F-engine kernels of n_freq 18432 and 20480 (split frames).
// Compiled apart from fengine.cu so that the groups of lengths build in
// parallel; fengine_impl.cuh holds the templates.

#include "fengine_impl.cuh"

namespace corrgb {

corr_status fengine_launch_split_a(int n_freq, const TwiddleTables &tw, const FengineArgs &a,
                                   int num_sms, cudaStream_t stream) {
    switch (n_freq) {
    case 18432: return launch_half<9216>(a, tw, num_sms, stream);
    case 20480: return launch_half<10240>(a, tw, num_sms, stream);
    default: return failf(CORR_ERR_INTERNAL, "fengine_launch_split_a: n_freq=%d", n_freq);
    }
}

} // namespace corrgb
