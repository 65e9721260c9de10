// fengine_large.cu -- F-engine kernels of n_freq 10240, 12288, 14336 and 16384.
// Compiled apart from fengine.cu so that the groups of lengths build in
// parallel; fengine_impl.cuh holds the templates.

#include "fengine_impl.cuh"

namespace corrgb {

corr_status fengine_launch_large(int n_freq, const TwiddleTables &tw, const FengineArgs &a,
                                 int num_sms, cudaStream_t stream) {
    switch (n_freq) {
    case 10240: return launch_size<10240>(a, tw, num_sms, stream);
    case 12288: return launch_size<12288>(a, tw, num_sms, stream);
    case 14336: return launch_size<14336>(a, tw, num_sms, stream);
    case 16384: return launch_size<16384>(a, tw, num_sms, stream);
    default: return failf(CORR_ERR_INTERNAL, "fengine_launch_large: n_freq=%d", n_freq);
    }
}

} // namespace corrgb
