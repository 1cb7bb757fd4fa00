// Kernel instantiations for grid sizes 16, 24, 32, 48.
#include "dispatch_impl.cuh"

namespace fftdock {

const SizeOps* size_ops_small(int n) {
    switch (n) {
        case 16: return SizeOpsImpl<16>::ops();
        case 24: return SizeOpsImpl<24>::ops();
        case 32: return SizeOpsImpl<32>::ops();
        case 48: return SizeOpsImpl<48>::ops();
        default: return nullptr;
    }
}

}  // namespace fftdock
