// Kernel instantiations for grid sizes 96, 112.
#include "dispatch_impl.cuh"

namespace fftdock {

const SizeOps* size_ops_big(int n) {
    switch (n) {
        case 96: return SizeOpsImpl<96>::ops();
        case 112: return SizeOpsImpl<112>::ops();
        default: return nullptr;
    }
}

}  // namespace fftdock
