// Kernel instantiations for grid sizes 128.
#include "dispatch_impl.cuh"

namespace fftdock {

const SizeOps* size_ops_n128(int n) {
    switch (n) {
        case 128: return SizeOpsImpl<128>::ops();
        default: return nullptr;
    }
}

}  // namespace fftdock
