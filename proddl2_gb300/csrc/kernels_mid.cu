// Kernel instantiations for grid sizes 64, 80.
#include "dispatch_impl.cuh"

namespace fftdock {

const SizeOps* size_ops_mid(int n) {
    switch (n) {
        case 64: return SizeOpsImpl<64>::ops();
        case 80: return SizeOpsImpl<80>::ops();
        default: return nullptr;
    }
}

}  // namespace fftdock
