// Kernel instantiations for grid sizes 144.
#include "dispatch_impl.cuh"

namespace fftdock {

const SizeOps* size_ops_n144(int n) {
    switch (n) {
        case 144: return SizeOpsImpl<144>::ops();
        default: return nullptr;
    }
}

}  // namespace fftdock
