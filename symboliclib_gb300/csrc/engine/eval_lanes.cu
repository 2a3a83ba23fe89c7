// Interpreter instantiations with several lanes per work item (one item per
// thread).
#include "device.cuh"
#include "kernels.hpp"

namespace symgb {
namespace engine {

template <int LANES>
static const void* byMode(int mode) {
    switch (mode) {
        case 0: return (const void*)evalKernel<1, LANES, 0>;
        case MODE_L2: return (const void*)evalKernel<1, LANES, MODE_L2>;
        case MODE_LIB: return (const void*)evalKernel<1, LANES, MODE_LIB>;
        case MODE_L2 | MODE_LIB: return (const void*)evalKernel<1, LANES, MODE_L2 | MODE_LIB>;
        default: return nullptr;
    }
}

const void* evalKernelOneItem(int lanes, int mode) {
    switch (lanes) {
        case 2: return byMode<2>(mode);
        case 4: return byMode<4>(mode);
        case 8: return byMode<8>(mode);
        default: return nullptr;
    }
}

}  // namespace engine
}  // namespace symgb
