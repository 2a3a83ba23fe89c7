// Interpreter instantiations with one lane per work item (1, 2 or 4 items per
// thread), and the variant dispatch.
#include "device.cuh"
#include "kernels.hpp"

namespace symgb {
namespace engine {

template <int ITEMS>
static const void* byMode(int mode) {
    switch (mode) {
        case 0: return (const void*)evalKernel<ITEMS, 1, 0>;
        case MODE_L2: return (const void*)evalKernel<ITEMS, 1, MODE_L2>;
        case MODE_LIB: return (const void*)evalKernel<ITEMS, 1, MODE_LIB>;
        case MODE_L2 | MODE_LIB: return (const void*)evalKernel<ITEMS, 1, MODE_L2 | MODE_LIB>;
        default: return nullptr;
    }
}

const void* evalKernelOneLane(int items, int mode) {
    switch (items) {
        case 1: return byMode<1>(mode);
        case 2: return byMode<2>(mode);
        case 4: return byMode<4>(mode);
        default: return nullptr;
    }
}

const void* evalKernelFor(int items, int lanes, int mode) {
    if (lanes == 1) return evalKernelOneLane(items, mode);
    if (items == 1) return evalKernelOneItem(lanes, mode);
    return nullptr;
}

}  // namespace engine
}  // namespace symgb
