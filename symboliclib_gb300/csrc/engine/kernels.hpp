// Interpreter kernel variants, instantiated in their own translation units
// (eval_items.cu, eval_lanes.cu) so the build compiles them in parallel.
#pragma once

namespace symgb {
namespace engine {

// evalKernel<items, lanes, mode> (device.cuh) as a launchable function
// pointer.  Shapes: items 1, 2 or 4 with one lane, or one item with 2, 4 or 8
// lanes; mode is a combination of MODE_L2 and MODE_LIB.  Null for other shapes.
const void* evalKernelFor(int items, int lanes, int mode);

// The two halves of evalKernelFor, one per translation unit.
const void* evalKernelOneLane(int items, int mode);
const void* evalKernelOneItem(int lanes, int mode);

}  // namespace engine
}  // namespace symgb
