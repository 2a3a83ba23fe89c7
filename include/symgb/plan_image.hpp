// Flattened, C-ABI form of a front-end Plan (the symgb_plan_desc of symgb.h)
// with the storage it points into.
#pragma once
#include <cstdint>
#include <vector>

#include "../symgb.h"
#include "frontend.hpp"

namespace symgb {

struct PlanImage {
    symgb_plan_desc desc{};
    std::vector<symgb_kernel_desc> kernels;
    std::vector<std::vector<symgb_node>> nodes;
    std::vector<std::vector<std::int32_t>> access;
    std::vector<std::uint64_t> argStart, argLength, outStart, outLength;
    std::vector<std::uint32_t> indexData, outIndexData;
    std::vector<double> constData;

    PlanImage() = default;
    PlanImage(const PlanImage&) = delete;
    PlanImage& operator=(const PlanImage&) = delete;
};

// Fills `img` from `plan` (templates serialised post-order, tables copied).
void buildPlanImage(Plan& plan, PlanImage& img, unsigned threadsPerBlock);

// Post-order node list of a template expression tree.
std::vector<symgb_node> serializeTemplate(const Symbolic& t);

}  // namespace symgb
