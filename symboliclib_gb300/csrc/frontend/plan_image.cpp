// Plan -> symgb_plan_desc flattening.
#include "symgb/plan_image.hpp"

#include "symgb/traverse.hpp"

namespace symgb {

std::vector<symgb_node> serializeTemplate(const Symbolic& t) {
    std::vector<symgb_node> out;
    postOrderTraverse(t, [&](const Symbolic& x) {
        symgb_node n{};
        n.op = x.op();
        n.nchild = (int)x.numChilds();
        if (x.op() == CONST) {
            n.value = x.constant();
        } else if (x.op() == VAR) {
            n.a = x.variable()[0];
            n.b = x.variable()[1];
        }
        out.push_back(n);
    });
    return out;
}

void buildPlanImage(Plan& P, PlanImage& img, unsigned threadsPerBlock) {
    const std::size_t K = P.kernels.size();
    img.kernels.assign(K, symgb_kernel_desc{});
    img.nodes.assign(K, {});
    img.access.assign(K, {});
    for (std::size_t k = 0; k < K; ++k) {
        ComputeKernel& ck = P.kernels[k];
        img.nodes[k] = serializeTemplate(ck.templateExpression());
        for (auto& a : ck.access()) {
            img.access[k].push_back(a.baseRow);
            img.access[k].push_back(a.offset);
        }
        symgb_kernel_desc& d = img.kernels[k];
        d.num_instances = ck.numInstances();
        d.output_offset = ck.outputOffset;
        d.index_offset = ck.indexOffset;
        d.constants_offset = ck.constantsOffset;
        d.num_output_rows = (std::uint32_t)ck.numOutputRows();
        d.num_index_rows = (std::uint32_t)ck.numVariableRows();
        d.num_constant_rows = (std::uint32_t)ck.numConstantRows();
        d.level = P.kernelLevel[k];
        d.num_nodes = (std::uint32_t)img.nodes[k].size();
        d.nodes = img.nodes[k].data();
        d.num_access = (std::uint32_t)ck.access().size();
        d.access = img.access[k].data();
    }
    img.argStart.assign(P.argStart.begin(), P.argStart.end());
    img.argLength.assign(P.argLength.begin(), P.argLength.end());
    img.outStart.assign(P.outputIndexStart.begin(), P.outputIndexStart.end());
    img.outLength.assign(P.outputIndexLength.begin(), P.outputIndexLength.end());
    img.indexData = P.positionData;
    img.outIndexData.assign(P.outputIdsFlat.begin(), P.outputIdsFlat.end());
    img.constData = P.constantData;

    symgb_plan_desc& d = img.desc;
    d.num_kernels = (std::uint32_t)K;
    d.kernels = img.kernels.data();
    d.num_args = (std::uint32_t)img.argStart.size();
    d.arg_start = img.argStart.data();
    d.arg_length = img.argLength.data();
    d.num_outputs = (std::uint32_t)img.outStart.size();
    d.output_start = img.outStart.data();
    d.output_length = img.outLength.data();
    d.num_total_memory = P.numTotalMemory;
    d.num_indices = img.indexData.size();
    d.num_output_values = img.outIndexData.size();
    d.num_constants = img.constData.size();
    d.threads_per_block = threadsPerBlock;
}

}  // namespace symgb
