// Golden-fixture generator: runs the reference SymbolicLib (built from its own
// sources by oracle/Makefile into oracle/_ref/libsymref.so) on the project's
// workload model code and writes, per workload,
//   <name>.plan.txt  - the reference's plan for a CUDA device (kernels, templates,
//                      index/constant/output tables) in the engine's canonical
//                      plan text;
//   <name>.refplan   - the same plan as an engine plan file, built from the
//                      reference's own kernel objects (buildRefPlan below);
//   <name>.in.bin    - the input values (float64, input containers concatenated);
//   <name>.out.bin   - the reference CPU ComputeUnit's results (float64), its
//                      generated code compiled without fast-math or FP
//                      contraction (SYMREF_STRICT=1), i.e. every operation in the
//                      reference's written order.
// Usage: gen_golden <outdir> <workload> <size> <seed>
// See make_golden.sh for the build and run recipe.
#include "ComputeUnit.hpp"
#include "Symbolic.hpp"
#include "SymbolicDifferentiation.hpp"
#include "SymbolicUtilities.hpp"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <limits>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>

#include "../../include/symgb.h"
#include "../../symboliclib_gb300/csrc/workloads/workloads.hpp"

using namespace symgb_workloads;

namespace {

// Read access to the reference's private plan members: explicit template
// instantiations may name private members, and the friend function defined by
// the instantiation hands out the member pointer.
template <class Tag, auto M>
struct Expose {
    friend constexpr auto member(Tag) { return M; }
};
#define SYMREF_EXPOSE(TAG, PTR)                    \
    struct TAG {                                   \
        friend constexpr auto member(TAG);         \
    };                                             \
    template struct Expose<TAG, PTR>;
SYMREF_EXPOSE(TKernels, &Sym::ComputeUnit<double>::kernels)
SYMREF_EXPOSE(TInputSizes, &Sym::ComputeUnit<double>::inputSizes)
SYMREF_EXPOSE(TOutputIds, &Sym::ComputeUnit<double>::outputIds)
SYMREF_EXPOSE(TInputDataSize, &Sym::ComputeUnit<double>::inputDataSize)
SYMREF_EXPOSE(TVariableDataSize, &Sym::ComputeUnit<double>::variableDataSize)
SYMREF_EXPOSE(TPositionData, &Sym::ComputeUnit<double>::positionData)
SYMREF_EXPOSE(TOutputIdsFlat, &Sym::ComputeUnit<double>::outputIdsFlat)
SYMREF_EXPOSE(TConstantData, &Sym::ComputeUnit<double>::constantData)
SYMREF_EXPOSE(TTemplate, &Sym::Kernel::templateExpression)
SYMREF_EXPOSE(TAccess, &Sym::Kernel::variableAccessData)
SYMREF_EXPOSE(TOutTable, &Sym::Kernel::outputVariableTable)
SYMREF_EXPOSE(TVarTable, &Sym::Kernel::variableTable)
SYMREF_EXPOSE(TConstTable, &Sym::Kernel::constantTable)
#define REF(obj, TAG) ((obj).*member(TAG{}))

const char* opName(int op) {
    static const char* names[30] = {"NOOP", "CONST", "VAR", "ADD", "MUL", "MULC", "DIV", "SQRT", "SIN", "COS",
                                    "TAN", "COT", "ASIN", "ACOS", "ATAN", "EXP", "LOG", "POW", "ASSIGN", "GROUP",
                                    "CONDPOS", "CONDNONZERO", "CONDZERO", "NEG", "DEFINE", "BLOCK", "REC",
                                    "FIXED", "FUNC", "CALL"};
    return op < 30 ? names[op] : "?";
}

void writeTemplate(const Sym::Symbolic& x, std::ostream& os) {
    if (x.op() == Sym::CONST) {
        std::uint64_t bits;
        double c = x.constant();
        std::memcpy(&bits, &c, 8);
        os << "#" << std::hex << bits << std::dec;
    } else if (x.op() == Sym::VAR) {
        os << "v(" << x.variable()[0] << "," << x.variable()[1] << ")";
    } else {
        os << "(" << opName(x.op());
        for (unsigned i = 0; i < x.numChilds(); ++i) {
            os << " ";
            writeTemplate(x[i], os);
        }
        os << ")";
    }
}

template <class T>
void writeList(std::ostream& os, const char* name, const T& v) {
    os << name << " " << v.size() << ":";
    for (auto& e : v) os << " " << e;
    os << "\n";
}

// Same text layout as symgb::dumpPlan.
void dumpRefPlan(Sym::ComputeUnit<double>& u, std::ostream& os) {
    auto& kernels = REF(u, TKernels);
    os << "kernels " << kernels.size() << "\n";
    for (std::size_t k = 0; k < kernels.size(); ++k) {
        auto& K = kernels[k];
        os << "kernel " << k << " n=" << K.numInstances() << " outOff=" << K.getGlobalOutputOffset()
           << " idxOff=" << K.getGlobalIndexOffset() << " constOff=" << K.getGlobalConstantsOffset() << "\n";
        os << "access";
        for (auto& a : REF(K, TAccess)) os << " " << a.baseVariableId << ":" << a.offset;
        os << "\n";
        os << "template ";
        writeTemplate(REF(K, TTemplate), os);
        os << "\n";
    }
    std::vector<std::size_t> argStart, argLength, outStart, outLength;
    std::size_t acc = 0;
    for (auto s : REF(u, TInputSizes)) {
        argStart.push_back(acc);
        argLength.push_back(s);
        acc += s;
    }
    acc = 0;
    for (auto& ids : REF(u, TOutputIds)) {
        outStart.push_back(acc);
        outLength.push_back(ids.size());
        acc += ids.size();
    }
    writeList(os, "argStart", argStart);
    writeList(os, "argLength", argLength);
    writeList(os, "outputIndexStart", outStart);
    writeList(os, "outputIndexLength", outLength);
    os << "numTotalMemory " << (REF(u, TInputDataSize) + REF(u, TVariableDataSize)) << "\n";
    writeList(os, "positionData", REF(u, TPositionData));
    writeList(os, "outputIds", REF(u, TOutputIdsFlat));
    os << "constantData " << REF(u, TConstantData).size() << ":";
    for (double c : REF(u, TConstantData)) {
        std::uint64_t bits;
        std::memcpy(&bits, &c, 8);
        os << " " << std::hex << bits << std::dec;
    }
    os << "\n";
}

// The reference-side binding of the engine's C ABI: the plan description
// (symgb_plan_desc) built straight from a reference ComputeUnit's own kernels
// and tables - the metadata its generated source bakes in as globals
// (ComputeUnit.cpp:371-407) and the templates its kernel bodies are printed
// from (ComputeKernel.cpp:329-381) - and written with symgb_plan_save.  This
// is the code a maintainer adds to ComputeUnit::compile in place of the code
// generator (INTEGRATION.md shows it as a patch).
struct RefPlanImage {
    std::vector<symgb_kernel_desc> kernels;
    std::vector<std::vector<symgb_node>> nodes;
    std::vector<std::vector<std::int32_t>> access;
    std::vector<std::uint64_t> argStart, argLength, outStart, outLength;
    std::vector<std::uint32_t> index, outIds;
    std::vector<double> constants;
    symgb_plan_desc desc{};
};

void serializeRef(const Sym::Symbolic& x, std::vector<symgb_node>& out) {
    for (unsigned i = 0; i < x.numChilds(); ++i) serializeRef(x[i], out);
    symgb_node n{};
    n.op = x.op();
    n.nchild = (int)x.numChilds();
    if (x.op() == Sym::CONST) {
        n.value = x.constant();
    } else if (x.op() == Sym::VAR) {
        n.a = x.variable()[0];
        n.b = x.variable()[1];
    }
    out.push_back(n);
}

void buildRefPlan(Sym::ComputeUnit<double>& u, RefPlanImage& img) {
    auto& kernels = REF(u, TKernels);
    const std::size_t K = kernels.size();
    img.index.assign(REF(u, TPositionData).begin(), REF(u, TPositionData).end());
    img.outIds.assign(REF(u, TOutputIdsFlat).begin(), REF(u, TOutputIdsFlat).end());
    img.constants.assign(REF(u, TConstantData).begin(), REF(u, TConstantData).end());
    img.kernels.assign(K, symgb_kernel_desc{});
    img.nodes.resize(K);
    img.access.resize(K);
    // Level of each kernel: one more than the deepest kernel whose output
    // slots it reads (kernels are in topological order), from its index table.
    std::vector<std::pair<std::uint64_t, std::size_t>> outRanges;  // (first slot, kernel)
    std::vector<int> level(K, 0);
    for (std::size_t k = 0; k < K; ++k) {
        auto& Kr = kernels[k];
        const std::uint64_t n = (std::uint64_t)Kr.numInstances();
        symgb_kernel_desc& d = img.kernels[k];
        d.num_instances = n;
        d.output_offset = Kr.getGlobalOutputOffset();
        d.index_offset = Kr.getGlobalIndexOffset();
        d.constants_offset = Kr.getGlobalConstantsOffset();
        d.num_output_rows = (std::uint32_t)REF(Kr, TOutTable).size();
        d.num_index_rows = (std::uint32_t)REF(Kr, TVarTable).size();
        d.num_constant_rows = (std::uint32_t)REF(Kr, TConstTable).size();
        serializeRef(REF(Kr, TTemplate), img.nodes[k]);
        for (auto& a : REF(Kr, TAccess)) {
            img.access[k].push_back(a.baseVariableId);
            img.access[k].push_back(a.offset);
        }
        int lv = 0;
        for (auto& a : REF(Kr, TAccess))
            for (std::uint64_t i = 0; i < n; ++i) {
                const std::uint64_t slot =
                    (std::uint32_t)(img.index[d.index_offset + (std::uint64_t)a.baseVariableId * n + i] + a.offset);
                auto it = std::upper_bound(outRanges.begin(), outRanges.end(),
                                           std::make_pair(slot, std::numeric_limits<std::size_t>::max()));
                if (it == outRanges.begin()) continue;  // an input slot
                --it;
                const symgb_kernel_desc& p = img.kernels[it->second];
                if (slot < p.output_offset + p.num_output_rows * p.num_instances) lv = std::max(lv, level[it->second] + 1);
            }
        level[k] = lv;
        d.level = lv;
        outRanges.insert(std::upper_bound(outRanges.begin(), outRanges.end(), std::make_pair(d.output_offset, k)),
                         std::make_pair(d.output_offset, k));
    }
    for (std::size_t k = 0; k < K; ++k) {
        img.kernels[k].num_nodes = (std::uint32_t)img.nodes[k].size();
        img.kernels[k].nodes = img.nodes[k].data();
        img.kernels[k].num_access = (std::uint32_t)(img.access[k].size() / 2);
        img.kernels[k].access = img.access[k].data();
    }
    std::uint64_t acc = 0;
    for (auto s : REF(u, TInputSizes)) {
        img.argStart.push_back(acc);
        img.argLength.push_back(s);
        acc += s;
    }
    acc = 0;
    for (auto& ids : REF(u, TOutputIds)) {
        img.outStart.push_back(acc);
        img.outLength.push_back(ids.size());
        acc += ids.size();
    }
    symgb_plan_desc& d = img.desc;
    d.num_kernels = (std::uint32_t)K;
    d.kernels = img.kernels.data();
    d.num_args = (std::uint32_t)img.argStart.size();
    d.arg_start = img.argStart.data();
    d.arg_length = img.argLength.data();
    d.num_outputs = (std::uint32_t)img.outStart.size();
    d.output_start = img.outStart.data();
    d.output_length = img.outLength.data();
    d.num_total_memory = REF(u, TInputDataSize) + REF(u, TVariableDataSize);
    d.num_indices = img.index.size();
    d.num_output_values = img.outIds.size();
    d.num_constants = img.constants.size();
    d.threads_per_block = 128;
}

void writeBin(const std::string& path, const std::vector<double>& v) {
    std::ofstream f(path, std::ios::binary);
    f.write((const char*)v.data(), v.size() * sizeof(double));
}

struct RefFix {
    template <class A>
    void operator()(A& K9, A& D9) const {
        Sym::makeFixed(K9, D9);
    }
};

std::vector<Sym::Symbolic> variables(std::size_t n, int group) {
    std::vector<Sym::Symbolic> v;
    v.reserve(n);
    for (std::size_t i = 0; i < n; ++i) v.emplace_back((int)i, group);
    return v;
}

// Builds the reference plan (CUDA device layout) and runs the reference CPU unit.
template <class... Inputs>
void run(const std::string& out, const std::vector<Sym::Symbolic>& outputs, const std::vector<double>& inputValues,
         const std::vector<std::vector<double>>& inputs, const std::vector<std::vector<Sym::Symbolic>>& inputSyms) {
    {
        Sym::ComputeUnit<double>* u = nullptr;
        if (inputSyms.size() == 1)
            u = new Sym::ComputeUnit<double>(Sym::Device(Sym::UseCuda(), Sym::ThreadsPerBlock(128)), inputSyms[0], outputs);
        else
            u = new Sym::ComputeUnit<double>(Sym::Device(Sym::UseCuda(), Sym::ThreadsPerBlock(128)), inputSyms[0],
                                             inputSyms[1], outputs);
        std::ofstream f(out + ".plan.txt");
        dumpRefPlan(*u, f);
        RefPlanImage img;
        buildRefPlan(*u, img);
        if (symgb_plan_save((out + ".refplan").c_str(), &img.desc, img.index.data(), img.outIds.data(),
                            img.constants.data()) != 0) {
            std::fprintf(stderr, "symgb_plan_save: %s\n", symgb_plan_last_error());
            std::exit(1);
        }
        // never compiled; not destroyed to keep the process free of dlclose
    }
    Sym::ComputeUnit<double>* cpu = nullptr;
    if (inputSyms.size() == 1)
        cpu = new Sym::ComputeUnit<double>(Sym::Device(Sym::NumThreads(1)), inputSyms[0], outputs);
    else
        cpu = new Sym::ComputeUnit<double>(Sym::Device(Sym::NumThreads(1)), inputSyms[0], inputSyms[1], outputs);
    cpu->compile();
    std::vector<double> res(outputs.size());
    if (inputs.size() == 1)
        cpu->execute(inputs[0]);
    else
        cpu->execute(inputs[0], inputs[1]);
    cpu->getResults(res);
    writeBin(out + ".in.bin", inputValues);
    writeBin(out + ".out.bin", res);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: gen_golden <outdir> <workload> <size> <seed>\n");
        return 2;
    }
    const std::string dir = argv[1], w = argv[2];
    const int size = std::atoi(argv[3]);
    const std::uint64_t seed = std::strtoull(argv[4], nullptr, 10);
    const std::string out = dir + "/" + w + "_" + std::to_string(size);
    Sym::Symbolic::varIdCounter = 0;  // fresh EXPLICIT_INTERMEDIATE numbering

    if (w == "ata") {
        CSC<double> A = stencilMatrix(size, 2, seed);
        auto AS = variables(A.nnz(), 0);
        CSC<Sym::Symbolic> B = ataPlusA(A, AS);
        run(out, B.values, A.values, {A.values}, {AS});
    } else if (w == "cotan") {
        TriMesh m = cotanMesh(size, seed);
        auto VS = variables(m.V.size(), 0);
        CSC<Sym::Symbolic> L = cotanLaplacian(VS, m.nv, m.F);
        run(out, L.values, m.V, {m.V}, {VS});
    } else if (w == "cloth") {
        ClothRest r = clothRest(size);
        std::vector<double> X, vel;
        clothState(r, seed, X, vel);
        auto XS = variables(X.size(), 0), VS = variables(vel.size(), 1);
        CSC<Sym::Symbolic> A = clothMatrix(r, XS, VS, RefFix());
        std::vector<double> all(X);
        all.insert(all.end(), vel.begin(), vel.end());
        run(out, A.values, all, {X, vel}, {XS, VS});
    } else if (w == "random") {
        Rng rng(seed ^ 0x5eedULL);
        const int m = std::max(8, size / 2);
        std::vector<double> vals(m);
        for (auto& v : vals) v = rng.uniform(0.5, 1.5);
        auto VS = variables(vals.size(), 0);
        auto outv = randomExpressions(VS, size, seed);
        run(out, outv, vals, {vals}, {VS});
    } else if (w == "neohookean") {
        TetMesh m = tetMesh(size);
        std::vector<double> X = tetState(m, seed);
        auto XS = variables(X.size(), 0);
        auto E = neoHookeanEnergies(m, XS);
        auto upper = Sym::hessianSparse(Sym::Symbolic(Sym::ADD, E), XS);
        CSC<Sym::Symbolic> H = symmetricFromUpper((int)X.size(), upper);
        run(out, H.values, X, {X}, {XS});
    } else {
        std::fprintf(stderr, "unknown workload %s\n", w.c_str());
        return 2;
    }
    std::fflush(stdout);
    // The reference unloads its OpenMP library in ~ComputeUnit, which crashes;
    // leave without running destructors.
    std::_Exit(0);
}
