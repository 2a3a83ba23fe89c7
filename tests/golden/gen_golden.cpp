// Golden-fixture generator: runs the reference SymbolicLib (built from its own
// sources by oracle/Makefile into oracle/_ref/libsymref.so) on the project's
// workload model code and writes, per workload,
//   <name>.plan.txt  - the reference's plan for a CUDA device (kernels, templates,
//                      index/constant/output tables) in the engine's canonical
//                      plan text;
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

#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>

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
