// C ABI over the synthetic workloads: builds a workload's expressions with the
// engine's front end, plans it, and exposes the plan, its tables, the seeded
// input values and the FP64 values of the same model evaluated in double
// arithmetic.  Used by the tests and the benchmark through ctypes.
#include <chrono>
#include <cstring>
#include <memory>
#include <sstream>
#include <string>

#include "symgb/differentiation.hpp"
#include "symgb/frontend.hpp"
#include "symgb/parallel.hpp"
#include "symgb/plan_image.hpp"
#include "symgb/utilities.hpp"
#include "workloads.hpp"

using namespace symgb_workloads;

namespace {

struct Workload {
    symgb::Plan plan;
    symgb::PlanImage image;
    std::vector<std::vector<double>> inputs;
    std::vector<double> numeric;  // model evaluated in double
    std::string planText;
    double frontSeconds = 0.0;
    double modelSeconds = 0.0;  // building the symbolic outputs (the workload's own model code)
    std::uint64_t outputs = 0;
    int rows = 0, cols = 0;              // output matrix (CSC workloads)
    std::vector<int> colPtr, rowIdx;
};

thread_local std::string g_err;

std::vector<symgb::Symbolic> variables(std::size_t n, int group) {
    std::vector<symgb::Symbolic> v;
    v.reserve(n);
    for (std::size_t i = 0; i < n; ++i) v.emplace_back((int)i, group);
    return v;
}

struct Fix {
    template <class A>
    void operator()(A& K9, A& D9) const {
        symgb::makeFixed(K9, D9);
    }
    // All faces at once: each face's variable count first, then every face
    // numbered from its prefix sum, so the variables are those of the
    // face-by-face loop.
    template <class A, class For>
    void batch(std::vector<A>& K9s, std::vector<A>& D9s, For& forEach) const {
        const std::size_t n = K9s.size();
        auto spans = [&](std::size_t f) {
            return std::vector<std::pair<symgb::Symbolic*, std::size_t>>{{K9s[f].data(), K9s[f].size()},
                                                                         {D9s[f].data(), D9s[f].size()}};
        };
        std::vector<int> first(n + 1, 0);
        forEach(n, [&](std::size_t b, std::size_t e) {
            for (std::size_t f = b; f < e; ++f) first[f + 1] = symgb::fixedVariableCount(spans(f));
        });
        int& counter = symgb::Symbolic::uniqueVariableCounter();
        first[0] = counter;
        for (std::size_t f = 0; f < n; ++f) first[f + 1] += first[f];
        forEach(n, [&](std::size_t b, std::size_t e) {
            for (std::size_t f = b; f < e; ++f) symgb::makeFixedSpansAt(spans(f), first[f]);
        });
        counter = first[n];
    }
};
// The front end's worker pool for the independent per-element parts of the
// model code; handles to shared nodes (the input variables) are copied from
// several threads, so reference counts are atomic meanwhile.
struct PoolFor {
    template <class F>
    void operator()(std::size_t n, F&& fn) const {
        symgb::Symbolic::ConcurrentRefs concurrent;
        symgb::parallelFor(n, 64, [&](std::size_t b, std::size_t e) { fn(b, e); });
    }
};
struct NoFix {
    template <class A>
    void operator()(A&, A&) const {}
};

}  // namespace

extern "C" {

typedef struct Workload* symgbw_t;

const char* symgbw_last_error(void) { return g_err.c_str(); }

// workload: "ata" (side), "cotan" (side), "cloth" (side), "neohookean" (cells
// per side), "random" (outputs), "literals" (outputs).  vector_width: 0 for
// the device layout, k > 0 for the reference CPU layout with SIMD width k.
int symgbw_build(const char* name, int size, unsigned long long seed, int vector_width, int want_text, symgbw_t* out) {
    try {
        std::unique_ptr<Workload> w(new Workload());
        symgb::DeviceConfig dev;
        dev.vectorWidth = (unsigned)std::max(0, vector_width);
        dev.cudaDevice = vector_width == 0;
        symgb::PlanBuilder pb(dev);
        symgb::Symbolic::uniqueVariableCounter() = 0;
        const std::string n = name;
        const auto t0 = std::chrono::steady_clock::now();
        if (n == "ata") {
            CSC<double> A = stencilMatrix(size, 2, seed);
            auto AS = variables(A.nnz(), 0);
            CSC<symgb::Symbolic> B = ataPlusA(A, AS);
            pb.addContainer(AS.data(), AS.size());
            pb.addContainer(B.values.data(), B.values.size());
            w->inputs.push_back(A.values);
            w->numeric = ataPlusA(A, A.values).values;
            w->outputs = B.nnz();
            w->rows = B.rows, w->cols = B.cols, w->colPtr = B.colPtr, w->rowIdx = B.rowIdx;
        } else if (n == "cotan") {
            TriMesh m = cotanMesh(size, seed);
            auto VS = variables(m.V.size(), 0);
            CSC<symgb::Symbolic> L = cotanLaplacian(VS, m.nv, m.F);
            pb.addContainer(VS.data(), VS.size());
            pb.addContainer(L.values.data(), L.values.size());
            w->inputs.push_back(m.V);
            w->numeric = cotanLaplacian(m.V, m.nv, m.F).values;
            w->outputs = L.nnz();
            w->rows = L.rows, w->cols = L.cols, w->colPtr = L.colPtr, w->rowIdx = L.rowIdx;
        } else if (n == "cloth") {
            ClothRest r = clothRest(size);
            std::vector<double> X, vel;
            clothState(r, seed, X, vel);
            auto XS = variables(X.size(), 0), VS = variables(vel.size(), 1);
            CSC<symgb::Symbolic> A = clothMatrix(r, XS, VS, Fix(), PoolFor());
            pb.addContainer(XS.data(), XS.size());
            pb.addContainer(VS.data(), VS.size());
            pb.addContainer(A.values.data(), A.values.size());
            w->inputs.push_back(X);
            w->inputs.push_back(vel);
            w->numeric = clothMatrix(r, X, vel, NoFix()).values;
            w->outputs = A.nnz();
            w->rows = A.rows, w->cols = A.cols, w->colPtr = A.colPtr, w->rowIdx = A.rowIdx;
        } else if (n == "random") {
            Rng rng(seed ^ 0x5eedULL);
            const int m = std::max(8, size / 2);
            std::vector<double> vals(m);
            for (auto& v : vals) v = rng.uniform(0.5, 1.5);
            auto VS = variables(vals.size(), 0);
            auto out = randomExpressions(VS, size, seed);
            pb.addContainer(VS.data(), VS.size());
            pb.addContainer(out.data(), out.size());
            w->inputs.push_back(vals);
            w->numeric = randomExpressions(vals, size, seed);
            w->outputs = out.size();
        } else if (n == "literals") {
            Rng rng(seed ^ 0x11ULL);
            const int m = std::max(64, size / 4);
            std::vector<double> vals(m);
            for (auto& v : vals) v = rng.uniform(-1.0, 1.0);
            auto VS = variables(vals.size(), 0);
            auto out = literalSums(VS, size, 40);
            pb.addContainer(VS.data(), VS.size());
            pb.addContainer(out.data(), out.size());
            w->inputs.push_back(vals);
            w->numeric = literalSums(vals, size, 40);
            w->outputs = out.size();
        } else if (n == "neohookean") {
            TetMesh m = tetMesh(size);
            std::vector<double> X = tetState(m, seed);
            auto XS = variables(X.size(), 0);
            auto E = neoHookeanEnergies(m, XS);
            auto upper = symgb::hessianSparse(symgb::Symbolic(symgb::ADD, E), XS);
            CSC<symgb::Symbolic> H = symmetricFromUpper((int)X.size(), upper, PoolFor());
            pb.addContainer(XS.data(), XS.size());
            pb.addContainer(H.values.data(), H.values.size());
            w->inputs.push_back(X);
            w->numeric = symmetricFromUpper((int)X.size(), neoHookeanHessianUpper(m, X)).values;
            w->outputs = H.nnz();
            w->rows = H.rows, w->cols = H.cols, w->colPtr = H.colPtr, w->rowIdx = H.rowIdx;
        } else {
            g_err = "unknown workload " + n;
            return -1;
        }
        w->modelSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        w->plan = pb.build();
        w->frontSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        symgb::buildPlanImage(w->plan, w->image, 128);
        if (want_text) {
            std::ostringstream os;
            symgb::dumpPlan(w->plan, os);
            w->planText = os.str();
        }
        *out = w.release();
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

void symgbw_free(symgbw_t w) { delete w; }

const symgb_plan_desc* symgbw_plan(symgbw_t w) { return &w->image.desc; }
const uint32_t* symgbw_index_data(symgbw_t w) { return w->image.indexData.data(); }
const uint32_t* symgbw_out_index_data(symgbw_t w) { return w->image.outIndexData.data(); }
const double* symgbw_const_data(symgbw_t w) { return w->image.constData.data(); }
int symgbw_num_inputs(symgbw_t w) { return (int)w->inputs.size(); }
const double* symgbw_input(symgbw_t w, int i, uint64_t* n) {
    *n = w->inputs[i].size();
    return w->inputs[i].data();
}
const double* symgbw_numeric(symgbw_t w, uint64_t* n) {
    *n = w->numeric.size();
    return w->numeric.data();
}
uint64_t symgbw_plan_text(symgbw_t w, char* buf, uint64_t cap) {
    if (buf && cap) {
        const std::size_t k = std::min<std::size_t>(cap - 1, w->planText.size());
        std::memcpy(buf, w->planText.data(), k);
        buf[k] = 0;
    }
    return w->planText.size();
}
double symgbw_front_seconds(symgbw_t w) { return w->frontSeconds; }
double symgbw_model_seconds(symgbw_t w) { return w->modelSeconds; }

// Pattern of the output matrix (CSC; 0 rows when the workload has none):
// col_ptr has cols + 1 entries, row_idx nnz.
int symgbw_pattern(symgbw_t w, int* rows, int* cols, const int** col_ptr, const int** row_idx) {
    if (!w) return -1;
    *rows = w->rows;
    *cols = w->cols;
    *col_ptr = w->colPtr.data();
    *row_idx = w->rowIdx.data();
    return 0;
}

}  // extern "C"
