// Synthetic workloads of the engine, written once as model code over a scalar
// type NT.  Instantiated with the engine's symgb::Symbolic they produce the
// expressions a ComputeUnit compiles; with double they are the numeric FP64
// oracle of the same quantity.  The code uses only NT arithmetic (+ - * /,
// unary -, sqrt found by argument-dependent lookup) and NT(double), so any
// scalar type with the reference's operator semantics can instantiate it.
//
// Sparse assembly sums duplicate triplets left to right in insertion order and
// stores values column-major with sorted rows (compressed sparse column), the
// storage order of an Eigen::SparseMatrix built with setFromTriplets.
#pragma once
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <functional>
#include <map>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

namespace symgb_workloads {

// ---------------------------------------------------------------- random

// Seeded generator with a fixed, platform-independent output sequence
// (splitmix64 seeding of xoshiro256**).
struct Rng {
    std::uint64_t s[4];
    explicit Rng(std::uint64_t seed) {
        for (auto& w : s) {
            seed += 0x9e3779b97f4a7c15ULL;
            std::uint64_t z = seed;
            z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
            z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
            w = z ^ (z >> 31);
        }
    }
    static std::uint64_t rotl(std::uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    std::uint64_t next() {
        const std::uint64_t r = rotl(s[1] * 5, 7) * 9;
        const std::uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
    double uniform(double lo, double hi) { return lo + (hi - lo) * uniform(); }
    std::uint64_t below(std::uint64_t n) { return next() % n; }
};

// ---------------------------------------------------------------- sparse

template <class NT>
struct Triplet {
    int row, col;
    NT value;
};

template <class NT>
struct CSC {
    int rows = 0, cols = 0;
    std::vector<int> colPtr, rowIdx;
    std::vector<NT> values;
    std::size_t nnz() const { return values.size(); }
};

// Runs fn(begin, end) over [0, n): serially (the default of the model
// functions below) or, when the engine's front end passes its worker pool,
// in parallel chunks.  Model code only parallelises loops whose iterations
// write disjoint results, so the expressions built do not depend on it.
struct SerialFor {
    template <class F>
    void operator()(std::size_t n, F&& fn) const {
        fn(std::size_t(0), n);
    }
};

// Duplicates are summed as ((t1 + t2) + t3) ... in triplet order.  Columns are
// independent: triplets are bucketed by column (keeping their order) and the
// columns summed by `forEach`.
template <class NT, class For = SerialFor>
CSC<NT> assemble(int rows, int cols, const std::vector<Triplet<NT>>& trips, For&& forEach = For()) {
    std::vector<std::size_t> start((std::size_t)cols + 1, 0), order(trips.size());
    for (const auto& t : trips) ++start[(std::size_t)t.col + 1];
    for (int c = 0; c < cols; ++c) start[c + 1] += start[c];
    {
        std::vector<std::size_t> fill(start.begin(), start.end() - 1);
        for (std::size_t i = 0; i < trips.size(); ++i) order[fill[trips[i].col]++] = i;
    }
    std::vector<std::vector<std::pair<int, NT>>> colEntries(cols);
    forEach((std::size_t)cols, [&](std::size_t cb, std::size_t ce) {
        for (std::size_t c = cb; c < ce; ++c) {
            std::map<int, NT> m;
            for (std::size_t q = start[c]; q < start[c + 1]; ++q) {
                const auto& t = trips[order[q]];
                auto it = m.find(t.row);
                if (it == m.end())
                    m.emplace(t.row, t.value);
                else
                    it->second = it->second + t.value;
            }
            colEntries[c].assign(m.begin(), m.end());
        }
    });
    CSC<NT> A;
    A.rows = rows;
    A.cols = cols;
    A.colPtr.assign(cols + 1, 0);
    for (int c = 0; c < cols; ++c) A.colPtr[c + 1] = A.colPtr[c] + (int)colEntries[c].size();
    A.rowIdx.resize(A.colPtr[cols]);
    A.values.resize(A.colPtr[cols]);
    forEach((std::size_t)cols, [&](std::size_t cb, std::size_t ce) {
        for (std::size_t c = cb; c < ce; ++c) {
            int k = A.colPtr[c];
            for (auto& e : colEntries[c]) {
                A.rowIdx[k] = e.first;
                A.values[k++] = std::move(e.second);
            }
            colEntries[c] = {};
        }
    });
    return A;
}

// A `fix` with a member batch(K9s, D9s, forEach) treats all faces at once
// (with the same result as fix(K9s[f], D9s[f]) face after face).
template <class F, class A, class For, class = void>
struct HasBatchFix : std::false_type {};
template <class F, class A, class For>
struct HasBatchFix<F, A, For,
                   std::void_t<decltype(std::declval<const F&>().batch(std::declval<std::vector<A>&>(),
                                                                       std::declval<std::vector<A>&>(),
                                                                       std::declval<For&>()))>> : std::true_type {};

// Lower triangle (row >= col) of a CSC matrix.
template <class NT>
CSC<NT> lowerTriangle(const CSC<NT>& A) {
    CSC<NT> L;
    L.rows = A.rows;
    L.cols = A.cols;
    L.colPtr.assign(A.cols + 1, 0);
    for (int c = 0; c < A.cols; ++c) {
        for (int k = A.colPtr[c]; k < A.colPtr[c + 1]; ++k)
            if (A.rowIdx[k] >= c) {
                L.rowIdx.push_back(A.rowIdx[k]);
                L.values.push_back(A.values[k]);
            }
        L.colPtr[c + 1] = (int)L.values.size();
    }
    return L;
}

// ---------------------------------------------------------------- meshes

struct TriMesh {
    int nv = 0;
    std::vector<double> V;  // nv x 3, column-major: V[v + d * nv]
    std::vector<std::array<int, 3>> F;
};

// nx x ny vertex grid; every quad split along the (i,j)-(i+1,j+1) diagonal.
inline std::vector<std::array<int, 3>> gridFaces(int nx, int ny) {
    std::vector<std::array<int, 3>> F;
    F.reserve(2 * (nx - 1) * (ny - 1));
    for (int j = 0; j + 1 < ny; ++j)
        for (int i = 0; i + 1 < nx; ++i) {
            const int v00 = i + j * nx, v10 = v00 + 1, v01 = v00 + nx, v11 = v01 + 1;
            F.push_back({v00, v10, v11});
            F.push_back({v00, v11, v01});
        }
    return F;
}

// Cotangent-Laplacian mesh: unit-square grid, x,y jittered by +-0.2 spacing,
// z = 0.1 sin(3x) cos(2y).
inline TriMesh cotanMesh(int side, std::uint64_t seed) {
    TriMesh m;
    m.nv = side * side;
    m.V.assign(3 * (std::size_t)m.nv, 0.0);
    const double h = 1.0 / (side - 1);
    Rng rng(seed);
    for (int j = 0; j < side; ++j)
        for (int i = 0; i < side; ++i) {
            const int v = i + j * side;
            const double x = i * h + rng.uniform(-0.2 * h, 0.2 * h);
            const double y = j * h + rng.uniform(-0.2 * h, 0.2 * h);
            m.V[v] = x;
            m.V[v + m.nv] = y;
            m.V[v + 2 * (std::size_t)m.nv] = 0.1 * std::sin(3 * x) * std::cos(2 * y);
        }
    m.F = gridFaces(side, side);
    return m;
}

// ---------------------------------------------------------------- vector helpers

template <class NT>
struct Vec3 {
    NT x, y, z;
};

template <class NT>
Vec3<NT> operator-(const Vec3<NT>& a, const Vec3<NT>& b) {
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}

template <class NT>
NT dot(const Vec3<NT>& a, const Vec3<NT>& b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}

template <class NT>
Vec3<NT> cross(const Vec3<NT>& a, const Vec3<NT>& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

template <class NT>
NT norm(const Vec3<NT>& a) {
    using std::sqrt;
    return sqrt(dot(a, a));
}

template <class NT>
Vec3<NT> row3(const std::vector<NT>& V, int nv, int v) {
    return {V[v], V[v + nv], V[v + 2 * (std::size_t)nv]};
}

// ---------------------------------------------------------------- workload 1: B = A^T A + A

// A: side^2 x side^2; 5-point stencil of a side x side grid plus `extra` random
// off-diagonal rows per column; pattern only (values are filled by the caller).
inline CSC<double> stencilMatrix(int side, int extra, std::uint64_t seed) {
    const int n = side * side;
    Rng rng(seed);
    std::vector<Triplet<double>> t;
    for (int c = 0; c < n; ++c) {
        const int i = c % side, j = c / side;
        std::vector<int> rowsC{c};
        if (i > 0) rowsC.push_back(c - 1);
        if (i + 1 < side) rowsC.push_back(c + 1);
        if (j > 0) rowsC.push_back(c - side);
        if (j + 1 < side) rowsC.push_back(c + side);
        int added = 0;
        while (added < extra && n > 6) {
            const int r = (int)rng.below((std::uint64_t)n);
            if (std::find(rowsC.begin(), rowsC.end(), r) != rowsC.end()) continue;
            rowsC.push_back(r);
            ++added;
        }
        for (int r : rowsC) t.push_back({r, c, 1.0});
    }
    CSC<double> A = assemble(n, n, t);
    for (double& v : A.values) v = rng.uniform(-1.0, 1.0);
    return A;
}

// Values of A^T A + A on the union pattern.  (A^T A)_ij = sum over k of
// A_ki A_kj, k ascending; an entry present in both terms is (A^T A)_ij + A_ij.
template <class NT>
CSC<NT> ataPlusA(const CSC<double>& pattern, const std::vector<NT>& a) {
    const int n = pattern.cols;
    // rows of A: for each row k, the (column, value index) pairs in column order
    std::vector<std::vector<std::pair<int, int>>> rowsOf(pattern.rows);
    for (int c = 0; c < n; ++c)
        for (int k = pattern.colPtr[c]; k < pattern.colPtr[c + 1]; ++k) rowsOf[pattern.rowIdx[k]].push_back({c, k});
    CSC<NT> B;
    B.rows = n;
    B.cols = n;
    B.colPtr.assign(n + 1, 0);
    for (int j = 0; j < n; ++j) {
        std::map<int, NT> acc;
        for (int kk = pattern.colPtr[j]; kk < pattern.colPtr[j + 1]; ++kk) {
            const int k = pattern.rowIdx[kk];
            for (auto& e : rowsOf[k]) {  // A_ki for all columns i of row k
                NT prod = a[e.second] * a[kk];
                auto it = acc.find(e.first);
                if (it == acc.end())
                    acc.emplace(e.first, prod);
                else
                    it->second = it->second + prod;
            }
        }
        for (int kk = pattern.colPtr[j]; kk < pattern.colPtr[j + 1]; ++kk) {
            const int i = pattern.rowIdx[kk];
            auto it = acc.find(i);
            if (it == acc.end())
                acc.emplace(i, a[kk]);
            else
                it->second = it->second + a[kk];
        }
        for (auto& e : acc) {
            B.rowIdx.push_back(e.first);
            B.values.push_back(e.second);
        }
        B.colPtr[j + 1] = (int)B.values.size();
    }
    return B;
}

// ---------------------------------------------------------------- workload 2: cotangent Laplacian

// Per face and corner j with opposite edge (j1, j2): w = dot(e0, e1) / |e0' x e1'|,
// triplets (j1,j1,-w) (j2,j2,-w) (j1,j2,w) (j2,j1,w).
template <class NT>
CSC<NT> cotanLaplacian(const std::vector<NT>& V, int nv, const std::vector<std::array<int, 3>>& F) {
    std::vector<Triplet<NT>> t;
    t.reserve(12 * F.size());
    for (const auto& f : F) {
        const Vec3<NT> a0 = row3(V, nv, f[0]);
        const NT area = norm(cross(a0 - row3(V, nv, f[1]), a0 - row3(V, nv, f[2])));
        for (int j = 0; j < 3; ++j) {
            const int j1 = f[(j + 1) % 3], j2 = f[(j + 2) % 3];
            const Vec3<NT> pj = row3(V, nv, f[j]);
            const NT w = dot(pj - row3(V, nv, j1), pj - row3(V, nv, j2)) / area;
            t.push_back({j1, j1, -w});
            t.push_back({j2, j2, -w});
            t.push_back({j1, j2, w});
            t.push_back({j2, j1, w});
        }
    }
    return assemble(nv, nv, t);
}

// ---------------------------------------------------------------- workload 3: Baraff-Witkin cloth

struct ClothParams {
    double kStretch = 1e3, kStretchDamping = 100.0;
    double kShear = 1e2, kShearDamping = 1.0;
    double kBend = 1e-1, kBendDamping = 1e-5;
    double totalMass = 2.5;
    double h = 0.05;
};

// Rest-state quantities (double) of a cloth mesh.
struct ClothRest {
    TriMesh mesh;  // rest positions
    ClothParams p;
    std::vector<double> area;                 // per face
    std::vector<std::array<double, 6>> B;     // per face, 3x2 row-major
    std::vector<std::array<double, 4>> Vinv;  // per face, 2x2 row-major
    std::vector<std::array<int, 4>> E4;       // interior edges: x0 x1 (edge), x2, x3 (opposite)
    std::vector<std::array<double, 16>> Q;    // per interior edge, 4x4 bend stiffness
};

inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
inline double norm3(const double* a) { return std::sqrt(dot3(a, a)); }

// Cloth rest mesh: side x side grid at unit spacing in the plane z = 0.
inline ClothRest clothRest(int side, const ClothParams& p = ClothParams()) {
    ClothRest r;
    r.p = p;
    TriMesh& m = r.mesh;
    m.nv = side * side;
    m.V.assign(3 * (std::size_t)m.nv, 0.0);
    for (int j = 0; j < side; ++j)
        for (int i = 0; i < side; ++i) {
            m.V[i + j * side] = i;
            m.V[i + j * side + m.nv] = j;
        }
    m.F = gridFaces(side, side);
    auto P = [&](int v, double* o) {
        for (int d = 0; d < 3; ++d) o[d] = m.V[v + d * (std::size_t)m.nv];
    };
    for (const auto& f : m.F) {
        double p0[3], p1[3], p2[3], v1[3], v2[3], c[3];
        P(f[0], p0);
        P(f[1], p1);
        P(f[2], p2);
        for (int d = 0; d < 3; ++d) {
            v1[d] = p1[d] - p0[d];
            v2[d] = p2[d] - p0[d];
        }
        cross3(v1, v2, c);
        r.area.push_back(0.5 * norm3(c));
        double u[3], nrm[3], w[3];
        const double l1 = norm3(v1);
        for (int d = 0; d < 3; ++d) u[d] = v1[d] / l1;
        cross3(u, v2, nrm);
        cross3(nrm, u, w);
        const double lw = norm3(w);
        for (int d = 0; d < 3; ++d) w[d] /= lw;
        const double a = l1, b = dot3(v2, u), c2 = 0.0, d2 = dot3(v2, w);
        const double det = a * d2 - b * c2;
        const std::array<double, 4> inv{d2 / det, -b / det, -c2 / det, a / det};
        r.Vinv.push_back(inv);
        r.B.push_back({-inv[0] - inv[2], -inv[1] - inv[3], inv[0], inv[1], inv[2], inv[3]});
    }
    // Interior edges with the two opposite vertices.
    std::map<std::pair<int, int>, std::pair<int, int>> edgeFaces;  // (min,max) -> (face, face)
    for (int fi = 0; fi < (int)m.F.size(); ++fi)
        for (int e = 0; e < 3; ++e) {
            const int a = m.F[fi][e], b = m.F[fi][(e + 1) % 3];
            auto key = std::make_pair(std::min(a, b), std::max(a, b));
            auto it = edgeFaces.find(key);
            if (it == edgeFaces.end())
                edgeFaces.emplace(key, std::make_pair(fi, -1));
            else
                it->second.second = fi;
        }
    for (auto& ef : edgeFaces) {
        if (ef.second.second < 0) continue;
        const auto& f0 = m.F[ef.second.first];
        const auto& f1 = m.F[ef.second.second];
        const int x0 = ef.first.first, x1 = ef.first.second;
        int x2 = -1, x3 = -1;
        for (int k = 0; k < 3; ++k) {
            if (f0[k] != x0 && f0[k] != x1) x2 = f0[k];
            if (f1[k] != x0 && f1[k] != x1) x3 = f1[k];
        }
        r.E4.push_back({x0, x1, x2, x3});
        double x[4][3];
        for (int k = 0; k < 4; ++k) P(r.E4.back()[k], x[k]);
        double e0[3], e1[3], e2[3], e3[3], e4[3], ne0[3];
        for (int d = 0; d < 3; ++d) {
            e0[d] = x[1][d] - x[0][d];
            e1[d] = x[2][d] - x[0][d];
            e2[d] = x[3][d] - x[0][d];
            e3[d] = x[2][d] - x[1][d];
            e4[d] = x[3][d] - x[1][d];
            ne0[d] = -e0[d];
        }
        auto cot = [](const double* v, const double* w) {
            double c[3];
            cross3(v, w, c);
            return dot3(v, w) / norm3(c);
        };
        const double c01 = cot(e0, e1), c02 = cot(e0, e2), c03 = cot(ne0, e3), c04 = cot(ne0, e4);
        const double K0[4] = {c03 + c04, c01 + c02, -c01 - c03, -c02 - c04};
        double c[3];
        cross3(e0, e1, c);
        const double A0 = norm3(c);
        cross3(e0, e2, c);
        const double A1 = norm3(c);
        const double coef = -3.0 / (A0 + A1);
        std::array<double, 16> Q;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) Q[4 * i + j] = coef * K0[i] * K0[j];
        r.Q.push_back(Q);
    }
    return r;
}

// Deformed state: rest + sum of three random-phase sinusoids (amplitude 0.05
// each, per coordinate), velocities uniform in [-0.1, 0.1].
inline void clothState(const ClothRest& r, std::uint64_t seed, std::vector<double>& X, std::vector<double>& vel) {
    const int nv = r.mesh.nv;
    Rng rng(seed);
    X = r.mesh.V;
    for (int d = 0; d < 3; ++d)
        for (int s = 0; s < 3; ++s) {
            const double kx = rng.uniform(0.05, 0.3), ky = rng.uniform(0.05, 0.3), ph = rng.uniform(0.0, 6.283185307179586);
            for (int v = 0; v < nv; ++v)
                X[v + d * (std::size_t)nv] += 0.05 * std::sin(kx * r.mesh.V[v] + ky * r.mesh.V[v + nv] + ph);
        }
    vel.resize(3 * (std::size_t)nv);
    for (auto& v : vel) v = rng.uniform(-0.1, 0.1);
}

// Lower triangle of A = M - h (D + h K) for the Baraff-Witkin stretch, shear
// and quadratic bend energies (after the reference example
// examples/BaraffWitkin: implementation/cloth.cpp:96-110,
// implementation/stretch_shear_forces_impl.hpp:63-261,
// implementation/bend_quadratic_forces.cpp:53-155).  `fix(K9, D9)` is applied
// to every face's 9x9 stiffness and damping blocks (makeFixed for symbolic
// scalars, nothing for double).  The faces' blocks are independent and built
// by `forEach` (serially by default); `fix` and the assembly then proceed in
// face order, so the result does not depend on it.
template <class NT, class Fix, class For = SerialFor>
CSC<NT> clothMatrix(const ClothRest& r, const std::vector<NT>& X, const std::vector<NT>& Vel, Fix&& fix,
                    For&& forEach = For()) {
    using std::sqrt;
    const int n = r.mesh.nv;
    const auto& p = r.p;
    std::vector<Triplet<NT>> tK, tD;
    const std::size_t nf = r.mesh.F.size();
    std::vector<std::array<NT, 81>> K9s(nf), D9s(nf);
    forEach(nf, [&](std::size_t fb, std::size_t fe) {
    for (std::size_t fi = fb; fi < fe; ++fi) {
        const auto& f = r.mesh.F[fi];
        const double a = r.area[fi];
        const auto& Vi = r.Vinv[fi];
        const auto& B = r.B[fi];
        auto Bf = [&](int i, int c) { return B[2 * i + c]; };
        // deformation gradient J = D * Vinv, D = [x1 - x0, x2 - x0]
        NT Dm[3][2], J[3][2];
        for (int d = 0; d < 3; ++d) {
            Dm[d][0] = X[f[1] + d * n] - X[f[0] + d * n];
            Dm[d][1] = X[f[2] + d * n] - X[f[0] + d * n];
        }
        for (int d = 0; d < 3; ++d)
            for (int c = 0; c < 2; ++c) J[d][c] = Dm[d][0] * NT(Vi[0 + c]) + Dm[d][1] * NT(Vi[2 + c]);
        NT Jnorm[2], Jn[3][2];
        for (int c = 0; c < 2; ++c) Jnorm[c] = sqrt(J[0][c] * J[0][c] + J[1][c] * J[1][c] + J[2][c] * J[2][c]);
        for (int d = 0; d < 3; ++d)
            for (int c = 0; c < 2; ++c) Jn[d][c] = J[d][c] / Jnorm[c];
        NT v[3][3];
        for (int i = 0; i < 3; ++i)
            for (int d = 0; d < 3; ++d) v[i][d] = Vel[f[i] + d * n];

        std::array<NT, 81>& K9 = K9s[fi];
        std::array<NT, 81>& D9 = D9s[fi];
        // stretch
        NT C[2] = {NT(a) * (Jnorm[0] - NT(1.0)), NT(a) * (Jnorm[1] - NT(1.0))};
        NT dC[3][3][2];  // dC[i][d][c]
        NT Cdot[2] = {NT(0.0), NT(0.0)};
        for (int i = 0; i < 3; ++i)
            for (int c = 0; c < 2; ++c) {
                for (int d = 0; d < 3; ++d) dC[i][d][c] = NT(a * Bf(i, c)) * Jn[d][c];
                Cdot[c] = Cdot[c] + (dC[i][0][c] * v[i][0] + dC[i][1][c] * v[i][1] + dC[i][2][c] * v[i][2]);
            }
        NT IJ[2][3][3];
        for (int c = 0; c < 2; ++c)
            for (int d = 0; d < 3; ++d)
                for (int e = 0; e < 3; ++e)
                    IJ[c][d][e] = NT(a) * (NT(d == e ? 1.0 : 0.0) - Jn[d][c] * Jn[e][c]) / Jnorm[c];
        // shear
        const NT Cs = NT(a) * (J[0][0] * J[0][1] + J[1][0] * J[1][1] + J[2][0] * J[2][1]);
        NT Cdv[3][3];  // Cdv[i][d]
        NT Cdots = NT(0.0);
        for (int i = 0; i < 3; ++i) {
            for (int d = 0; d < 3; ++d) Cdv[i][d] = NT(a) * (NT(Bf(i, 0)) * J[d][1] + NT(Bf(i, 1)) * J[d][0]);
            Cdots = Cdots + (Cdv[i][0] * v[i][0] + Cdv[i][1] * v[i][1] + Cdv[i][2] * v[i][2]);
        }
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                const double bx = Bf(i, 0) * Bf(j, 0), by = Bf(i, 1) * Bf(j, 1);
                const double dCdvdv = a * (Bf(i, 0) * Bf(j, 1) + Bf(i, 1) * Bf(j, 0));
                for (int d = 0; d < 3; ++d)
                    for (int e = 0; e < 3; ++e) {
                        const NT dxx = NT(bx) * IJ[0][d][e], dyy = NT(by) * IJ[1][d][e];
                        const NT outer = dC[i][d][0] * dC[j][e][0] + dC[i][d][1] * dC[j][e][1];
                        NT Ks = NT(-p.kStretch) * (outer + dxx * C[0] + dyy * C[1]);
                        NT KD = dxx * Cdot[0] + dyy * Cdot[1];
                        if (d == e) KD = NT(2.0) * KD;
                        Ks = Ks + NT(-p.kStretchDamping) * KD;
                        const NT Ds = NT(-p.kStretchDamping) * outer;
                        const NT so = Cdv[i][d] * Cdv[j][e];
                        NT Kh = so;
                        if (d == e) Kh = Kh + NT(dCdvdv) * Cs;
                        Kh = NT(-p.kShear) * Kh;
                        if (d == e) Kh = Kh + NT(-p.kShearDamping * dCdvdv) * Cdots;
                        const NT Dh = NT(-p.kShearDamping) * so;
                        K9[(3 * i + d) * 9 + 3 * j + e] = Ks + Kh;
                        D9[(3 * i + d) * 9 + 3 * j + e] = Ds + Dh;
                    }
            }
    }
    });
    using FixT = std::decay_t<Fix>;
    using ForT = std::decay_t<For>;
    if constexpr (HasBatchFix<FixT, std::array<NT, 81>, ForT>::value) {
        fix.batch(K9s, D9s, forEach);
    } else {
        for (std::size_t fi = 0; fi < nf; ++fi) fix(K9s[fi], D9s[fi]);
    }
    for (std::size_t fi = 0; fi < nf; ++fi) {
        const auto& f = r.mesh.F[fi];
        const std::array<NT, 81>& K9 = K9s[fi];
        const std::array<NT, 81>& D9 = D9s[fi];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int d = 0; d < 3; ++d)
                    for (int e = 0; e < 3; ++e) {
                        const int row = f[i] + d * n, col = f[j] + e * n;
                        if (row >= col) {
                            tK.push_back({row, col, K9[(3 * i + d) * 9 + 3 * j + e]});
                            tD.push_back({row, col, D9[(3 * i + d) * 9 + 3 * j + e]});
                        }
                    }
    }
    // With a worker pool, the faces' handles are dropped in parallel too (a
    // serial loop just lets the vectors go).
    constexpr bool kPooled = !std::is_same_v<std::decay_t<For>, SerialFor>;
    if constexpr (kPooled)
        forEach(nf, [&](std::size_t fb, std::size_t fe) {
            for (std::size_t fi = fb; fi < fe; ++fi) {
                K9s[fi] = {};
                D9s[fi] = {};
            }
        });
    K9s.clear();
    D9s.clear();
    // quadratic bend: constant stiffness k Q and damping kd Q per interior edge
    std::vector<Triplet<NT>> bK, bD;
    for (std::size_t e = 0; e < r.E4.size(); ++e)
        for (int dim = 0; dim < 3; ++dim)
            for (int v1 = 0; v1 < 4; ++v1)
                for (int v2 = 0; v2 <= v1; ++v2) {
                    const int i1 = r.E4[e][v1] + dim * n, i2 = r.E4[e][v2] + dim * n;
                    const double q = r.Q[e][4 * v1 + v2];
                    bK.push_back({i1, i2, NT(p.kBend * q)});
                    bD.push_back({i1, i2, NT(p.kBendDamping * q)});
                    if (v2 != v1) {
                        bK.push_back({i2, i1, NT(p.kBend * q)});
                        bD.push_back({i2, i1, NT(p.kBendDamping * q)});
                    }
                }
    const int N = 3 * n;
    CSC<NT> Kss = assemble(N, N, tK, forEach), Dss = assemble(N, N, tD, forEach), Kb = assemble(N, N, bK, forEach),
            Db = assemble(N, N, bD, forEach);
    tK.clear();
    tD.clear();
    // A = M - h (D + h K) on the union pattern, lower triangle.
    const double mass = p.totalMass / n;
    std::vector<std::map<int, NT>> Kc(N), Dc(N);
    auto addInto = [](std::vector<std::map<int, NT>>& dst, const CSC<NT>& S, std::size_t c) {
        for (int k = S.colPtr[c]; k < S.colPtr[c + 1]; ++k) {
            auto it = dst[c].find(S.rowIdx[k]);
            if (it == dst[c].end())
                dst[c].emplace(S.rowIdx[k], S.values[k]);
            else
                it->second = it->second + S.values[k];
        }
    };
    // Column by column (columns are independent).
    std::vector<std::vector<std::pair<int, NT>>> colA(N);
    forEach((std::size_t)N, [&](std::size_t cb, std::size_t ce) {
    for (std::size_t cc = cb; cc < ce; ++cc) {
        const int c = (int)cc;
        addInto(Kc, Kss, cc);
        addInto(Kc, Kb, cc);
        addInto(Dc, Dss, cc);
        addInto(Dc, Db, cc);
        std::map<int, int> rowsU;
        for (auto& e : Kc[c]) rowsU[e.first] |= 1;
        for (auto& e : Dc[c]) rowsU[e.first] |= 2;
        rowsU[c] |= 4;
        for (auto& ru : rowsU) {
            const int row = ru.first;
            if (row < c) continue;
            NT inner;
            if ((ru.second & 3) == 3)
                inner = Dc[c].at(row) + NT(p.h) * Kc[c].at(row);
            else if (ru.second & 1)
                inner = NT(p.h) * Kc[c].at(row);
            else if (ru.second & 2)
                inner = Dc[c].at(row);
            NT val;
            if (ru.second & 3) {
                const NT t = NT(p.h) * inner;
                val = (row == c) ? NT(mass) - t : -t;
            } else {
                val = NT(mass);
            }
            colA[c].emplace_back(row, std::move(val));
        }
        Kc[c].clear();
        Dc[c].clear();
    }
    });
    CSC<NT> A;
    A.rows = N;
    A.cols = N;
    A.colPtr.assign(N + 1, 0);
    for (int c = 0; c < N; ++c) A.colPtr[c + 1] = A.colPtr[c] + (int)colA[c].size();
    A.rowIdx.resize(A.colPtr[N]);
    A.values.resize(A.colPtr[N]);
    forEach((std::size_t)N, [&](std::size_t cb, std::size_t ce) {
        for (std::size_t c = cb; c < ce; ++c) {
            int k = A.colPtr[c];
            for (auto& e : colA[c]) {
                A.rowIdx[k] = e.first;
                A.values[k++] = std::move(e.second);
            }
            colA[c] = {};
        }
    });
    if constexpr (kPooled)
        for (CSC<NT>* M : {&Kss, &Dss, &Kb, &Db})  // the summands' handles, dropped in parallel too
            forEach(M->values.size(), [&](std::size_t b, std::size_t e) {
                for (std::size_t i = b; i < e; ++i) M->values[i] = NT();
            });
    return A;
}

// ---------------------------------------------------------------- workload 5: Neo-Hookean tets

// Tetrahedral mesh of a cells^3 cube grid at unit spacing, 5 tets per cell
// (the split alternates with cell parity so faces match), with rest-shape
// quantities.  The deformed state compresses z by 10% and adds uniform noise.
struct TetMesh {
    int nv = 0;
    std::vector<double> rest;                 // nv x 3 column-major
    std::vector<std::array<int, 4>> T;
    std::vector<std::array<double, 9>> Dminv; // per tet, 3x3 row-major inverse of [x1-x0, x2-x0, x3-x0]
    std::vector<double> volume;               // per tet, rest volume
    double mu = 1.0, lambda = 10.0;
};

inline TetMesh tetMesh(int cells) {
    TetMesh m;
    const int s = cells + 1;
    m.nv = s * s * s;
    m.rest.assign(3 * (std::size_t)m.nv, 0.0);
    auto vid = [&](int i, int j, int k) { return i + s * (j + s * k); };
    for (int k = 0; k < s; ++k)
        for (int j = 0; j < s; ++j)
            for (int i = 0; i < s; ++i) {
                const int v = vid(i, j, k);
                m.rest[v] = i;
                m.rest[v + m.nv] = j;
                m.rest[v + 2 * (std::size_t)m.nv] = k;
            }
    static const int split[5][4] = {{0, 1, 2, 4}, {3, 2, 1, 7}, {5, 4, 7, 1}, {6, 7, 4, 2}, {1, 2, 4, 7}};
    for (int k = 0; k < cells; ++k)
        for (int j = 0; j < cells; ++j)
            for (int i = 0; i < cells; ++i) {
                const int flip = (i + j + k) & 1;
                for (const auto& t : split) {
                    std::array<int, 4> tet;
                    for (int a = 0; a < 4; ++a) {
                        const int c = t[a] ^ flip;  // mirror the split in x for odd cells
                        tet[a] = vid(i + (c & 1), j + ((c >> 1) & 1), k + ((c >> 2) & 1));
                    }
                    double D[9];
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c)
                            D[3 * r + c] = m.rest[tet[c + 1] + r * (std::size_t)m.nv] - m.rest[tet[0] + r * (std::size_t)m.nv];
                    double det = D[0] * (D[4] * D[8] - D[5] * D[7]) - D[1] * (D[3] * D[8] - D[5] * D[6]) +
                                 D[2] * (D[3] * D[7] - D[4] * D[6]);
                    if (det < 0) {
                        std::swap(tet[1], tet[2]);
                        for (int r = 0; r < 3; ++r) std::swap(D[3 * r + 0], D[3 * r + 1]);
                        det = -det;
                    }
                    std::array<double, 9> inv;
                    inv[0] = (D[4] * D[8] - D[5] * D[7]) / det;
                    inv[1] = (D[2] * D[7] - D[1] * D[8]) / det;
                    inv[2] = (D[1] * D[5] - D[2] * D[4]) / det;
                    inv[3] = (D[5] * D[6] - D[3] * D[8]) / det;
                    inv[4] = (D[0] * D[8] - D[2] * D[6]) / det;
                    inv[5] = (D[2] * D[3] - D[0] * D[5]) / det;
                    inv[6] = (D[3] * D[7] - D[4] * D[6]) / det;
                    inv[7] = (D[1] * D[6] - D[0] * D[7]) / det;
                    inv[8] = (D[0] * D[4] - D[1] * D[3]) / det;
                    m.T.push_back(tet);
                    m.Dminv.push_back(inv);
                    m.volume.push_back(det / 6.0);
                }
            }
    return m;
}

inline std::vector<double> tetState(const TetMesh& m, std::uint64_t seed) {
    Rng rng(seed);
    std::vector<double> X(m.rest);
    for (int v = 0; v < m.nv; ++v) X[v + 2 * (std::size_t)m.nv] *= 0.9;
    for (auto& x : X) x += rng.uniform(-0.01, 0.01);
    return X;
}

// Per-tet energy V0 * psi(F), F = Ds Dm^-1, with the log-free Neo-Hookean
// psi = mu/2 (tr(F^T F) - 3) - mu (J - 1) + lambda/2 (J - 1)^2, J = det F
// (zero energy and stress at rest; no logarithm, whose derivative rule the
// symbolic differentiation does not have).
template <class NT>
std::vector<NT> neoHookeanEnergies(const TetMesh& m, const std::vector<NT>& X) {
    std::vector<NT> E;
    E.reserve(m.T.size());
    const std::size_t n = m.nv;
    for (std::size_t t = 0; t < m.T.size(); ++t) {
        const auto& tet = m.T[t];
        const auto& Mi = m.Dminv[t];
        NT Ds[3][3], F[3][3];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) Ds[r][c] = X[tet[c + 1] + r * n] - X[tet[0] + r * n];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) F[r][c] = Ds[r][0] * NT(Mi[c]) + Ds[r][1] * NT(Mi[3 + c]) + Ds[r][2] * NT(Mi[6 + c]);
        NT Ic = F[0][0] * F[0][0];
        for (int q = 1; q < 9; ++q) Ic = Ic + F[q / 3][q % 3] * F[q / 3][q % 3];
        const NT J = F[0][0] * (F[1][1] * F[2][2] - F[1][2] * F[2][1]) - F[0][1] * (F[1][0] * F[2][2] - F[1][2] * F[2][0]) +
                     F[0][2] * (F[1][0] * F[2][1] - F[1][1] * F[2][0]);
        const NT Jm1 = J - NT(1.0);
        const NT psi = NT(0.5 * m.mu) * (Ic - NT(3.0)) - NT(m.mu) * Jm1 + NT(0.5 * m.lambda) * (Jm1 * Jm1);
        E.push_back(NT(m.volume[t]) * psi);
    }
    return E;
}

// Symmetric Hessian from upper-triangle (row, col, value) entries: each
// off-diagonal entry is also added transposed, duplicates summed in order.
template <class NT, class For = SerialFor>
CSC<NT> symmetricFromUpper(int n, const std::vector<std::tuple<int, int, NT>>& upper, For&& forEach = For()) {
    std::vector<Triplet<NT>> t;
    t.reserve(2 * upper.size());
    for (const auto& e : upper) t.push_back({std::get<0>(e), std::get<1>(e), std::get<2>(e)});
    for (const auto& e : upper)
        if (std::get<0>(e) != std::get<1>(e)) t.push_back({std::get<1>(e), std::get<0>(e), std::get<2>(e)});
    return assemble(n, n, t, forEach);
}

// Analytic FP64 Hessian of the same energy (the numeric oracle of workload 5):
// d2psi/dF_rc dF_pq = mu d_rp d_cq + lambda C_rc C_pq + (lambda (J-1) - mu) e_rpb e_cqe F_be,
// C = cof(F), mapped to the tet's 12 coordinates through dF_rc/dx_(v,d) = d_rd G_vc.
inline std::vector<std::tuple<int, int, double>> neoHookeanHessianUpper(const TetMesh& m, const std::vector<double>& X) {
    std::vector<std::tuple<int, int, double>> out;
    const std::size_t n = m.nv;
    auto eps = [](int a, int b, int c) { return (a == b || b == c || a == c) ? 0 : (((b - a + 3) % 3 == 1) ? 1 : -1); };
    for (std::size_t t = 0; t < m.T.size(); ++t) {
        const auto& tet = m.T[t];
        const auto& Mi = m.Dminv[t];
        double Ds[3][3], F[3][3], C[3][3], G[4][3];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) Ds[r][c] = X[tet[c + 1] + r * n] - X[tet[0] + r * n];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) F[r][c] = Ds[r][0] * Mi[c] + Ds[r][1] * Mi[3 + c] + Ds[r][2] * Mi[6 + c];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c)
                C[r][c] = F[(r + 1) % 3][(c + 1) % 3] * F[(r + 2) % 3][(c + 2) % 3] -
                          F[(r + 1) % 3][(c + 2) % 3] * F[(r + 2) % 3][(c + 1) % 3];
        const double J = F[0][0] * C[0][0] + F[0][1] * C[0][1] + F[0][2] * C[0][2];
        for (int c = 0; c < 3; ++c) {
            G[0][c] = -(Mi[c] + Mi[3 + c] + Mi[6 + c]);
            for (int v = 1; v < 4; ++v) G[v][c] = Mi[3 * (v - 1) + c];
        }
        double HF[9][9];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c)
                for (int p = 0; p < 3; ++p)
                    for (int q = 0; q < 3; ++q) {
                        double dC = 0.0;
                        for (int b = 0; b < 3; ++b)
                            for (int e = 0; e < 3; ++e) dC += eps(r, p, b) * eps(c, q, e) * F[b][e];
                        HF[3 * r + c][3 * p + q] = m.mu * (r == p && c == q) + m.lambda * C[r][c] * C[p][q] +
                                                   (m.lambda * (J - 1.0) - m.mu) * dC;
                    }
        for (int v = 0; v < 4; ++v)
            for (int d = 0; d < 3; ++d)
                for (int w = 0; w < 4; ++w)
                    for (int e = 0; e < 3; ++e) {
                        const int gi = tet[v] + d * (int)n, gj = tet[w] + e * (int)n;
                        if (gi > gj) continue;
                        double h = 0.0;
                        for (int c = 0; c < 3; ++c)
                            for (int q = 0; q < 3; ++q) h += G[v][c] * G[w][q] * HF[3 * d + c][3 * e + q];
                        out.emplace_back(gi, gj, m.volume[t] * h);
                    }
    }
    return out;
}

// ---------------------------------------------------------------- random expression workloads

// Random expression DAGs for training the schedule cost model.  `nShared`
// random sub-expressions over the inputs are shared by the outputs (they
// become intermediate blocks and dependency levels); each output applies one
// of a few random template shapes to random inputs and shared values.  Shapes
// mix sums, products, quotients and square roots of well-conditioned operands.
template <class NT>
struct RandomShape {
    // post-order op list: 0 leaf, 1 add, 2 sub, 3 mul, 4 div, 5 sqrt-of-sum-of-squares
    std::vector<int> ops;
};

inline RandomShape<double> randomShape(Rng& rng, int depth) {
    RandomShape<double> s;
    std::function<void(int)> gen = [&](int d) {
        if (d == 0 || (d < depth && rng.uniform() < 0.25)) {  // the root is always an operation
            s.ops.push_back(0);
            return;
        }
        const int op = 1 + (int)rng.below(5);
        gen(d - 1);
        gen(d - 1);
        s.ops.push_back(op);
    };
    gen(depth);
    return s;
}

template <class NT, class Leaf>
NT applyShape(const RandomShape<double>& s, Leaf&& leaf) {
    std::vector<NT> st;
    for (int op : s.ops) {
        if (op == 0) {
            st.push_back(leaf());
            continue;
        }
        NT b = st.back();
        st.pop_back();
        NT a = st.back();
        st.pop_back();
        using std::sqrt;
        switch (op) {
            case 1: st.push_back(a + b); break;
            case 2: st.push_back(a - b); break;
            case 3: st.push_back(a * b); break;
            case 4: st.push_back(a / (b * b + NT(1.0))); break;
            default: st.push_back(sqrt(a * a + b * b + NT(1.0))); break;
        }
    }
    return st.back();
}

// Sums of `terms` products literal_k * in[...], the same literals in every
// output, so one kernel template holds `terms` distinct literals (more than a
// program loads up front: the rest stay literal-load entries).
template <class NT>
std::vector<NT> literalSums(const std::vector<NT>& in, int outputs, int terms) {
    const int m = (int)in.size();
    std::vector<NT> out;
    out.reserve(outputs);
    for (int o = 0; o < outputs; ++o) {
        NT s = NT(1.0 + 1.0 / 3.0) * in[(o * 13) % m];
        for (int k = 1; k < terms; ++k) s = s + NT(1.0 + 0.125 * k + 1.0 / (k + 3)) * in[(o * 13 + k * 7) % m];
        out.push_back(s);
    }
    return out;
}

template <class NT>
std::vector<NT> randomExpressions(const std::vector<NT>& in, int outputs, std::uint64_t seed) {
    Rng rng(seed);
    const int nShapes = 1 + (int)rng.below(4), nShared = (int)rng.below(3) * (outputs / 8 + 1);
    std::vector<RandomShape<double>> shapes;
    for (int k = 0; k < nShapes; ++k) shapes.push_back(randomShape(rng, 2 + (int)rng.below(4)));
    const RandomShape<double> sharedShape = randomShape(rng, 2 + (int)rng.below(3));
    const int m = (int)in.size();
    std::vector<NT> shared;
    for (int k = 0; k < nShared; ++k)
        shared.push_back(applyShape<NT>(sharedShape, [&]() { return in[rng.below((std::uint64_t)m)]; }));
    std::vector<NT> out;
    out.reserve(outputs);
    for (int o = 0; o < outputs; ++o) {
        const auto& sh = shapes[rng.below((std::uint64_t)nShapes)];
        out.push_back(applyShape<NT>(sh, [&]() {
            if (!shared.empty() && rng.uniform() < 0.3) return shared[rng.below(shared.size())];
            return in[rng.below((std::uint64_t)m)];
        }));
    }
    return out;
}

}  // namespace symgb_workloads
