// Batched preconditioned Krylov solves on the device, for the step
// after assembly: solving A x = b with the cloth system matrix the engine
// evaluates (reference examples/BaraffWitkin/implementation/cloth.cpp:96-111
// assembles A = M - h (D + h K) and b; examples/BaraffWitkin/main.cpp:56 keeps
// its lower triangle, which is what the engine's cloth workload outputs).
// Conjugate gradient needs A positive definite; the cloth matrices of a
// stretched and compressed sheet are symmetric but indefinite (negative
// diagonal entries occur), for which BiCGSTAB is provided.  The default
// preconditioner scales by 1 / |A_ii| (equal to Jacobi for a positive definite
// A; with the signed diagonal of an indefinite A, BiCGSTAB breaks down);
// BiCGSTAB can instead use block Jacobi with the exact inverses of the b x b
// diagonal blocks of one node's unknowns (b = 3 for the cloth: a vertex's x, y
// and z rows, which the cloth matrix stores n apart).
//
// The pattern (lower-triangle or full CSC) is turned once into a full CSR
// with, per CSR entry, the index of its value in the engine's result buffer.
// Each solve gathers the values of all S systems into [entry][set] order and
// iterates on vectors laid out [row][set], so threads along the set index
// read contiguous memory.  Per-set scalars (step lengths, dot products) live on
// the device; the host looks at the residuals every kCheck iterations.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "symgb.h"
#include "unit.hpp"

namespace {

constexpr int kThreads = 256;
constexpr int kCheck = 16;  // iterations between host convergence checks

// vals[e * S + s] = in[s * nIn + src[e]]
__global__ void gatherValues(const double* __restrict__ in, std::uint64_t nIn, const std::int64_t* __restrict__ src,
                             std::uint64_t nnz, unsigned S, double* __restrict__ vals) {
    const std::uint64_t t = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nnz * S) return;
    const std::uint64_t e = t / S;
    const unsigned s = (unsigned)(t - e * S);
    vals[t] = in[(std::uint64_t)s * nIn + (std::uint64_t)src[e]];
}

// Start: x = 0, r = b, z = p = r / diag; rz = r.z, bb = b.b.
__global__ void cgStart(const double* __restrict__ b, const double* __restrict__ vals,
                        const std::int64_t* __restrict__ diagPos, std::uint64_t n, unsigned S, double* __restrict__ x,
                        double* __restrict__ r, double* __restrict__ p, double* __restrict__ invDiag,
                        double* __restrict__ rz, double* __restrict__ bb) {
    extern __shared__ double red[];
    for (unsigned q = threadIdx.x; q < 2 * S; q += blockDim.x) red[q] = 0.0;
    __syncthreads();
    const std::uint64_t t = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double vrz = 0.0, vbb = 0.0;
    unsigned s = 0;
    if (t < n * S) {
        const std::uint64_t i = t / S;
        s = (unsigned)(t - i * S);
        const double bi = b[(std::uint64_t)s * n + i];
        const double d = diagPos[i] >= 0 ? vals[(std::uint64_t)diagPos[i] * S + s] : 0.0;
        const double inv = d != 0.0 ? 1.0 / fabs(d) : 1.0;
        x[t] = 0.0;
        r[t] = bi;
        p[t] = bi * inv;
        invDiag[t] = inv;
        vrz = bi * bi * inv;
        vbb = bi * bi;
    }
    if (vrz != 0.0) atomicAdd(&red[s], vrz);
    if (vbb != 0.0) atomicAdd(&red[S + s], vbb);
    __syncthreads();
    for (unsigned q = threadIdx.x; q < S; q += blockDim.x) {
        if (red[q] != 0.0) atomicAdd(&rz[q], red[q]);
        if (red[S + q] != 0.0) atomicAdd(&bb[q], red[S + q]);
    }
}

// q = A p, pq += p.q
__global__ void cgSpmv(const std::int64_t* __restrict__ rowPtr, const int* __restrict__ col,
                       const double* __restrict__ vals, const double* __restrict__ p, std::uint64_t n, unsigned S,
                       double* __restrict__ q, double* __restrict__ pq) {
    extern __shared__ double red[];
    for (unsigned k = threadIdx.x; k < S; k += blockDim.x) red[k] = 0.0;
    __syncthreads();
    const std::uint64_t t = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    unsigned s = 0;
    if (t < n * S) {
        const std::uint64_t i = t / S;
        s = (unsigned)(t - i * S);
        double acc = 0.0;
        for (std::int64_t e = rowPtr[i]; e < rowPtr[i + 1]; ++e)
            acc = fma(vals[(std::uint64_t)e * S + s], p[(std::uint64_t)col[e] * S + s], acc);
        q[t] = acc;
        v = acc * p[t];
    }
    if (v != 0.0) atomicAdd(&red[s], v);
    __syncthreads();
    for (unsigned k = threadIdx.x; k < S; k += blockDim.x)
        if (red[k] != 0.0) atomicAdd(&pq[k], red[k]);
}

// alpha = rz / pq; x += alpha p; r -= alpha q; rzNew += r.(r / diag); rr += r.r
__global__ void cgUpdate(const double* __restrict__ p, const double* __restrict__ q, const double* __restrict__ invDiag,
                         std::uint64_t n, unsigned S, const double* __restrict__ rz, const double* __restrict__ pq,
                         double* __restrict__ x, double* __restrict__ r, double* __restrict__ rzNew,
                         double* __restrict__ rr) {
    extern __shared__ double red[];
    for (unsigned k = threadIdx.x; k < 2 * S; k += blockDim.x) red[k] = 0.0;
    __syncthreads();
    const std::uint64_t t = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0.0, c = 0.0;
    unsigned s = 0;
    if (t < n * S) {
        s = (unsigned)(t % S);
        const double alpha = pq[s] != 0.0 ? rz[s] / pq[s] : 0.0;
        x[t] = fma(alpha, p[t], x[t]);
        const double ri = fma(-alpha, q[t], r[t]);
        r[t] = ri;
        a = ri * ri * invDiag[t];
        c = ri * ri;
    }
    if (a != 0.0) atomicAdd(&red[s], a);
    if (c != 0.0) atomicAdd(&red[S + s], c);
    __syncthreads();
    for (unsigned k = threadIdx.x; k < S; k += blockDim.x) {
        if (red[k] != 0.0) atomicAdd(&rzNew[k], red[k]);
        if (red[S + k] != 0.0) atomicAdd(&rr[k], red[S + k]);
    }
}

// p = r / diag + beta p with beta = rzNew / rz
__global__ void cgDirection(const double* __restrict__ r, const double* __restrict__ invDiag, std::uint64_t n,
                            unsigned S, const double* __restrict__ rz, const double* __restrict__ rzNew,
                            double* __restrict__ p) {
    const std::uint64_t t = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * S) return;
    const unsigned s = (unsigned)(t % S);
    const double beta = rz[s] != 0.0 ? rzNew[s] / rz[s] : 0.0;
    p[t] = fma(beta, p[t], r[t] * invDiag[t]);
}

// out[s * n + i] = x[i * S + s]
__global__ void cgFinish(const double* __restrict__ x, std::uint64_t n, unsigned S, double* __restrict__ out) {
    const std::uint64_t t = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * S) return;
    const std::uint64_t s = t / n, i = t - s * n;
    out[t] = x[i * S + s];
}

// ---------------------------------------------------------------- BiCGSTAB
// Jacobi right-preconditioned BiCGSTAB (van der Vorst).  Scalars per set:
// R[3] ring of rho = rhat.r (R[it % 3] current, R[(it + 2) % 3] previous,
// R[(it + 1) % 3] accumulated for the next iteration), rv, ts, tt, rr, bb,
// alpha, omega.

// x = 0, r = rhat = b, p = v = 0, invDiag; R[0] = bb = b.b, R[2] = 1
__global__ void bStart(const double* __restrict__ b, const double* __restrict__ vals,
                       const std::int64_t* __restrict__ diagPos, std::uint64_t n, unsigned S, double* __restrict__ x,
                       double* __restrict__ r, double* __restrict__ rhat, double* __restrict__ p,
                       double* __restrict__ v, double* __restrict__ invDiag, double* __restrict__ R0,
                       double* __restrict__ bb) {
    extern __shared__ double red[];
    for (unsigned q = threadIdx.x; q < S; q += blockDim.x) red[q] = 0.0;
    __syncthreads();
    const std::uint64_t t = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double vbb = 0.0;
    unsigned s = 0;
    if (t < n * S) {
        const std::uint64_t i = t / S;
        s = (unsigned)(t - i * S);
        const double bi = b[(std::uint64_t)s * n + i];
        const double d = diagPos[i] >= 0 ? vals[(std::uint64_t)diagPos[i] * S + s] : 0.0;
        x[t] = 0.0;
        r[t] = bi;
        rhat[t] = bi;
        p[t] = 0.0;
        v[t] = 0.0;
        invDiag[t] = d != 0.0 ? 1.0 / fabs(d) : 1.0;
        vbb = bi * bi;
    }
    if (vbb != 0.0) atomicAdd(&red[s], vbb);
    __syncthreads();
    for (unsigned q = threadIdx.x; q < S; q += blockDim.x)
        if (red[q] != 0.0) {
            atomicAdd(&R0[q], red[q]);
            atomicAdd(&bb[q], red[q]);
        }
}

// p = r + beta (p - omega v), beta = (rho / rhoPrev) (alpha / omega); ph = p / diag
__global__ void bDirection(const double* __restrict__ r, const double* __restrict__ v,
                           const double* __restrict__ invDiag, std::uint64_t n, unsigned S,
                           const double* __restrict__ rho, const double* __restrict__ rhoPrev,
                           const double* __restrict__ alpha, const double* __restrict__ omega, double* __restrict__ p,
                           double* __restrict__ ph) {
    const std::uint64_t t = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * S) return;
    const unsigned s = (unsigned)(t % S);
    const double den = rhoPrev[s] * omega[s];
    const double beta = den != 0.0 ? (rho[s] * alpha[s]) / den : 0.0;
    const double pi = fma(beta, fma(-omega[s], v[t], p[t]), r[t]);
    p[t] = pi;
    ph[t] = pi * invDiag[t];
}

// y = A z, d1 += w1.y, d2 += y.y (w1, d2 optional)
__global__ void bSpmv(const std::int64_t* __restrict__ rowPtr, const int* __restrict__ col,
                      const double* __restrict__ vals, const double* __restrict__ z, std::uint64_t n, unsigned S,
                      const double* __restrict__ w1, double* __restrict__ y, double* __restrict__ d1,
                      double* __restrict__ d2) {
    extern __shared__ double red[];
    for (unsigned k = threadIdx.x; k < 2 * S; k += blockDim.x) red[k] = 0.0;
    __syncthreads();
    const std::uint64_t t = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0.0, c = 0.0;
    unsigned s = 0;
    if (t < n * S) {
        const std::uint64_t i = t / S;
        s = (unsigned)(t - i * S);
        double acc = 0.0;
        for (std::int64_t e = rowPtr[i]; e < rowPtr[i + 1]; ++e)
            acc = fma(vals[(std::uint64_t)e * S + s], z[(std::uint64_t)col[e] * S + s], acc);
        y[t] = acc;
        a = acc * w1[t];
        c = acc * acc;
    }
    if (a != 0.0) atomicAdd(&red[s], a);
    if (d2 && c != 0.0) atomicAdd(&red[S + s], c);
    __syncthreads();
    for (unsigned k = threadIdx.x; k < S; k += blockDim.x) {
        if (red[k] != 0.0) atomicAdd(&d1[k], red[k]);
        if (d2 && red[S + k] != 0.0) atomicAdd(&d2[k], red[S + k]);
    }
}

// alpha = rho / rv; s = r - alpha v; sh = s / diag
__global__ void bHalf(const double* __restrict__ r, const double* __restrict__ v, const double* __restrict__ invDiag,
                      std::uint64_t n, unsigned S, const double* __restrict__ rho, const double* __restrict__ rv,
                      double* __restrict__ alpha, double* __restrict__ sv, double* __restrict__ sh) {
    const std::uint64_t t = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * S) return;
    const unsigned s = (unsigned)(t % S);
    const double a = rv[s] != 0.0 ? rho[s] / rv[s] : 0.0;
    if (t < S) alpha[s] = a;  // row 0 of each set records it
    const double si = fma(-a, v[t], r[t]);
    sv[t] = si;
    sh[t] = si * invDiag[t];
}

// omega = ts / tt; x += alpha ph + omega sh; r = s - omega t; rhoNext += rhat.r; rr += r.r
__global__ void bFinishStep(const double* __restrict__ ph, const double* __restrict__ sh, const double* __restrict__ sv,
                            const double* __restrict__ tv, const double* __restrict__ rhat, std::uint64_t n, unsigned S,
                            const double* __restrict__ alpha, const double* __restrict__ ts,
                            const double* __restrict__ tt, double* __restrict__ omega, double* __restrict__ x,
                            double* __restrict__ r, double* __restrict__ rhoNext, double* __restrict__ rr) {
    extern __shared__ double red[];
    for (unsigned k = threadIdx.x; k < 2 * S; k += blockDim.x) red[k] = 0.0;
    __syncthreads();
    const std::uint64_t t = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0.0, c = 0.0;
    unsigned s = 0;
    if (t < n * S) {
        s = (unsigned)(t % S);
        const double om = tt[s] != 0.0 ? ts[s] / tt[s] : 0.0;
        if (t < S) omega[s] = om;
        x[t] = fma(om, sh[t], fma(alpha[s], ph[t], x[t]));
        const double ri = fma(-om, tv[t], sv[t]);
        r[t] = ri;
        a = rhat[t] * ri;
        c = ri * ri;
    }
    if (a != 0.0) atomicAdd(&red[s], a);
    if (c != 0.0) atomicAdd(&red[S + s], c);
    __syncthreads();
    for (unsigned k = threadIdx.x; k < S; k += blockDim.x) {
        if (red[k] != 0.0) atomicAdd(&rhoNext[k], red[k]);
        if (red[S + k] != 0.0) atomicAdd(&rr[k], red[S + k]);
    }
}

// ---------------------------------------------------------------- block Jacobi
// Blocks of B unknowns: block j holds rows j * B + a (stride 1, unknowns of one
// node stored together) or j + a * stride (stride n / B, each coordinate's
// unknowns stored together, as the cloth matrix orders them).

__device__ __forceinline__ std::uint64_t blockRow(std::uint64_t j, int a, int B, std::uint64_t stride) {
    return stride == 1 ? j * (std::uint64_t)B + (std::uint64_t)a : j + (std::uint64_t)a * stride;
}

// inv[(j * B * B + a * B + c) * S + s] = (A_jj^-1)[a][c] of set s, by Gauss-Jordan
// elimination with partial pivoting; a block with a zero pivot takes the
// inverse of its absolute diagonal instead (the scaled-Jacobi fallback).
template <int B>
__global__ void blockInvert(const double* __restrict__ vals, const std::int64_t* __restrict__ pos, std::uint64_t nb,
                            unsigned S, double* __restrict__ inv) {
    const std::uint64_t t = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nb * S) return;
    const std::uint64_t j = t / S;
    const unsigned s = (unsigned)(t - j * S);
    double m[B][2 * B];
#pragma unroll
    for (int a = 0; a < B; ++a)
#pragma unroll
        for (int c = 0; c < B; ++c) {
            const std::int64_t e = pos[j * B * B + a * B + c];
            m[a][c] = e >= 0 ? vals[(std::uint64_t)e * S + s] : 0.0;
            m[a][B + c] = a == c ? 1.0 : 0.0;
        }
    bool singular = false;
#pragma unroll
    for (int c = 0; c < B; ++c) {
        int piv = c;
#pragma unroll
        for (int a = c + 1; a < B; ++a)
            if (fabs(m[a][c]) > fabs(m[piv][c])) piv = a;
        if (m[piv][c] == 0.0) {
            singular = true;
            break;
        }
#pragma unroll
        for (int q = 0; q < 2 * B; ++q) {
            const double tmp = m[c][q];
            m[c][q] = m[piv][q];
            m[piv][q] = tmp;
        }
        const double d = 1.0 / m[c][c];
#pragma unroll
        for (int q = 0; q < 2 * B; ++q) m[c][q] *= d;
#pragma unroll
        for (int a = 0; a < B; ++a)
            if (a != c) {
                const double f = m[a][c];
#pragma unroll
                for (int q = 0; q < 2 * B; ++q) m[a][q] = fma(-f, m[c][q], m[a][q]);
            }
    }
#pragma unroll
    for (int a = 0; a < B; ++a)
#pragma unroll
        for (int c = 0; c < B; ++c) {
            double v;
            if (!singular) {
                v = m[a][B + c];
            } else {
                const std::int64_t e = pos[j * B * B + a * B + a];
                const double d = e >= 0 ? vals[(std::uint64_t)e * S + s] : 0.0;
                v = a == c ? (d != 0.0 ? 1.0 / fabs(d) : 1.0) : 0.0;
            }
            inv[(j * B * B + a * B + c) * S + s] = v;
        }
}

// y = M^-1 x with M the block diagonal of A (vectors [row][set]).
template <int B>
__global__ void blockApply(const double* __restrict__ inv, const double* __restrict__ x, std::uint64_t n,
                           std::uint64_t stride, unsigned S, double* __restrict__ y) {
    const std::uint64_t t = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * S) return;
    const std::uint64_t i = t / S;
    const unsigned s = (unsigned)(t - i * S);
    const std::uint64_t j = stride == 1 ? i / B : i % stride;
    const int a = stride == 1 ? (int)(i % B) : (int)(i / stride);
    double acc = 0.0;
#pragma unroll
    for (int c = 0; c < B; ++c)
        acc = fma(inv[(j * B * B + a * B + c) * S + s], x[blockRow(j, c, B, stride) * S + s], acc);
    y[t] = acc;
}

unsigned blocksFor(std::uint64_t work) { return (unsigned)((work + kThreads - 1) / kThreads); }

void blockInvertLaunch(int B, const double* vals, const std::int64_t* pos, std::uint64_t nb, unsigned S, double* inv,
                       cudaStream_t st) {
    const unsigned g = blocksFor(nb * S);
    switch (B) {
        case 2: blockInvert<2><<<g, kThreads, 0, st>>>(vals, pos, nb, S, inv); break;
        case 3: blockInvert<3><<<g, kThreads, 0, st>>>(vals, pos, nb, S, inv); break;
        default: blockInvert<4><<<g, kThreads, 0, st>>>(vals, pos, nb, S, inv); break;
    }
}

void blockApplyLaunch(int B, const double* inv, const double* x, std::uint64_t n, std::uint64_t stride, unsigned S,
                      double* y, cudaStream_t st) {
    const unsigned g = blocksFor(n * S);
    switch (B) {
        case 2: blockApply<2><<<g, kThreads, 0, st>>>(inv, x, n, stride, S, y); break;
        case 3: blockApply<3><<<g, kThreads, 0, st>>>(inv, x, n, stride, S, y); break;
        default: blockApply<4><<<g, kThreads, 0, st>>>(inv, x, n, stride, S, y); break;
    }
}

}  // namespace

struct symgb_solver {
    std::uint64_t n = 0, nnzIn = 0, nnzFull = 0;
    unsigned S = 1;
    symgb::engine::DevBuf<std::int64_t> rowPtr, src, diagPos;
    symgb::engine::DevBuf<int> col;
    symgb::engine::DevBuf<double> vals, x, r, p, q, invDiag, scalars, rhat, v, ph, sv, sh, t;
    double* hostScalars = nullptr;  // pinned copy of rr and bb
    // Host copy of the full CSR (block positions) and the block preconditioner.
    std::vector<std::int64_t> rowPtrHost;
    std::vector<int> colHost;
    int block = 1;                  // unknowns per block (1: scaled Jacobi)
    std::uint64_t blockStride = 1;  // 1: contiguous blocks; n / block: one unknown per coordinate group
    symgb::engine::DevBuf<std::int64_t> blockPos;
    symgb::engine::DevBuf<double> blockInv;
    ~symgb_solver() {
        if (hostScalars) cudaFreeHost(hostScalars);
    }
};

extern "C" {

int symgb_solver_create(int64_t n, const int64_t* col_ptr, const int32_t* row_idx, int lower_only, int num_sets,
                    symgb_solver_t* out) {
    using symgb::engine::setLastError;
    if (!out || !col_ptr || n < 1 || num_sets < 1 || num_sets > kThreads)
        return setLastError(SYMGB_ERR_ARGUMENT, "solver: bad argument (num_sets 1..256)");
    const std::uint64_t nnzIn = (std::uint64_t)col_ptr[n];
    if (nnzIn && !row_idx) return setLastError(SYMGB_ERR_ARGUMENT, "solver: null row indices");
    // Full CSR of the symmetric matrix, entry -> input value index.
    std::vector<std::vector<std::pair<int, std::int64_t>>> rows((std::size_t)n);
    std::vector<std::int64_t> diag((std::size_t)n, -1);
    for (std::int64_t j = 0; j < n; ++j) {
        if (col_ptr[j] > col_ptr[j + 1]) return setLastError(SYMGB_ERR_ARGUMENT, "solver: column pointers decrease");
        for (std::int64_t e = col_ptr[j]; e < col_ptr[j + 1]; ++e) {
            const int i = row_idx[e];
            if (i < 0 || i >= n) return setLastError(SYMGB_ERR_ARGUMENT, "solver: row index out of range");
            if (lower_only && i < j) return setLastError(SYMGB_ERR_ARGUMENT, "solver: entry above the diagonal");
            rows[(std::size_t)i].push_back({(int)j, e});
            if (i != j && lower_only) rows[(std::size_t)j].push_back({i, e});
        }
    }
    // diag[i]: the CSR position of entry (i, i), -1 if the pattern has none
    std::vector<std::int64_t> rowPtr(1, 0), src;
    std::vector<int> col;
    for (std::size_t i = 0; i < rows.size(); ++i) {
        auto& rw = rows[i];
        std::sort(rw.begin(), rw.end());
        diag[i] = -1;
        for (auto& c : rw) {
            if (c.first == (int)i) diag[i] = (std::int64_t)col.size();
            col.push_back(c.first);
            src.push_back(c.second);
        }
        rowPtr.push_back((std::int64_t)col.size());
    }
    auto* s = new symgb_solver();
    s->n = (std::uint64_t)n;
    s->nnzIn = nnzIn;
    s->nnzFull = col.size();
    s->S = (unsigned)num_sets;
    const std::uint64_t work = s->n * s->S;
    auto fail = [&](const char* what) {
        delete s;
        return setLastError(SYMGB_ERR_NOMEM, std::string("solver: ") + what);
    };
    if (s->rowPtr.alloc(rowPtr.size()) || s->src.alloc(src.size()) || s->col.alloc(col.size()) ||
        s->diagPos.alloc(diag.size()) || s->vals.alloc(s->nnzFull * s->S) || s->x.alloc(work) || s->r.alloc(work) ||
        s->p.alloc(work) || s->q.alloc(work) || s->invDiag.alloc(work) || s->scalars.alloc(16 * (std::size_t)s->S))
        return fail("device allocation failed");
    if (cudaMallocHost(&s->hostScalars, 2 * s->S * sizeof(double)) != cudaSuccess) return fail("pinned allocation failed");
    cudaMemcpy(s->rowPtr.ptr, rowPtr.data(), rowPtr.size() * 8, cudaMemcpyHostToDevice);
    if (!src.empty()) cudaMemcpy(s->src.ptr, src.data(), src.size() * 8, cudaMemcpyHostToDevice);
    if (!col.empty()) cudaMemcpy(s->col.ptr, col.data(), col.size() * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(s->diagPos.ptr, diag.data(), diag.size() * 8, cudaMemcpyHostToDevice);
    if (cudaGetLastError() != cudaSuccess) return fail("upload failed");
    s->rowPtrHost = std::move(rowPtr);
    s->colHost = std::move(col);
    *out = s;
    return SYMGB_OK;
}

int symgb_solver_set_block_preconditioner(symgb_solver_t s, int block_size, int64_t stride) {
    using symgb::engine::setLastError;
    if (!s || block_size < 1 || block_size > 4) return setLastError(SYMGB_ERR_ARGUMENT, "solver: block size 1..4");
    if (block_size == 1) {
        s->block = 1;
        return SYMGB_OK;
    }
    const std::uint64_t n = s->n, B = (std::uint64_t)block_size;
    if (n % B) return setLastError(SYMGB_ERR_ARGUMENT, "solver: unknowns not a multiple of the block size");
    if (stride != 1 && (std::uint64_t)stride * B != n)
        return setLastError(SYMGB_ERR_ARGUMENT, "solver: stride must be 1 or n / block_size");
    const std::uint64_t nb = n / B;
    auto row = [&](std::uint64_t j, std::uint64_t a) { return stride == 1 ? j * B + a : j + a * (std::uint64_t)stride; };
    std::vector<std::int64_t> pos(nb * B * B, -1);
    for (std::uint64_t j = 0; j < nb; ++j)
        for (std::uint64_t a = 0; a < B; ++a) {
            const std::uint64_t r = row(j, a);
            const int* b = s->colHost.data() + s->rowPtrHost[r];
            const int* e = s->colHost.data() + s->rowPtrHost[r + 1];
            for (std::uint64_t c = 0; c < B; ++c) {
                const int* f = std::lower_bound(b, e, (int)row(j, c));
                if (f != e && *f == (int)row(j, c)) pos[(j * B + a) * B + c] = (std::int64_t)(f - s->colHost.data());
            }
        }
    if (s->blockPos.alloc(pos.size()) || s->blockInv.alloc(pos.size() * s->S))
        return setLastError(SYMGB_ERR_NOMEM, "solver: device allocation failed");
    if (cudaMemcpy(s->blockPos.ptr, pos.data(), pos.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess)
        return setLastError(SYMGB_ERR_CUDA, "solver: upload failed");
    s->block = block_size;
    s->blockStride = (std::uint64_t)stride;
    return SYMGB_OK;
}

int symgb_solver_multiply(symgb_solver_t s, const double* values, const double* p_dev, double* q_dev, void* stream) {
    using symgb::engine::setLastError;
    if (!s || !values || !p_dev || !q_dev) return setLastError(SYMGB_ERR_ARGUMENT, "solver: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    const std::uint64_t work = s->n * s->S;
    gatherValues<<<blocksFor(s->nnzFull * s->S), kThreads, 0, st>>>(values, s->nnzIn, s->src.ptr, s->nnzFull, s->S,
                                                                    s->vals.ptr);
    // p_dev and q_dev are [set][row]; the same transpose kernel with the roles
    // of rows and sets swapped gives the [row][set] copy of p.
    cgFinish<<<blocksFor(work), kThreads, 0, st>>>(p_dev, s->S, (unsigned)s->n, s->p.ptr);
    cudaMemsetAsync(s->scalars.ptr, 0, 8 * s->S * sizeof(double), st);
    cgSpmv<<<blocksFor(work), kThreads, s->S * sizeof(double), st>>>(s->rowPtr.ptr, s->col.ptr, s->vals.ptr, s->p.ptr,
                                                                      s->n, s->S, s->q.ptr, s->scalars.ptr);
    cgFinish<<<blocksFor(work), kThreads, 0, st>>>(s->q.ptr, s->n, s->S, q_dev);
    if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess)
        return setLastError(SYMGB_ERR_CUDA, "solver: multiply failed");
    return SYMGB_OK;
}

static int solveCg(symgb_solver_t s, const double* values, const double* b_dev, double* x_dev, double tol, int max_iter,
                   void* stream, int* iterations, double* max_rel_residual) {
    using symgb::engine::setLastError;
    if (!s || !values || !b_dev || !x_dev || max_iter < 0) return setLastError(SYMGB_ERR_ARGUMENT, "solver: bad argument");
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned S = s->S;
    const std::uint64_t work = s->n * S;
    // scalars: rz[2][S] (by iteration parity), pq[S], rr[S], bb[S]
    double* rz = s->scalars.ptr;
    double* pq = rz + 2 * S;
    double* rr = pq + S;
    double* bb = rr + S;
    const std::size_t smem1 = S * sizeof(double), smem2 = 2 * S * sizeof(double);
    gatherValues<<<blocksFor(s->nnzFull * S), kThreads, 0, st>>>(values, s->nnzIn, s->src.ptr, s->nnzFull, S,
                                                                 s->vals.ptr);
    cudaMemsetAsync(s->scalars.ptr, 0, 8 * (std::size_t)S * sizeof(double), st);
    cgStart<<<blocksFor(work), kThreads, smem2, st>>>(b_dev, s->vals.ptr, s->diagPos.ptr, s->n, S, s->x.ptr, s->r.ptr,
                                                     s->p.ptr, s->invDiag.ptr, rz, bb);
    int it = 0;
    double worst = 0.0;
    std::vector<double> bbHost(S);
    bool haveBb = false;
    while (it < max_iter) {
        const int block = std::min(kCheck, max_iter - it);
        for (int k = 0; k < block; ++k, ++it) {
            double* rzOld = rz + (it & 1) * S;
            double* rzNew = rz + ((it + 1) & 1) * S;
            cudaMemsetAsync(pq, 0, 2 * S * sizeof(double), st);  // pq and rr
            cudaMemsetAsync(rzNew, 0, S * sizeof(double), st);
            cgSpmv<<<blocksFor(work), kThreads, smem1, st>>>(s->rowPtr.ptr, s->col.ptr, s->vals.ptr, s->p.ptr, s->n, S,
                                                            s->q.ptr, pq);
            cgUpdate<<<blocksFor(work), kThreads, smem2, st>>>(s->p.ptr, s->q.ptr, s->invDiag.ptr, s->n, S, rzOld, pq,
                                                              s->x.ptr, s->r.ptr, rzNew, rr);
            cgDirection<<<blocksFor(work), kThreads, 0, st>>>(s->r.ptr, s->invDiag.ptr, s->n, S, rzOld, rzNew,
                                                             s->p.ptr);
        }
        if (!haveBb) {
            cudaMemcpyAsync(bbHost.data(), bb, S * sizeof(double), cudaMemcpyDeviceToHost, st);
            haveBb = true;
        }
        cudaMemcpyAsync(s->hostScalars, rr, S * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return setLastError(SYMGB_ERR_CUDA, "solver: solve failed");
        worst = 0.0;
        for (unsigned k = 0; k < S; ++k) {
            const double rel = bbHost[k] > 0 ? std::sqrt(s->hostScalars[k] / bbHost[k]) : 0.0;
            worst = std::max(worst, rel);
        }
        if (worst <= tol) break;
    }
    cgFinish<<<blocksFor(work), kThreads, 0, st>>>(s->x.ptr, s->n, S, x_dev);
    if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess)
        return setLastError(SYMGB_ERR_CUDA, "solver: solve failed");
    if (iterations) *iterations = it;
    if (max_rel_residual) *max_rel_residual = max_iter ? worst : 1.0;
    return SYMGB_OK;
}

static int solveBicgstab(symgb_solver_t s, const double* values, const double* b_dev, double* x_dev, double tol,
                         int max_iter, void* stream, int* iterations, double* max_rel_residual) {
    using symgb::engine::setLastError;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned S = s->S;
    const std::uint64_t work = s->n * S;
    if (!s->rhat.ptr && (s->rhat.alloc(work) || s->v.alloc(work) || s->ph.alloc(work) || s->sv.alloc(work) ||
                         s->sh.alloc(work) || s->t.alloc(work)))
        return setLastError(SYMGB_ERR_NOMEM, "solver: device allocation failed");
    double* R = s->scalars.ptr;  // R[3][S]
    double* rv = R + 3 * S;      // rv, ts, tt, rr contiguous
    double* ts = rv + S;
    double* tt = ts + S;
    double* rr = tt + S;
    double* bb = rr + S;
    double* alpha = bb + S;
    double* omega = alpha + S;
    const std::size_t smem1 = S * sizeof(double), smem2 = 2 * S * sizeof(double);
    gatherValues<<<blocksFor(s->nnzFull * S), kThreads, 0, st>>>(values, s->nnzIn, s->src.ptr, s->nnzFull, S,
                                                                 s->vals.ptr);
    cudaMemsetAsync(s->scalars.ptr, 0, 16 * (std::size_t)S * sizeof(double), st);
    bStart<<<blocksFor(work), kThreads, smem1, st>>>(b_dev, s->vals.ptr, s->diagPos.ptr, s->n, S, s->x.ptr, s->r.ptr,
                                                    s->rhat.ptr, s->p.ptr, s->v.ptr, s->invDiag.ptr, R, bb);
    const bool blocks = s->block > 1;
    if (blocks) blockInvertLaunch(s->block, s->vals.ptr, s->blockPos.ptr, s->n / s->block, S, s->blockInv.ptr, st);
    {
        std::vector<double> ones(3 * (std::size_t)S, 1.0);  // R[2] (previous rho), alpha, omega = 1
        cudaMemcpyAsync(R + 2 * S, ones.data(), S * sizeof(double), cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(alpha, ones.data(), 2 * S * sizeof(double), cudaMemcpyHostToDevice, st);
        cudaStreamSynchronize(st);  // `ones` lives on this stack
    }
    int it = 0;
    double worst = 0.0;
    std::vector<double> bbHost(S);
    bool haveBb = false;
    while (it < max_iter) {
        const int block = std::min(kCheck, max_iter - it);
        for (int k = 0; k < block; ++k, ++it) {
            double* rho = R + (it % 3) * S;
            double* rhoPrev = R + ((it + 2) % 3) * S;
            double* rhoNext = R + ((it + 1) % 3) * S;
            cudaMemsetAsync(rv, 0, 4 * S * sizeof(double), st);
            cudaMemsetAsync(rhoNext, 0, S * sizeof(double), st);
            bDirection<<<blocksFor(work), kThreads, 0, st>>>(s->r.ptr, s->v.ptr, s->invDiag.ptr, s->n, S, rho, rhoPrev,
                                                            alpha, omega, s->p.ptr, s->ph.ptr);
            if (blocks) blockApplyLaunch(s->block, s->blockInv.ptr, s->p.ptr, s->n, s->blockStride, S, s->ph.ptr, st);
            bSpmv<<<blocksFor(work), kThreads, smem2, st>>>(s->rowPtr.ptr, s->col.ptr, s->vals.ptr, s->ph.ptr, s->n, S,
                                                           s->rhat.ptr, s->v.ptr, rv, nullptr);
            bHalf<<<blocksFor(work), kThreads, 0, st>>>(s->r.ptr, s->v.ptr, s->invDiag.ptr, s->n, S, rho, rv, alpha,
                                                       s->sv.ptr, s->sh.ptr);
            if (blocks) blockApplyLaunch(s->block, s->blockInv.ptr, s->sv.ptr, s->n, s->blockStride, S, s->sh.ptr, st);
            bSpmv<<<blocksFor(work), kThreads, smem2, st>>>(s->rowPtr.ptr, s->col.ptr, s->vals.ptr, s->sh.ptr, s->n, S,
                                                           s->sv.ptr, s->t.ptr, ts, tt);
            bFinishStep<<<blocksFor(work), kThreads, smem2, st>>>(s->ph.ptr, s->sh.ptr, s->sv.ptr, s->t.ptr,
                                                                 s->rhat.ptr, s->n, S, alpha, ts, tt, omega, s->x.ptr,
                                                                 s->r.ptr, rhoNext, rr);
        }
        if (!haveBb) {
            cudaMemcpyAsync(bbHost.data(), bb, S * sizeof(double), cudaMemcpyDeviceToHost, st);
            haveBb = true;
        }
        cudaMemcpyAsync(s->hostScalars, rr, S * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return setLastError(SYMGB_ERR_CUDA, "solver: solve failed");
        worst = 0.0;
        for (unsigned k = 0; k < S; ++k)
            worst = std::max(worst, bbHost[k] > 0 ? std::sqrt(s->hostScalars[k] / bbHost[k]) : 0.0);
        if (worst <= tol) break;
    }
    cgFinish<<<blocksFor(work), kThreads, 0, st>>>(s->x.ptr, s->n, S, x_dev);
    if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess)
        return setLastError(SYMGB_ERR_CUDA, "solver: solve failed");
    if (iterations) *iterations = it;
    if (max_rel_residual) *max_rel_residual = max_iter ? worst : 1.0;
    return SYMGB_OK;
}

int symgb_solver_solve(symgb_solver_t s, int method, const double* values, const double* b, double* x, double tol,
                       int max_iter, void* stream, int* iterations, double* max_rel_residual) {
    using symgb::engine::setLastError;
    if (!s || !values || !b || !x || max_iter < 0) return setLastError(SYMGB_ERR_ARGUMENT, "solver: bad argument");
    if (method == SYMGB_SOLVER_CG) return solveCg(s, values, b, x, tol, max_iter, stream, iterations, max_rel_residual);
    if (method == SYMGB_SOLVER_BICGSTAB)
        return solveBicgstab(s, values, b, x, tol, max_iter, stream, iterations, max_rel_residual);
    return setLastError(SYMGB_ERR_ARGUMENT, "solver: unknown method");
}

void symgb_solver_destroy(symgb_solver_t s) { delete s; }

}  // extern "C"
