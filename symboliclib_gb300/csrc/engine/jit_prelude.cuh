// Device functions shared by the interpreter (device.cuh, compiled by nvcc
// into libsymgb.so) and by the compiled executor's generated kernels
// (codegen.cpp, compiled at run time by NVRTC, which receives this file's
// text as the prelude of every generated module).  Self-contained: no
// includes, only CUDA built-ins, so it compiles unchanged in both settings.
// Included inside an anonymous namespace by device.cuh.
#ifndef SYMGB_ERR_TIMEOUT
#define SYMGB_ERR_TIMEOUT (-4)
#endif

// Negation flips the sign (C's unary minus; exact, -(+0) = -0).  Written as
// the language's negation so the compiler can fold it into the sign modifier
// of the FMA, add or multiply that consumes it: no instruction of its own and
// no step in the dependency chain.
__device__ __forceinline__ double symgbNegate(double x) { return -x; }

// Fast-mode division, reciprocal and square root (OP_FDIV, OP_FREC, OP_FSQRT;
// exact mode keeps the IEEE operations).  Each starts from the hardware's
// approximate reciprocal or reciprocal square root (PTX rcp.approx.ftz.f64 /
// rsqrt.approx.ftz.f64), refines it by Newton-Raphson and ends with one
// correction step that uses the residual an FMA computes exactly
// (P. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Develop. 34(1), 1990; for the square
// root the coupled iteration of Goldschmidt's method).  With a start error e
// the result carries e^3 or less beside its final rounding, so it stays within
// one unit in the last place for any e below 2^-18.  Operands outside the
// exponent window where every intermediate is a normal finite number (this
// includes zero, subnormal, infinite and NaN operands and negative
// square-root arguments) take the IEEE operation instead, except a zero
// dividend, whose quotient a * (1/b) is already exact.
__device__ __forceinline__ double symgbRcpApprox(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    return r;
}
__device__ __forceinline__ double symgbRsqrtApprox(double x) {
    double r;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    return r;
}
// Sign and biased exponent (12 bits).
__device__ __forceinline__ unsigned symgbSignExp(double x) { return (unsigned)__double2hiint(x) >> 20; }
// The IEEE operations for operands outside the window, out of line: inlined,
// the compiler evaluates them beside the fast sequence and selects, which
// costs the sum of both.
__device__ __noinline__ double symgbIeeeDiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __noinline__ double symgbIeeeSqrt(double x) { return __dsqrt_rn(x); }

// a / b for |a|, |b| in [2^-500, 2^501); elsewhere the IEEE division.
__device__ __forceinline__ double symgbFastDiv(double a, double b) {
    const double r0 = symgbRcpApprox(b);
    const double r = __fma_rn(r0, __fma_rn(-b, r0, 1.0), r0);
    const double q0 = __dmul_rn(a, r);
    double q = __fma_rn(r, __fma_rn(-b, q0, a), q0);
    const bool zeroA = (((unsigned)__double2hiint(a) << 1) | (unsigned)__double2loint(a)) == 0u;
    if (zeroA) q = q0;
    if (__builtin_expect((symgbSignExp(b) & 0x7ffu) - 523u > 1000u ||
                             (!zeroA && (symgbSignExp(a) & 0x7ffu) - 523u > 1000u),
                         0))
        q = symgbIeeeDiv(a, b);
    return q;
}
// 1 / x for |x| in [2^-1000, 2^1001); elsewhere the IEEE division.
__device__ __forceinline__ double symgbFastRec(double x) {
    double r = symgbRcpApprox(x);
    r = __fma_rn(r, __fma_rn(-x, r, 1.0), r);
    r = __fma_rn(r, __fma_rn(-x, r, 1.0), r);
    if (__builtin_expect((symgbSignExp(x) & 0x7ffu) - 23u > 2000u, 0)) r = symgbIeeeDiv(1.0, x);
    return r;
}
// sqrt(x) for x in [2^-900, 2^901); elsewhere the IEEE square root.
__device__ __forceinline__ double symgbFastSqrt(double x) {
    const double y = symgbRsqrtApprox(x);
    double g = __dmul_rn(x, y);          // sqrt(x) (1 + e)
    const double h = __dmul_rn(0.5, y);  // 1 / (2 sqrt(x)) (1 + e)
    g = __fma_rn(g, __fma_rn(-g, h, 0.5), g);
    g = __fma_rn(__fma_rn(-g, g, x), h, g);
    if (__builtin_expect(symgbSignExp(x) - 123u > 1800u, 0)) g = symgbIeeeSqrt(x);
    return g;
}

__device__ __forceinline__ unsigned long long symgbGlobalTimerNs() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier for a cooperative launch.  B has the fields count,
// generation (unsigned) and error (int).  The wait is bounded: after
// `timeoutNs` the waiting block records SYMGB_ERR_TIMEOUT in bar->error and in
// the host-mapped flag `hostError`, and leaves.  Every block checks bar->error
// after each barrier and returns false when it is set.  `expected` is the
// number of arrivals that completes the barrier (gridDim.x in normal use).
template <class B>
__device__ bool symgbGridBarrier(B* bar, int* hostError, unsigned long long timeoutNs, unsigned expected) {
    __syncthreads();
    __shared__ int failed;
    if (threadIdx.x == 0) {
        volatile unsigned int* gen = &bar->generation;
        volatile int* err = &bar->error;
        const unsigned int g = *gen;
        __threadfence();
        if (atomicAdd(&bar->count, 1u) == expected - 1) {
            atomicExch(&bar->count, 0u);
            __threadfence();
            atomicAdd(&bar->generation, 1u);
        } else {
            const unsigned long long t0 = symgbGlobalTimerNs();
            while (*gen == g) {
                if (*err) break;
                if (symgbGlobalTimerNs() - t0 > timeoutNs) {
                    atomicExch(&bar->error, SYMGB_ERR_TIMEOUT);
                    *(volatile int*)hostError = SYMGB_ERR_TIMEOUT;
                    break;
                }
                __nanosleep(100);
            }
        }
        __threadfence();
        failed = *err != 0;
    }
    __syncthreads();
    return !failed;
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may start while the previous kernel of its stream is still
// running; it waits here until that kernel has finished and its writes are
// visible.  Without the launch attribute the wait returns at once.  The
// trigger lets the next such kernel be scheduled as soon as every block of
// this one has started (it still waits for this one to finish).
__device__ __forceinline__ void symgbDependencyWait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void symgbLaunchDependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
