/* CPU oracle for the engine's device path.  TEST INFRASTRUCTURE ONLY: called by
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
 * checker; the engine never links or calls it.
 *
 * Restates what the reference's generated code does in execute() and
 * getResults():
 *   run():  for every kernel k in order and every instance i < n_k, evaluate the
 *           kernel's template statements (src/ComputeUnit.cpp:409-421, body text
 *           from src/ComputeKernel.cpp:329-381 with pack length 0):
 *             DEFINE r = e        -> const RealT r = e;
 *             ASSIGN out[a] = e   -> y[n*a + i] = e;   y = x + outputOffset[k]
 *             index variable a    -> x[p[n*base + i] + offset]
 *             constant row a      -> c[n*a + i]
 *           with n-ary sums and products evaluated left to right as C does
 *           (fully parenthesised infix text, src/CodeGenerator.cpp:38-61);
 *   getResult(k): d[j] = x[outIds[outputIndexStart[k] + j]]
 *           (src/StringResources.h:70-73, 129-134).
 * Every operation is a separate IEEE double operation (compile with
 * -ffp-contract=off, no -ffast-math): the reference's order, nothing fused.
 * The template arrives as post-order symgb_node records (include/symgb.h). */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/symgb.h"

enum { N_CONST = 1, N_VAR = 2, N_ADD = 3, N_MUL = 4, N_MULC = 5, N_DIV = 6, N_SQRT = 7, N_SIN = 8, N_COS = 9,
       N_TAN = 10, N_ASIN = 12, N_ACOS = 13, N_ATAN = 14, N_EXP = 15, N_LOG = 16, N_POW = 17, N_ASSIGN = 18,
       N_NEG = 23, N_DEFINE = 24, N_BLOCK = 25, N_REC = 26 };

typedef struct {
    const symgb_kernel_desc* k;
    const uint32_t* p;
    const double* c;
    double* x;
    double* locals;  /* indexed by local id */
    int32_t* first;  /* first[j]: index of node j's first descendant (post-order subtree start) */
    uint64_t i;
    int bad;
} ctx_t;

/* Value of node j (the subtree ending at j in the post-order list). */
static double eval(ctx_t* t, int j) {
    const symgb_node* nd = &t->k->nodes[j];
    const uint64_t n = t->k->num_instances, i = t->i;
    switch (nd->op) {
        case N_CONST: return nd->value;
        case N_VAR:
            if (nd->b == -3) {
                const int32_t base = t->k->access[2 * nd->a], off = t->k->access[2 * nd->a + 1];
                return t->x[(int64_t)t->p[n * (uint64_t)base + i] + off];
            }
            if (nd->b == -4) return t->c[n * (uint64_t)nd->a + i];
            if (nd->b == 253) return t->locals[nd->a];
            t->bad = 1;
            return 0.0;
        default: break;
    }
    /* children of j, in order: walk back from j-1 over sibling subtrees */
    int kids[64];
    int nc = nd->nchild, pos = j - 1;
    int* ks = nc <= 64 ? kids : (int*)malloc(sizeof(int) * nc);
    for (int c = nc - 1; c >= 0; --c) {
        ks[c] = pos;
        pos = t->first[pos] - 1;
    }
    double r = 0.0;
    switch (nd->op) {
        case N_ADD:
            r = eval(t, ks[0]);
            for (int c = 1; c < nc; ++c) r = r + eval(t, ks[c]);
            break;
        case N_MUL:
        case N_MULC:
            r = eval(t, ks[0]);
            for (int c = 1; c < nc; ++c) r = r * eval(t, ks[c]);
            break;
        case N_DIV: r = eval(t, ks[0]) / eval(t, ks[1]); break;
        case N_NEG: r = -eval(t, ks[0]); break;
        case N_SQRT: r = sqrt(eval(t, ks[0])); break;
        case N_REC: r = 1.0 / eval(t, ks[0]); break;
        case N_SIN: r = sin(eval(t, ks[0])); break;
        case N_COS: r = cos(eval(t, ks[0])); break;
        case N_TAN: r = tan(eval(t, ks[0])); break;
        case N_ASIN: r = asin(eval(t, ks[0])); break;
        case N_ACOS: r = acos(eval(t, ks[0])); break;
        case N_ATAN: r = atan(eval(t, ks[0])); break;
        case N_EXP: r = exp(eval(t, ks[0])); break;
        case N_LOG: r = log(eval(t, ks[0])); break;
        case N_POW: {
            const double a = eval(t, ks[0]);
            r = pow(a, eval(t, ks[1]));
            break;
        }
        default: t->bad = 1;
    }
    if (ks != kids) free(ks);
    return r;
}

static void statement(ctx_t* t, int j) {
    const symgb_node* nd = &t->k->nodes[j];
    if (nd->op == N_BLOCK) { /* nested statement list, printed inline by the reference */
        int kids[256];
        const int nc = nd->nchild;
        int* ks = nc <= 256 ? kids : (int*)malloc(sizeof(int) * nc);
        int pos = j - 1;
        for (int c = nc - 1; c >= 0; --c) {
            ks[c] = pos;
            pos = t->first[pos] - 1;
        }
        for (int c = 0; c < nc; ++c) statement(t, ks[c]);
        if (ks != kids) free(ks);
        return;
    }
    const int rhs = j - 1, lhs = t->first[rhs] - 1;
    const symgb_node* name = &t->k->nodes[lhs];
    const double v = eval(t, rhs);
    if (nd->op == N_DEFINE) {
        t->locals[name->a] = v;
    } else if (nd->op == N_ASSIGN) {
        t->x[t->k->output_offset + t->k->num_instances * (uint64_t)name->a + t->i] = v;
    } else {
        t->bad = 1;
    }
}

/* Evaluates all kernels of `plan` on x (num_total_memory doubles, inputs
 * already placed at arg_start).  Returns 0, or -1 on a template it cannot
 * evaluate. */
int oracle_run(const symgb_plan_desc* plan, const uint32_t* index_data, const double* const_data, double* x) {
    int status = 0;
    for (uint32_t kk = 0; kk < plan->num_kernels; ++kk) {
        const symgb_kernel_desc* k = &plan->kernels[kk];
        const int nn = (int)k->num_nodes;
        int32_t* first = (int32_t*)malloc(sizeof(int32_t) * (nn > 0 ? nn : 1));
        int maxLocal = 0;
        /* subtree start of every node */
        int32_t* stack = (int32_t*)malloc(sizeof(int32_t) * (nn > 0 ? nn : 1));
        int sp = 0;
        for (int j = 0; j < nn; ++j) {
            int st = j;
            for (int c = 0; c < k->nodes[j].nchild; ++c) st = stack[--sp];
            first[j] = st;
            stack[sp++] = st;
            if (k->nodes[j].op == N_VAR && k->nodes[j].b == 253 && k->nodes[j].a + 1 > maxLocal) maxLocal = k->nodes[j].a + 1;
        }
        free(stack);
        double* locals = (double*)calloc((size_t)maxLocal + 1, sizeof(double));
        /* statements: children of the root BLOCK */
        const int root = nn - 1;
        int stmts[1];
        int* st = NULL;
        int ns = 0;
        if (k->nodes[root].op == N_BLOCK) {
            ns = k->nodes[root].nchild;
            st = (int*)malloc(sizeof(int) * (ns > 0 ? ns : 1));
            int pos = root - 1;
            for (int c = ns - 1; c >= 0; --c) {
                st[c] = pos;
                pos = first[pos] - 1;
            }
        } else {
            stmts[0] = root;
            st = stmts;
            ns = 1;
        }
        ctx_t t;
        t.k = k;
        t.p = index_data + k->index_offset;
        t.c = const_data + k->constants_offset;
        t.x = x;
        t.locals = locals;
        t.first = first;
        t.bad = 0;
        for (uint64_t i = 0; i < k->num_instances; ++i) {
            t.i = i;
            for (int s = 0; s < ns; ++s) statement(&t, st[s]);
        }
        if (t.bad) status = -1;
        if (st != stmts) free(st);
        free(locals);
        free(first);
    }
    return status;
}

/* d[j] = x[ids[start + j]] */
void oracle_gather(const double* x, const uint32_t* out_index_data, uint64_t start, uint64_t len, double* d) {
    for (uint64_t j = 0; j < len; ++j) d[j] = x[out_index_data[start + j]];
}
