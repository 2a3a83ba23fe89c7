/* symgb - GB300 execution engine for SymbolicLib ComputeUnit plans.
 *
 * C ABI of the device path.  It replaces the library that the reference's
 * ComputeUnit::compile generates, builds with nvcc and dlopen()s
 * (src/ComputeUnit.cpp:77-169, src/StringResources.h:15-161).  That library
 * exports five functions over process-global state, with the plan's metadata
 * (kernel count, instance counts, offsets, template bodies) baked into its
 * source as globals (src/ComputeUnit.cpp:368-450).  Here the same five calls
 * take a unit handle, and the baked-in metadata is passed once as a plan
 * description (symgb_unit_create).  Every call returns 0 on success or a
 * negative error code; symgb_last_error() describes the last failure on the
 * calling thread.  No call exits the process.
 *
 * Plain pointers and sizes only; the library owns all device memory it
 * allocates.  A unit is not thread-safe; distinct units are independent.
 */
#ifndef SYMGB_H
#define SYMGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SYMGB_OK 0
#define SYMGB_ERR_ARGUMENT (-1)  /* invalid argument or plan */
#define SYMGB_ERR_CUDA (-2)      /* CUDA runtime error */
#define SYMGB_ERR_STATE (-3)     /* call out of order (e.g. run before init) */
#define SYMGB_ERR_TIMEOUT (-4)   /* a bounded device-side wait gave up */
#define SYMGB_ERR_NOMEM (-5)     /* device allocation failed */
#define SYMGB_ERR_DEVICE (-6)    /* device-side check failed (bounds) */

/* Template node, post-order.  Operation codes are the reference IR's
 * (src/Operations.hpp:9-38).  Leaves:
 *   op = 1 (CONST): value
 *   op = 2 (VAR):   a = id, b = group, with group
 *       -2  output row a            (reference y[n*a + i])
 *       -3  index variable a        (reference x[p[n*base + i] + offset], base and
 *                                    offset from the kernel's access table)
 *       -4  per-instance constant a (reference c[n*a + i])
 *       253 local value a           (reference "r<a>")
 * Inner nodes: op with nchild children (the preceding sub-trees).
 * Statements: 24 (DEFINE local = expr), 18 (ASSIGN output = expr), 25 (BLOCK). */
typedef struct symgb_node {
    int32_t op;
    int32_t nchild;
    int32_t a;
    int32_t b;
    double value;
} symgb_node;

typedef struct symgb_kernel_desc {
    uint64_t num_instances;     /* reference numInstances[k] */
    uint64_t output_offset;     /* reference outputOffset[k] (first x slot written) */
    uint64_t index_offset;      /* reference indexOffset[k] */
    uint64_t constants_offset;  /* reference constantsOffset[k] */
    uint32_t num_output_rows;
    uint32_t num_index_rows;
    uint32_t num_constant_rows;
    int32_t level;              /* longest dependency path from the inputs */
    uint32_t num_nodes;
    const symgb_node* nodes;    /* template, post-order */
    uint32_t num_access;
    const int32_t* access;      /* (base row, offset) per index variable */
} symgb_kernel_desc;

typedef struct symgb_plan_desc {
    uint32_t num_kernels;
    const symgb_kernel_desc* kernels;  /* in execution order */
    uint32_t num_args;
    const uint64_t* arg_start;         /* reference argStart[] */
    const uint64_t* arg_length;        /* reference argLength[] */
    uint32_t num_outputs;
    const uint64_t* output_start;      /* reference outputIndexStart[] */
    const uint64_t* output_length;     /* reference outputIndexLength[] */
    uint64_t num_total_memory;         /* reference numTotalMemory */
    uint64_t num_indices;              /* reference numIndizes */
    uint64_t num_output_values;        /* reference numOutputValues */
    uint64_t num_constants;            /* reference numConst */
    uint32_t threads_per_block;        /* reference Device ThreadsPerBlock */
} symgb_plan_desc;

typedef struct symgb_unit* symgb_unit_t;

/* Execution schedules. */
#define SYMGB_SCHEDULE_PLAIN 0       /* one launch per kernel, one thread per instance
                                        and value set (the reference's run()) */
#define SYMGB_SCHEDULE_LEVELS 1      /* one launch per dependency level, all kernels of
                                        the level in one grid */
#define SYMGB_SCHEDULE_PERSISTENT 2  /* one cooperative launch; levels separated by
                                        bounded grid barriers */

/* Arithmetic modes. */
#define SYMGB_MATH_EXACT 0  /* every operation rounded separately, in template order
                               (bit-identical to the reference without FP contraction) */
#define SYMGB_MATH_FAST 1   /* multiply-add pairs fused into FMA */

typedef struct symgb_schedule {
    int32_t kind;               /* SYMGB_SCHEDULE_* */
    int32_t math;               /* SYMGB_MATH_* */
    int32_t threads_per_block;  /* 0 = plan default */
    int32_t items_per_tile;     /* work items per CTA tile in fused schedules (0 = auto) */
    int32_t blocks_per_sm;      /* CTAs per SM.  Interpreter, persistent: 0 = occupancy maximum;
                                   plain and levels: 0 = one CTA per tile, > 0 caps the grid at
                                   this many CTAs per SM, each taking several tiles.  Compiled
                                   executor: > 0 is the minimum of resident CTAs per SM its
                                   kernels are compiled for (__launch_bounds__), which caps their
                                   registers; 0 = the compiler's choice */
    int32_t use_graph;          /* capture run() into a CUDA graph and replay it */
    int32_t items_per_thread;   /* work items per thread per pass: 1, 2 or 4 (0 = 1) */
    int32_t fusion_depth;       /* LEVELS: consecutive levels per launch (0/1 = one level; a
                                   group of several levels is one cooperative launch) */
    int32_t lanes_per_item;     /* threads sharing one work item: 1, 2, 4 or 8 (0 = 1).  They
                                   split every bundle of the program and share the item's
                                   register file, which divides its shared memory per thread */
    int32_t executor;           /* SYMGB_EXEC_*: how kernel templates run (below) */
} symgb_schedule;

/* Executors.  Both compute every value with the same operations in the same
 * order, so their results are bit-identical in either math mode.
 *   COMPILED: each template becomes straight-line CUDA C++ (the form of the
 *     reference's generated kernels, ComputeUnit.cpp:409-421), one work item
 *     per thread, compiled for sm_103a by NVRTC at the first run of a
 *     configuration (math mode, value sets, schedule, block sizes) and cached
 *     for the process; consecutive launches overlap their start-up
 *     (programmatic dependent launch).  A thread takes items_per_thread work
 *     items (1, 2 or 4, unrolled); lanes_per_item, items_per_tile and
 *     fusion_depth do not apply.
 *   INTERPRETER: one precompiled kernel runs every template as a bundled
 *     register-machine program (no run-time compilation). */
#define SYMGB_EXEC_COMPILED 0
#define SYMGB_EXEC_INTERPRETER 1

/* Compiles (or finds in the cache) the compiled executor's module for the
 * unit's current schedule, value-set count and kernel shapes, so that a later
 * run - or a graph capture, during which nothing may be compiled - does not
 * pay for it.  *compile_seconds (if not NULL) receives the time this call
 * spent (0 when cached).  No-op for the interpreter. */
int symgb_prepare(symgb_unit_t u, double* compile_seconds);

/* Host-only introspection of the compiled executor (no device needed): the
 * generated CUDA C++ source of schedule `kind` (SYMGB_SCHEDULE_*) for the
 * unit's current math mode, value sets and block sizes.  Writes up to `cap`
 * bytes (NUL-terminated when it fits) and returns the source length, or a
 * negative error.  symgb_compile_check compiles that source with NVRTC for
 * sm_103a without loading it (the compile log is in symgb_last_error on
 * failure) and reports the compile time. */
int64_t symgb_compiled_source(symgb_unit_t u, int kind, char* buf, uint64_t cap);
int symgb_compile_check(symgb_unit_t u, int kind, double* seconds);

/* Registers per thread of each launch of the compiled module of schedule
 * `kind` (compiled and loaded if needed; needs an initialised unit): writes up
 * to `cap` entries in launch order and returns the number of launches. */
int symgb_compiled_registers(symgb_unit_t u, int kind, int* registers, int cap);

/* Data path of the compiled executor's loads (index and constant tables and
 * the x gathers): the read-only path (ld.global.nc, the default), cached in
 * L1 (ld.global.ca) or in L2 only (ld.global.cg).  Values are the same; the
 * choice changes which load queue the gathers wait in. */
#define SYMGB_LOAD_READONLY 0
#define SYMGB_LOAD_L1 1
#define SYMGB_LOAD_L2 2
int symgb_set_load_path(symgb_unit_t u, int path);

/* Which work items a thread of the compiled executor takes.
 *   STRIDED (default): items_per_thread work items tpb apart (consecutive
 *     threads on consecutive work items).
 *   GROUPED: items_per_thread consecutive instances of one value set; the
 *     thread reads their entries of each index and constant row with one
 *     vector load (128-bit for 4 instances of an index row) from copies of
 *     the tables whose rows are padded to a multiple of 4 entries, made on the
 *     device at first use (about the size of the tables; symgb_prepare makes
 *     them ahead of a graph capture).
 * Values are the same either way. */
#define SYMGB_ITEMS_STRIDED 0
#define SYMGB_ITEMS_GROUPED 1
int symgb_set_item_layout(symgb_unit_t u, int layout);

/* Direct result writes (default on): with the compiled executor and one
 * value set, output rows whose slots no kernel reads and that each name one
 * result position are stored by the kernels straight at their positions in
 * the unit's result buffer (container order, the CSC order of a sparse
 * output), instead of in x and a gather pass after the run; the results of
 * any other rows are gathered into that buffer when they are read.  The
 * plan is made by symgb_init.  A run waits on its stream for the unit's
 * asynchronous result copies still reading the previous results; batch
 * replays and symgb_time_kernels do not. */
int symgb_set_direct_outputs(symgb_unit_t u, int on);

/* Failure-handling tests only: the limit of every bounded grid-barrier wait
 * (default 2 s) and a number of arrivals each barrier waits for beyond the
 * grid (default 0; > 0 makes every barrier wait out its limit, so the run
 * returns SYMGB_ERR_TIMEOUT while the context stays usable). */
int symgb_set_barrier_limits(symgb_unit_t u, uint64_t timeout_ns, int extra_arrivals);

/* Launch shape of one kernel (items per thread, lanes per item, threads per
 * block; 0 = the schedule's value).  Used by the plain schedule for that
 * kernel's launch, and by the levels schedule for a level whose largest kernel
 * it is.  Changes no value. */
int symgb_set_kernel_shape(symgb_unit_t u, int k, int items_per_thread, int lanes_per_item, int threads_per_block);

/* Per-kernel timing for the autotuner: runs the plain schedule (one launch per
 * kernel, in execution order, with the kernels' shapes) `reps` times on the
 * unit's stream, writing the mean microseconds of each kernel's launch into
 * us_per_kernel[num_kernels].  With flush != NULL, flush_bytes of that device
 * buffer are overwritten before every repetition (L2 eviction).  The x slots
 * are written as by symgb_run. */
int symgb_time_kernels(symgb_unit_t u, int reps, void* flush, uint64_t flush_bytes, double* us_per_kernel);

/* --- the reference's generated-library calls, per unit ----------------------- */

/* Creates a unit from a plan description (copies it) and compiles the templates
 * into device programs.  Replaces the plan globals of the generated source. */
int symgb_unit_create(const symgb_plan_desc* plan, symgb_unit_t* out);

/* Allocates device memory and uploads the tables.  Replaces init()
 * (src/StringResources.h:75-123); null table pointers are an error (the
 * reference reads its table files from the working directory instead). */
int symgb_init(symgb_unit_t u, const uint32_t* index_data, const uint32_t* out_index_data, const double* const_data);

/* Copies input container i (arg_length[i] values) from host memory.
 * Replaces setArg (src/StringResources.h:125-127). */
int symgb_set_arg(symgb_unit_t u, const double* d, int i);

/* Evaluates all kernels and waits for completion.  Replaces run()
 * (src/ComputeUnit.cpp:440-447). */
int symgb_run(symgb_unit_t u);

/* Copies output container k (output_length[k] values, container order) to host
 * memory.  Replaces getResult (src/StringResources.h:129-134). */
int symgb_get_result(symgb_unit_t u, double* d, int k);

/* Replaces finish() (src/StringResources.h:136-138); releases device memory. */
int symgb_finish(symgb_unit_t u);

void symgb_unit_destroy(symgb_unit_t u);
const char* symgb_last_error(void);

/* --- schedules, value-set batches and device-resident use ------------------- */

int symgb_set_schedule(symgb_unit_t u, const symgb_schedule* s);
int symgb_get_schedule(symgb_unit_t u, symgb_schedule* s);

/* Number of value sets evaluated per run (1 .. 2^20, default 1).  Reallocates x. */
int symgb_set_num_sets(symgb_unit_t u, int num_sets);
int symgb_num_sets(symgb_unit_t u);

/* Input container i for all value sets: d[set * arg_length[i] + j]. */
int symgb_set_arg_sets(symgb_unit_t u, const double* d, int i);
/* Output container k for all value sets: d[set * output_length[k] + j]. */
int symgb_get_result_sets(symgb_unit_t u, double* d, int k);

/* Stream used by the unit (a cudaStream_t; 0 = the unit's own stream). */
int symgb_set_stream(symgb_unit_t u, void* stream);
/* Enqueues the evaluation without waiting. */
int symgb_run_async(symgb_unit_t u);
/* Device-to-device variants: `d` is a device pointer in the same layout as the
 * host variants; work is enqueued on the unit's stream without waiting. */
int symgb_set_arg_sets_device(symgb_unit_t u, const double* d, int i);
int symgb_get_result_sets_device(symgb_unit_t u, double* d, int k);
int symgb_synchronize(symgb_unit_t u);
/* Asynchronous host transfers, for overlapping one execute's transfers with
 * another's evaluation: `d` must be page-locked host memory (cudaHostAlloc or
 * cudaHostRegister; anything else is SYMGB_ERR_ARGUMENT).  The input copy is
 * enqueued on the unit's stream.  The result is gathered on the unit's stream
 * into a device buffer and copied to `d` on the unit's own copy stream, which
 * the unit's stream does not wait for (the next gather of the same container
 * does).  `d` must not be touched before symgb_synchronize, which waits for
 * both streams. */
int symgb_set_arg_sets_async(symgb_unit_t u, const double* d, int i);
int symgb_get_result_sets_async(symgb_unit_t u, double* d, int k);

/* Copy streams of symgb_get_result_sets_async (1..8, default 1): a result of
   n >= 8 MiB is split into min(count, n / 8 MiB) chunks, each copied on its
   own stream (several copy engines); the completion the next call waits for
   covers every chunk. */
int symgb_set_copy_streams(symgb_unit_t u, int count);

/* Batches of units (many patterns of uneven size): one evaluation of every
 * unit, each with its own schedule and value sets, captured into one CUDA graph
 * whose branches (`streams` of them, units assigned round-robin) run
 * concurrently.  Units must be initialized; their inputs are set as usual. */
typedef struct symgb_batch* symgb_batch_t;
int symgb_batch_create(symgb_unit_t* units, int n, int streams, symgb_batch_t* out);
int symgb_batch_run(symgb_batch_t b);                        /* replay and wait */
int symgb_batch_run_async(symgb_batch_t b, void* stream);    /* replay on `stream` (0 = own) */
int symgb_batch_launch_count(symgb_batch_t b);               /* kernels in the graph */
void symgb_batch_destroy(symgb_batch_t b);

/* Learned schedule cost model: an FP32 MLP (inputs -> hidden -> hidden -> 1,
 * ReLU) trained and evaluated on the GPU by the engine's own kernels.  X is
 * row-major [n][inputs] in host memory, y [n].  Parameters are flattened as
 * W1 (inputs x hidden), b1, W2 (hidden x hidden), b2, W3 (hidden), b3.
 * Training minimises the mean squared error with Adam over the full batch. */
typedef struct symgb_mlp* symgb_mlp_t;
int symgb_mlp_create(int inputs, int hidden, unsigned long long seed, symgb_mlp_t* out);
int symgb_mlp_num_params(symgb_mlp_t net);
int symgb_mlp_get_params(symgb_mlp_t net, float* params);
int symgb_mlp_set_params(symgb_mlp_t net, const float* params);
int symgb_mlp_forward(symgb_mlp_t net, const float* X, int n, float* y);
int symgb_mlp_gradient(symgb_mlp_t net, const float* X, const float* y, int n, float* grad, float* loss);
int symgb_mlp_train(symgb_mlp_t net, const float* X, const float* y, int n, int epochs, float lr, float* loss);
void symgb_mlp_destroy(symgb_mlp_t net);

/* Plan statistics (host side, no device needed). */
typedef struct symgb_stats {
    uint64_t num_kernels, num_levels;
    uint64_t num_inputs, num_outputs, num_intermediates;
    uint64_t index_entries, constant_entries;
    uint64_t flops;           /* per value set: adds, muls, negations */
    uint64_t divs, sqrts, transcendentals;
    uint64_t gathers;         /* x reads per value set */
    uint64_t max_registers;   /* largest per-thread register file of a kernel program */
    uint64_t program_words;   /* total device program length (64-bit words) */
    uint64_t bundles;         /* per value set: compute bundles dispatched (instances x bundles) */
    uint64_t bundle_entries;  /* per value set: operations in those bundles */
} symgb_stats;
int symgb_get_stats(symgb_unit_t u, symgb_stats* s);

/* Algorithmic bytes of one evaluation of `num_sets` value sets:
 * 8 N_in + 8 N_out + 16 N_int per set plus the index and constant tables once. */
uint64_t symgb_algorithmic_bytes(symgb_unit_t u, int num_sets);

/* Introspection: the device program of kernel k for a math mode (64-bit words
 * as executed by the interpreter kernels: the load section, then the compute
 * bundles, an end word and the literal table).  Writes up to `cap` words, the register count and the length of
 * the load section; returns the program length in words, or a negative error. */
int64_t symgb_kernel_program(symgb_unit_t u, int k, int math, uint64_t* words, uint64_t cap, int* registers,
                             int* num_loads);

/* Versioned plan file (host only; no device needed).  Stores a plan
 * description with its index, output-index and constant tables, so a plan
 * built once by the front end can be reloaded without rebuilding it.  It
 * extends the reference's raw table files indexData / constData / outIndexData
 * (src/Utilities.hpp:156-161) with the plan metadata and templates the
 * reference bakes into generated source, a format version and a checksum.
 * symgb_plan_load validates the file (magic, version, byte order, checksum,
 * sizes) and returns SYMGB_ERR_ARGUMENT for anything else; the loaded
 * description and tables live until symgb_plan_file_free.  Errors of these
 * calls are described by symgb_plan_last_error(). */
typedef struct symgb_plan_file* symgb_plan_file_t;
int symgb_plan_save(const char* path, const symgb_plan_desc* plan, const uint32_t* index_data,
                    const uint32_t* out_index_data, const double* const_data);
int symgb_plan_load(const char* path, symgb_plan_file_t* out);
const symgb_plan_desc* symgb_plan_file_desc(symgb_plan_file_t f);
const uint32_t* symgb_plan_file_index_data(symgb_plan_file_t f);
const uint32_t* symgb_plan_file_out_index_data(symgb_plan_file_t f);
const double* symgb_plan_file_const_data(symgb_plan_file_t f);
void symgb_plan_file_free(symgb_plan_file_t f);
const char* symgb_plan_last_error(void);

/* The step after assembly: batched Jacobi-preconditioned Krylov solves of
 * A x = b for symmetric A (the reference's cloth example assembles
 * A = M - h (D + h K) and b for an implicit step,
 * examples/BaraffWitkin/implementation/cloth.cpp:96-111, and keeps the lower
 * triangle of A, examples/BaraffWitkin/main.cpp:56).  The pattern is given
 * once on the host as CSC (col_ptr[n + 1], row_idx[nnz]; lower_only = 1 for a
 * lower triangle, 0 for the full matrix); num_sets systems (1..256) share it.
 * symgb_solver_solve takes device pointers: values [set][nnz] in the
 * pattern's order (e.g. symgb_get_result_sets_device of the unit that
 * assembles A), b and x [set][n].  Methods: conjugate gradient (A positive
 * definite) or BiCGSTAB (any nonsingular A; the cloth matrices of a deformed
 * sheet are indefinite).  It starts from x = 0 and stops once every system's
 * |r| / |b| <= tol (checked every 16 iterations) or after max_iter
 * iterations, reporting both.  symgb_solver_multiply computes q = A p. */
#define SYMGB_SOLVER_CG 0
#define SYMGB_SOLVER_BICGSTAB 1
typedef struct symgb_solver* symgb_solver_t;
int symgb_solver_create(int64_t n, const int64_t* col_ptr, const int32_t* row_idx, int lower_only, int num_sets,
                        symgb_solver_t* out);
int symgb_solver_solve(symgb_solver_t s, int method, const double* values, const double* b, double* x, double tol,
                       int max_iter, void* stream, int* iterations, double* max_rel_residual);
int symgb_solver_multiply(symgb_solver_t s, const double* values, const double* p, double* q, void* stream);
/* Block-Jacobi preconditioning for BiCGSTAB: the inverses of the b x b
 * diagonal blocks (b = block_size, 2..4; 1 restores the scaled Jacobi
 * default) of the unknowns {j b, ..., j b + b - 1} (stride 1) or
 * {j, j + stride, ..., j + (b - 1) stride} (stride = n / b: each coordinate's
 * unknowns stored together, e.g. a 3-D mesh's x, y and z rows n / 3 apart).
 * A block with a zero pivot falls back to the scaled Jacobi of its rows. */
int symgb_solver_set_block_preconditioner(symgb_solver_t s, int block_size, int64_t stride);
void symgb_solver_destroy(symgb_solver_t s);

/* Measured FP64 FMA throughput of the current device (FLOP/s, one FMA = 2). */
int symgb_measure_fp64_rate(double* flops_per_second);

/* Allocation-free evaluation, for callers that cannot allocate device memory
 * (a framework that owns all device memory through its own pool, or code that
 * must not allocate once running).  It has no counterpart in the reference.
 * The unit needs only symgb_unit_create (not symgb_init, which allocates).
 * Tables are host pointers (as for symgb_init), inputs[i] and outputs[k] are
 * device pointers to input container i and output container k (one value set).
 * All working memory - x, tables, programs, tiles and barrier state - lives in
 * one static device array of SYMGB_STATIC_SCRATCH_BYTES that every GPU loading
 * this entry point keeps until exit; plans that need more are rejected with
 * SYMGB_ERR_ARGUMENT.  No cudaMalloc / cudaFree or other allocating call is
 * made on the device side; on the host each call still builds the plan's
 * tables, programs and tiles in temporary host buffers and copies them into
 * the array, so its host cost grows with the plan.  The first call on a device
 * looks up the array's device address.  Every call reads a status word back
 * on `stream` and waits for `stream` before it returns, so a call cannot be
 * recorded into a CUDA graph.  Calls share the array; calls from several
 * threads must not overlap. */
#define SYMGB_STATIC_SCRATCH_BYTES (32ull << 20)
int symgb_run_static(symgb_unit_t u, const uint32_t* index_data, const uint32_t* out_index_data,
                     const double* const_data, const double* const* inputs, double* const* outputs, void* stream);

/* Number of kernel launches the last run issued (graph replays count the
 * kernels inside the graph). */
int symgb_last_launch_count(symgb_unit_t u);

#ifdef __cplusplus
}
#endif
#endif /* SYMGB_H */
