/* t1m_capi.h — C-ABI of libt1m_cuda.so, the GB300 (sm_103a) contraction engine.
 *
 * The reference (MatthiasReumann/t1m) is a header-only C++ library with no FFI;
 * its public boundary is the pair of t1m::contract templates
 * (include/t1m/t1m.h:560-568 real, :570-577 complex) over the non-owning
 * t1m::tensor view (include/t1m/t1m.h:31-66).  This header is the plain-C
 * surface those templates forward to in this project (include/t1m/t1m.h here
 * is the drop-in C++ API); every entry point below names the reference
 * interface it replaces.  No torch or CUDA types appear in the signatures:
 * streams are passed as void* (a cudaStream_t).
 *
 * Ownership: the caller owns every tensor.  Data pointers may be device
 * pointers (used in place) or host pointers (staged host->device and back by
 * the library, timed separately in the report).
 * Errors: every function returns a t1m_status (0 = success); the reference
 * only throws std::bad_alloc (t1m.h:455-458).
 * Threading: one context per host thread (or per stream); contexts share
 * nothing but read-only kernels.
 */
#ifndef T1M_CAPI_H
#define T1M_CAPI_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum t1m_status {
  T1M_OK = 0,
  T1M_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad dtype/rank/layout       */
  T1M_ERR_LABELS = 2,           /* label/extent mismatch, repeated label, a
                                   label in A, B and C (batch mode)          */
  T1M_ERR_ALLOC = 3,            /* device or host allocation failed (the
                                   reference's std::bad_alloc, t1m.h:455-458) */
  T1M_ERR_CUDA = 4,             /* a CUDA runtime call failed                */
  T1M_ERR_UNSUPPORTED = 5,      /* method not available for this dtype/shape */
  T1M_ERR_KERNEL_TIMEOUT = 6,   /* a bounded device-side wait ran out        */
  T1M_ERR_NO_DEVICE = 7         /* no CUDA device / not an sm_103 device     */
} t1m_status;

/* Element types: the reference's TensorScalar set (t1m.h:15-23). */
typedef enum t1m_dtype {
  T1M_FLOAT32 = 0,
  T1M_FLOAT64 = 1,
  T1M_COMPLEX64 = 2,  /* std::complex<float>, interleaved re/im  */
  T1M_COMPLEX128 = 3  /* std::complex<double>, interleaved re/im */
} t1m_dtype;

/* Memory layouts.  Values 0/1 match the reference's memory_layout enum
 * (t1m.h:29: row_major = 0, col_major = 1); the reference leaves row_major
 * strides uninitialised (t1m.h:51-52), here it is implemented.  T1M_STRIDED
 * takes explicit element strides. */
typedef enum t1m_layout {
  T1M_ROW_MAJOR = 0,
  T1M_COL_MAJOR = 1,
  T1M_STRIDED = 2
} t1m_layout;

/* How the contraction is computed on the GPU.  The reference always runs the
 * BLIS real micro-kernel on 1M-packed panels (t1m.h:508-554, mappings.h:91-99). */
typedef enum t1m_method {
  T1M_METHOD_AUTO = 0,       /* pick per dtype and shape; FP32 partials are
                                kept short enough for 1e-6 against FP64 (K
                                split, partials and epilogue in FP64)        */
  T1M_METHOD_PLAIN = 1,      /* SIMT FP32/FP64 FMA (the plain GPU form)      */
  T1M_METHOD_TC_3XTF32 = 2,  /* complex64: tcgen05 kind::tf32, hi/lo split,
                                3 products, FP32 accumulation in TMEM         */
  T1M_METHOD_TC_BF16X3 = 3,  /* complex64: tcgen05 kind::f16 (bf16), 2-way
                                split, 3 products                             */
  T1M_METHOD_TC_BF16X6 = 4,  /* complex64: bf16 3-way split, 6 products      */
  T1M_METHOD_DMMA = 5        /* complex128/float64: FP64 tensor MMA          */
} t1m_method;

/* A tensor view: the C form of t1m::tensor<T, ndim> (t1m.h:31-66). */
typedef struct t1m_tensor {
  int32_t ndim;            /* number of modes (>= 0)                          */
  int32_t layout;          /* t1m_layout                                      */
  const int64_t* extents;  /* ndim extents                                    */
  const int64_t* strides;  /* ndim element strides; read iff T1M_STRIDED      */
  void* data;              /* host or device pointer                          */
} t1m_tensor;

/* Filled by t1m_contract when non-null. */
typedef struct t1m_report {
  int32_t method;      /* t1m_method that ran                               */
  int32_t split_k;     /* K partitions (1 = none)                           */
  int64_t m, n, k;     /* matricised sizes (products of bundle extents)     */
  double flops;        /* 8*M*N*K complex, 2*M*N*K real                     */
  double kernel_ms;    /* device time of the compute kernels (CUDA events)  */
  double h2d_ms;       /* host->device staging time (0 for device operands) */
  double d2h_ms;       /* device->host staging time                         */
  int64_t h2d_bytes;
  int64_t d2h_bytes;
  int32_t kernels;     /* kernels launched by this call                     */
  int32_t path;        /* tensor-core products: T1M_PATH_* code of the last
                          product (how its operands were fetched); 0 for
                          the plain and FP64 kernels                         */
  double main_ms;      /* device time of the last tensor-core product's main
                          kernel alone (without its split, pack, panel and
                          split-K reduction passes); timed single calls with
                          device operands only, else 0                       */
} t1m_report;

/* t1m_report.path: bit 12 marks a tensor-core product; bits 0-3 the fetch
 * mode of A, bits 4-7 that of B; bit 8 the persistent kernel (else one tile
 * per CTA); bits 9/10 A/B densely repacked first (then loaded by TMA).
 * Bit 11 (T1M_PATH_PAIR): clusters of two CTAs share each MMA.
 * A modes: 0 gathered, 1 one TMA box [k][m], 2 TMA boxes per 16-row block of
 * unit-stride rows, 3 one TMA box [m][k], 4 per 16-row block with unit-stride
 * K, 5 per 16-row block and 16-K block (adjoint operands).
 * B modes: 0 gathered, 1 one TMA box [n][k], 2 one box [k][n], 3 per 16-column
 * block with unit-stride K, 4 per 16-column block and 16-K block (adjoint
 * operands), 5 B split once beforehand into panels (loaded by TMA). */
#define T1M_PATH_TC 0x1000
#define T1M_PATH_PAIR 0x800       /* CTA pairs (tcgen05 cta_group::2)        */
#define T1M_PATH_PERSISTENT 0x100
#define T1M_PATH_A_PACKED 0x200
#define T1M_PATH_B_PACKED 0x400
#define T1M_PATH_B_PANELS 5
#define T1M_PATH_PIECES 0x2000    /* CTA pairs over operands split into bf16
                                     pieces beforehand (T1M_TILE_PIECES)    */

typedef struct t1m_context t1m_context;

/* Flags for t1m_contract. */
#define T1M_FLAG_ACCUMULATE 1u /* reference semantics: C <- C + alpha*A*B,
                                  beta ignored (t1m.h:497-502, 543-548)     */
#define T1M_FLAG_CONJ_A 2u     /* use conj(A) (adjoint contractions)        */
#define T1M_FLAG_CONJ_B 4u     /* use conj(B)                               */
#define T1M_FLAG_NO_TIMING 8u  /* skip the CUDA events of the report        */

/* Create a context on `device` (the BLIS context slot of the reference,
 * `const cntx_t* cntx = bli_gks_query_cntx()`, t1m.h:566/575, becomes this
 * handle: stream, method and plan cache). */
int t1m_create(t1m_context** ctx, int device);
int t1m_destroy(t1m_context* ctx);
/* Run on a caller-owned cudaStream_t (NULL = the context's own stream).
 * Switching waits for the work queued on the previous stream (the context's
 * workspaces are shared by its calls). */
int t1m_set_stream(t1m_context* ctx, void* stream);
int t1m_set_method(t1m_context* ctx, int method);
/* Number of K partitions (split-K with an FP64 reduction of the partial
 * products); 0 = automatic (split when the output has too few tiles to fill
 * the GPU).  The reference streams K in KC chunks inside one thread
 * (t1m.h:512-548); this is its parallel counterpart. */
int t1m_set_split_k(t1m_context* ctx, int splits);
/* Cap, in bytes, on each optional workspace of the tensor-core products: B
 * split once into panels, and dense repacks of operands that would otherwise
 * be gathered element by element.  Products whose workspace would exceed it
 * run without (same results, bit for bit; only speed changes).  -1 (the
 * default) = no cap, 0 = never use them.  For callers with a tight device
 * memory budget; the split-K workspace is not optional and not capped here.
 * No reference counterpart (the reference packs into one aligned_alloc'ed
 * buffer per call, t1m.h:450-460). */
int t1m_set_workspace_limit(t1m_context* ctx, int64_t bytes);
/* Bound, in microseconds, on the device-side waits of grouped launches for
 * the items they depend on (0, the default: about two seconds).  Applies to
 * groups created afterwards.  A wait that runs out sets the error word, and
 * the call that synchronises next returns T1M_ERR_KERNEL_TIMEOUT. */
int t1m_set_wait_limit(t1m_context* ctx, int64_t microseconds);
/* Tile form of single tensor-core contractions (complex64).  T1M_TILE_PAIR
 * runs clusters of two CTAs whose MMAs (tcgen05 cta_group::2, 256 x 128 real
 * tiles) each read half of B from either CTA, where both operands load by
 * TMA; T1M_TILE_ONE keeps one 128 x 128 tile per CTA; T1M_TILE_AUTO (the
 * default) picks pairs where they apply.  The reference's counterpart is
 * BLIS's choice of micro-tile and cache blocking (bli/mappings.h:101-142). */
#define T1M_TILE_AUTO 0
#define T1M_TILE_ONE 1
#define T1M_TILE_PAIR 2
/* CTA pairs whose MMAs read both operands from shared memory, loaded by TMA
 * from copies split once into bf16 pieces (the bf16 methods; the copies
 * take the optional workspace: 2P bytes per real value of the 1M-expanded A
 * and of B, P = 3 pieces for BF16x6, 2 for BF16x3).  Same results as
 * T1M_TILE_PAIR, bit for bit.  Elsewhere it runs as T1M_TILE_PAIR. */
#define T1M_TILE_PIECES 3
int t1m_set_tile_form(t1m_context* ctx, int form);
/* Autotuning of single tensor-core contractions (on != 0; default off): per
 * shape class (element type, method, log2 of M, N and K, which operand
 * directions have unit stride) the tile form (one CTA or CTA pairs) and the
 * split-K count (the heuristic count, half or twice it, never below the
 * automatic method's precision minimum) are measured once on the call's own
 * operands, into scratch outputs, and the fastest is cached in the same file
 * as the grouped launches' choices ($T1M_TUNE_CACHE).  Applies when the tile
 * form and the split count are automatic.  The reference's counterpart is
 * BLIS's fixed block sizes (bli/mappings.h:101-142). */
int t1m_set_autotune(t1m_context* ctx, int on);
int t1m_synchronize(t1m_context* ctx);
const char* t1m_status_string(int status);
const char* t1m_last_error(const t1m_context* ctx);
/* Library version and the compute capability it was built for (103). */
int t1m_version(int* major, int* minor, int* sm);

/* Contract A and B into C by label strings (einstein notation).
 * Replaces t1m::contract (t1m.h:560-577).
 *
 * alpha, beta point to one scalar of `dtype` (complex: re, im).  Without
 * T1M_FLAG_ACCUMULATE: C <- alpha*A*B + beta*C (BLAS semantics; beta == 0
 * does not read C).  With it: C <- C + alpha*A*B exactly like the reference
 * (which ignores beta, and uses alpha = 1 for complex types).
 * Bundles follow the reference (t1m.h:90-136): contracted = labels of A and B,
 * free labels of A then B must appear in C.  Unlike the reference, empty
 * bundles (outer products, full contractions to a 0-mode C) are allowed. */
int t1m_contract(t1m_context* ctx, int dtype, const void* alpha,
                 const t1m_tensor* a, const char* labels_a, const t1m_tensor* b,
                 const char* labels_b, const void* beta, const t1m_tensor* c,
                 const char* labels_c, uint32_t flags, t1m_report* report);

/* Adjoint (vector-Jacobian product) of C = A*B for a real loss L, in the
 * conjugate-Wirtinger convention PyTorch uses for complex autograd:
 *   dA = dC * conj(B)   (labels: dC[labels_c], B[labels_b] -> dA[labels_a])
 *   dB = conj(A) * dC   (labels: A[labels_a], dC[labels_c] -> dB[labels_b])
 * da or db may be NULL (not computed).  Without T1M_FLAG_ACCUMULATE the
 * gradients are overwritten, with it they are added.  Both products run on
 * the same kernels as t1m_contract with conjugate-on-load, so the method and
 * split-K settings of the context apply.  No counterpart in the reference
 * (which has no differentiation); the report (if any) sums both products. */
int t1m_contract_vjp(t1m_context* ctx, int dtype, const t1m_tensor* dc,
                     const char* labels_c, const t1m_tensor* a, const char* labels_a,
                     const t1m_tensor* b, const char* labels_b, const t1m_tensor* da,
                     const t1m_tensor* db, uint32_t flags, t1m_report* report);

/* Grouped batches: many contractions of uneven shapes (for example the
 * updates of a tensor-network sweep) run as grouped launches instead of one
 * launch per call.  The reference has no batching (its counterpart is a loop
 * of t1m::contract calls, t1m.h:560-577).  All tensors are device pointers.
 * An item may read the C of an EARLIER item (depends_on = its index).
 * By default items run per dependency level as one launch per family
 * (tensor cores for complex64 items with at least 32 rows and columns, the
 * grouped plain kernel otherwise, a skinny tile for outputs with at most 16
 * columns) and one split-K reduction; when every item is a tensor-core item
 * the batch is one persistent launch with the dependencies resolved in the
 * kernel.  With T1M_GROUP_ONE_LAUNCH a complex64 batch (context method other
 * than PLAIN) is always ONE persistent launch of the tensor-core kernel:
 * every item with its own tile (16, 32, 64 or 128 output columns on the
 * tensor cores, or a SIMT tile for outputs of at most 8 columns),
 * dependencies resolved in the kernel (a tile of a dependent item waits for
 * every output tile of its dependency), and items with a long K split
 * across CTAs and reduced in the kernel (FP64 sum and epilogue by the split
 * that finishes last).  With T1M_GROUP_AUTOTUNE the family (per-family
 * launches) or the tile (one launch) of each shape class (log2 buckets of M,
 * N, K) is measured once and cached in a versioned file ($T1M_TUNE_CACHE,
 * default $HOME/.cache/t1m_gb300_tune.txt, keyed by GPU name, SM count and
 * driver).  With T1M_GROUP_GRAPH the launches are captured once into a CUDA
 * graph that t1m_group_launch replays. */
typedef struct t1m_group_item {
  const t1m_tensor* a;
  const char* labels_a;
  const t1m_tensor* b;
  const char* labels_b;
  const t1m_tensor* c;
  const char* labels_c;
  double alpha[2];     /* re, im (im ignored for real dtypes) */
  double beta[2];
  int32_t depends_on;  /* index of an earlier item whose C this item reads, or -1 */
  uint32_t flags;      /* T1M_FLAG_ACCUMULATE / _CONJ_A / _CONJ_B */
} t1m_group_item;

typedef struct t1m_group t1m_group;

#define T1M_GROUP_GRAPH 1u
#define T1M_GROUP_AUTOTUNE 2u
/* Failure injection for tests of the timeout path (host side; no fault on
 * the GPU): every dependent item of a single persistent launch waits for one
 * more tile than its dependency writes, a count nothing reaches.  Its bounded
 * waits run out (t1m_set_wait_limit), its remaining stages are drained
 * without loads, the launch completes, and t1m_group_launch reports
 * T1M_ERR_KERNEL_TIMEOUT; the context stays usable.  Outputs of such a
 * launch are undefined. */
#define T1M_GROUP_INJECT_UNMET_DEPENDENCY 4u
/* complex64 batches as one persistent launch (see above). */
#define T1M_GROUP_ONE_LAUNCH 8u
/* One-launch batches: the tile of every item with more than 8 output columns
 * forced to 16, 32, 64 or 128 columns on the tensor cores (exactly one of
 * these bits; tests and measurements); narrower outputs stay SIMT tiles. */
#define T1M_GROUP_TILE_16 16u
#define T1M_GROUP_TILE_32 32u
#define T1M_GROUP_TILE_64 64u
#define T1M_GROUP_TILE_128 128u

int t1m_group_create(t1m_context* ctx, int dtype, int n, const t1m_group_item* items,
                     uint32_t options, t1m_group** group);
/* Run the batch on the context's stream; with a report, wait and time it. */
int t1m_group_launch(t1m_group* group, t1m_report* report);
int t1m_group_destroy(t1m_group* group);

/* Contraction that allocates no memory.  No counterpart in the reference
 * (which allocates its packing workspace with aligned_alloc on every call,
 * t1m.h:450-460).
 *
 * For callers that cannot call cudaMalloc/cudaFree: applications that own all
 * device memory through their own pool or a fixed budget, and loops where an
 * allocation or a device-synchronising cudaFree is not acceptable.
 * t1m_contract allocates plan buffers, staging buffers and a split-K
 * workspace; this entry point instead uses one fixed scratch array of
 * T1M_NOALLOC_SCRATCH_BYTES that the library holds on every GPU that loads it
 * until the process exits (scatter vectors, split-K partial products, the
 * kernels' error word).  Same semantics, methods, flags and status codes as
 * t1m_contract, with these differences:
 *   - a, b, c must be device pointers; `stream` is a cudaStream_t (NULL = the
 *     legacy default stream); the call waits for that stream before returning;
 *   - a contraction whose scatter vectors do not fit the scratch is rejected
 *     (T1M_ERR_UNSUPPORTED); the split-K count shrinks to fit;
 *   - all calls share the one scratch array and each overwrites it: calls that
 *     overlap on the GPU (other host threads or streams) race;
 *   - the first call on a device looks up the scratch address; make that call
 *     before any stream capture.  The address is kept for the life of the
 *     process: calls after cudaDeviceReset are not supported.
 * On failure a message is written to err (err_len bytes, may be 0). */
#define T1M_NOALLOC_SCRATCH_BYTES (64u << 20)
int t1m_contract_noalloc(void* stream, int method, int dtype, const void* alpha,
                         const t1m_tensor* a, const char* labels_a, const t1m_tensor* b,
                         const char* labels_b, const void* beta, const t1m_tensor* c,
                         const char* labels_c, uint32_t flags, char* err,
                         int32_t err_len);

/* Result of label analysis (no GPU needed). */
typedef struct t1m_plan_info {
  int64_t m, n, k;           /* products of the free-A, free-B, contracted extents */
  int32_t modes_m, modes_n, modes_k;
  int32_t reserved;
} t1m_plan_info;

/* Validate labels/extents/strides and report the matricised sizes without
 * touching the GPU.  Replaces the reference's get_index_bundles and
 * matrix_layout (t1m.h:90-136, 246-268), with the validation the reference
 * lacks.  On failure a message is written to err (err_len bytes, may be 0). */
int t1m_analyze(int dtype, const t1m_tensor* a, const char* labels_a,
                const t1m_tensor* b, const char* labels_b, const t1m_tensor* c,
                const char* labels_c, t1m_plan_info* info, char* err,
                int32_t err_len);

#ifdef __cplusplus
}
#endif

#endif /* T1M_CAPI_H */
