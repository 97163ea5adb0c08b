/*
 * vulkpy_gb300.h -- C ABI of the GB300 (sm_103a) array engine.
 *
 * This is the drop-in boundary that replaces vulkpy's native module
 * `_vkarray` (vulkpy/_vkarray.cc:756-898, pybind11) and the GLSL compute
 * shaders it dispatches (vulkpy/shader/*.comp).  Every entry point takes
 * plain pointers and sizes, returns an int status (VKC_OK == 0), and
 * records a message retrievable with vkc_last_error() on failure.
 *
 * Memory passed to the compute entry points is device memory obtained from
 * vkc_alloc() (or any device pointer valid in the device's CUDA context).
 * All work is issued, in order, on the device's compute stream; nothing
 * blocks the host except the explicit wait / copy-to-host calls.
 *
 * Each declaration names the reference interface it replaces (file:line,
 * paths inside the vulkpy project).
 */
#ifndef VULKPY_GB300_H
#define VULKPY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define VKC_OK            0
#define VKC_ERR_INVALID   1  /* bad argument (shape, size, op code, NULL)   */
#define VKC_ERR_OOM       2  /* device or pinned host allocation failed      */
#define VKC_ERR_CUDA      3  /* a CUDA runtime / driver call failed           */
#define VKC_ERR_TIMEOUT   4  /* vkc_job_wait deadline passed (not an error of the GPU) */

/* ---- op codes -------------------------------------------------------- */
/* binary / scalar ops: vulkpy/shader/{add,sub,mul,div,pow,max,min}*.comp,
 * r{sub,div,pow}_scalar.comp */
enum vkc_binary_op {
  VKC_ADD = 0, VKC_SUB = 1, VKC_MUL = 2, VKC_DIV = 3,
  VKC_POW = 4, VKC_MAX = 5, VKC_MIN = 6,
  VKC_RSUB = 7, VKC_RDIV = 8, VKC_RPOW = 9  /* reversed: op(other, self) */
};

/* unary ops: vulkpy/shader/{abs,sign,sin,...,invsqrt}.comp */
enum vkc_unary_op {
  VKC_ABS = 0, VKC_SIGN = 1, VKC_SIN = 2, VKC_COS = 3, VKC_TAN = 4,
  VKC_ASIN = 5, VKC_ACOS = 6, VKC_ATAN = 7, VKC_SINH = 8, VKC_COSH = 9,
  VKC_TANH = 10, VKC_ASINH = 11, VKC_ACOSH = 12, VKC_ATANH = 13,
  VKC_EXP = 14, VKC_LOG = 15, VKC_EXP2 = 16, VKC_LOG2 = 17,
  VKC_SQRT = 18, VKC_INVSQRT = 19,
  VKC_COPY = 20          /* identity; used by broadcast_to */
};

/* reductions: vulkpy/shader/{sum,prod,maximum,minimum}{,_v1.3,_axis,_axis_rebroadcast}.comp */
enum vkc_reduce_op { VKC_SUM = 0, VKC_PROD = 1, VKC_MAXIMUM = 2, VKC_MINIMUM = 3 };

/* index reductions (numpy argmax/argmin; listed as missing in README.md:73) */
enum vkc_arg_op { VKC_ARGMAX = 0, VKC_ARGMIN = 1 };

/* summation precision for VKC_SUM / VKC_PROD over axis=None */
enum vkc_reduce_precision {
  VKC_RED_PLAIN = 0,        /* per-thread sequential fp32, tree combine          */
  VKC_RED_PAIRWISE = 1,     /* 16 fp32 accumulators per thread, tree combine      */
  VKC_RED_COMPENSATED = 2   /* Neumaier per thread, TwoSum tree, fp64 cross-block */
};

/* matmul arithmetic */
enum vkc_matmul_precision {
  VKC_MM_FP32 = 0,   /* SIMT fp32 FMA (the drop-in default)                   */
  VKC_MM_BF16 = 1,   /* tcgen05 bf16 x bf16 -> fp32 accumulate                */
  VKC_MM_BF16X3 = 2  /* tcgen05 split-bf16: hi*hi + hi*lo + lo*hi, fp32 acc   */
};

/* activation fused into the Dense epilogue */
enum vkc_activation { VKC_ACT_NONE = 0, VKC_ACT_RELU = 1, VKC_ACT_SIGMOID = 2 };

/* losses (vulkpy/nn/losses.py): CrossEntropyLoss, SoftmaxCrossEntropyLoss,
 * MSELoss, HuberLoss */
enum vkc_loss { VKC_LOSS_CE = 0, VKC_LOSS_SCE = 1, VKC_LOSS_MSE = 2, VKC_LOSS_HUBER = 3 };

typedef struct vkc_device* vkc_device_t;  /* one GPU + its streams        */
typedef struct vkc_job* vkc_job_t;        /* completion marker (an event) */

/* ---- errors ---------------------------------------------------------- */
/* Message of the last failing call on this thread ("" if none).
 * Replaces the std::runtime_error texts of vulkpy/_vkarray.cc:32,286,451,454,508. */
const char* vkc_last_error(void);
/* Library version string. */
const char* vkc_version(void);

/* ---- device: vulkpy/_vkarray.cc:460-574 (class GPU), createGPU 759-763 ---- */
int vkc_device_count(int* count);
/* Open GPU `index`.  `priority` in [0,1] maps to a CUDA stream priority
 * (replaces the queue priority of _vkarray.cc:472-485). */
int vkc_device_open(int index, float priority, vkc_device_t* out);
int vkc_device_close(vkc_device_t dev);
/* Block until all work issued on the device is done (GPU.wait, _vkarray.cc:560-562). */
int vkc_device_synchronize(vkc_device_t dev);
/* The cudaStream_t all compute entry points use (as void*). */
int vkc_device_stream(vkc_device_t dev, void** stream);
/* Route subsequent work to `stream` (a cudaStream_t of the same device, e.g.
 * torch's current stream); NULL restores the device's own stream.  For the
 * legacy default stream (handle 0 in most frameworks) pass cudaStreamLegacy
 * ((void*)1): NULL would select the device's own non-blocking stream, which
 * is not ordered with work on the default stream. */
int vkc_device_set_stream(vkc_device_t dev, void* stream);
/* Number of SMs and the device name (for logs and grid sizing). */
int vkc_device_info(vkc_device_t dev, int* sm_count, char* name, size_t name_len);
/* Read-and-clear the device error word: bit0 = a gather index was out of
 * range.  Synchronises the compute stream. */
int vkc_device_check_errors(vkc_device_t dev, uint32_t* flags);

/* ---- memory: Buffer<T> (_vkarray.cc:38-130), GPU::toBuffer/createBuffer ---- */
/* Stream-ordered device allocation on the compute stream (cudaMallocAsync).
 * Size 0 returns NULL and VKC_OK. */
int vkc_alloc(vkc_device_t dev, size_t bytes, void** ptr);
/* Stream-ordered free: safe while kernels that use `ptr` are still queued. */
int vkc_free(vkc_device_t dev, void* ptr);
/* Pinned (page-locked) host memory, for host mirrors and fast copies. */
int vkc_host_alloc(size_t bytes, void** ptr);
int vkc_host_free(void* ptr);
/* Upload into NEW device memory on the copy stream: allocates `bytes`,
 * copies from `src`, makes the compute stream wait for the copy, and blocks
 * the host only until the copy itself is done (not queued compute work).
 * Replaces GPU::toBuffer (_vkarray.cc:511-517, Buffer ctor 81-86). */
int vkc_upload(vkc_device_t dev, const void* src, size_t bytes, void** dptr);
/* vkc_upload without the host wait: returns once the copy is queued on the
 * copy stream; the compute stream waits for it on the device, and `*job`
 * completes with the copy.  `src` must be pinned (vkc_host_alloc) and stay
 * unchanged until `*job` completes.  No reference counterpart (vulkpy's
 * Buffer constructor copies synchronously, _vkarray.cc:81-86); lets the
 * upload of the next batch overlap the current compute. */
int vkc_upload_async(vkc_device_t dev, const void* src, size_t bytes, void** dptr, vkc_job_t* job);
/* Device->host copy into pinned `dst` on a separate read-back stream, after
 * every op issued so far on the compute stream but not after ops issued
 * later, without a host wait; `*job` completes with the copy.  Lets the
 * read-back of one batch's results overlap the next batch's compute.  Keep
 * `src` allocated and `dst` untouched until `*job` completes.  No reference
 * counterpart (vulkpy reads mapped memory, vkarray.py:186-188). */
int vkc_d2h_async(vkc_device_t dev, void* dst, const void* src, size_t bytes, vkc_job_t* job);
/* Make the compute stream wait (on the device) for `job`, e.g. before
 * reusing memory that an asynchronous copy still reads. */
int vkc_stream_wait_job(vkc_device_t dev, vkc_job_t job);
/* Host->device copy into existing memory, ordered after queued compute work.
 * A pageable `src` is staged before the call returns.  A pinned `src` is
 * read when the stream reaches the copy: keep it unchanged until `*job`
 * completes (pass job = NULL only for pageable sources). */
int vkc_h2d(vkc_device_t dev, void* dst, const void* src, size_t bytes, vkc_job_t* job);
/* Device->host copy after all queued compute work; blocks until done.
 * Replaces the mapped-memory read of _GPUArray.__array__ (vkarray.py:186-188). */
int vkc_d2h(vkc_device_t dev, void* dst, const void* src, size_t bytes);
/* Fill n floats with v (zeros(), Constant initializer; vkarray.py:1524-1542). */
int vkc_fill_f32(vkc_device_t dev, float* dst, size_t n, float v);
int vkc_fill_u32(vkc_device_t dev, uint32_t* dst, size_t n, uint32_t v);
int vkc_copy(vkc_device_t dev, void* dst, const void* src, size_t bytes);

/* ---- jobs: class Job (_vkarray.cc:392-457), Job.wait(timeout) 876-879 ---- */
/* Marker for "everything issued so far"; wait() on it = Array.wait(). */
int vkc_job_record(vkc_device_t dev, vkc_job_t* job);
/* Wait with a deadline (timeout_ns < 0: no deadline).  Returns VKC_ERR_TIMEOUT
 * with "Timeout at Command Wait" like _vkarray.cc:451. */
int vkc_job_wait(vkc_job_t job, int64_t timeout_ns);
/* *done = 1 when complete, 0 otherwise (non-blocking). */
int vkc_job_query(vkc_job_t job, int* done);
int vkc_job_destroy(vkc_job_t job);
/* Timing marker (a CUDA event with timing) on the compute stream, and the
 * elapsed milliseconds between two completed markers.  No reference
 * counterpart (vulkpy has no timers); used for CUDA-event benchmarking. */
int vkc_timer_record(vkc_device_t dev, vkc_job_t* job);
int vkc_job_elapsed_ms(vkc_job_t start, vkc_job_t end, float* ms);
/* Number of kernels this library has launched since load (all devices). */
int vkc_launch_count(uint64_t* count);
/* Programmatic dependent launch for the kernels of the training step (the
 * tensor-core GEMM, its operand pre-pass and split-K reduction, the Dense
 * backward's bias sums, the loss step, the grouped Adam): each may be
 * scheduled while the kernel before it on the stream finishes, and waits
 * on the device for its results.  On by default; enable = 0 launches them
 * as ordinary kernels.  No reference counterpart. */
int vkc_set_pdl(int enable);
/* Split-K inside the tensor-core GEMM: when a product is split over 2..8 K
 * ranges, the CTAs of one output tile run as a thread-block cluster, store
 * their partial sums, meet on a cluster mbarrier and each adds up its share
 * of the tile's rows (in K-range order, the same sums and epilogue as the
 * separate reduction launch, so the same bits).  Only for launches outside
 * a stream capture.  Off by default: it saves a launch's host cost (an
 * eager MLP step 6.1k -> 6.4k steps/s) but costs device time (in a CUDA
 * graph the separate reduction, overlapped by programmatic dependent
 * launch, gives 10.4k against 8.7k steps/s; an eager 1024^3 bf16 product
 * 0.022 against 0.026 ms).  No reference counterpart. */
int vkc_set_cluster_splitk(int enable);
/* The Dense backward (vkc_dense_backward*) runs the bias sum and the weight
 * GEMM on branch streams forked from the device's stream and joins them back
 * before it returns.  After vkc_side_defer(dev, 1) the joins wait: branches
 * forked by later calls queue behind the earlier ones, and
 * vkc_side_defer(dev, 0) joins them all back into the device's stream (the
 * gradients are complete on it from then on).  A training step defers
 * across its backward pass, so the weight GEMMs of every layer overlap the
 * chain of input-gradient GEMMs.  No reference counterpart. */
int vkc_side_defer(vkc_device_t dev, int defer);
/* Work on the side branch: after vkc_side_begin(dev) the device's calls go
 * to the side stream, which first waits for everything issued so far on the
 * device's stream and on the bias-sum branch; vkc_side_end(dev) returns to
 * the device's stream and joins the branch back (or, under vkc_side_defer,
 * leaves it for that join).  Sequence.train runs each layer's optimizer
 * step there as soon as the layer's gradients are issued.  Only from the
 * device's own stream.  No reference counterpart. */
int vkc_side_begin(vkc_device_t dev);
int vkc_side_end(vkc_device_t dev);
/* Number of device and pinned-host allocations this library has requested
 * since load (vkc_alloc, vkc_upload, vkc_host_alloc and every scratch
 * allocation inside an op).  No reference counterpart; lets a caller check
 * that a call allocated nothing. */
int vkc_alloc_count(uint64_t* count);
/* Device memory the device's stream-ordered pools hold now (reserved, in use
 * or cached): the pool of the compute stream's allocations and the pool of
 * uploads.  Diagnostics; no reference counterpart. */
int vkc_pool_reserved(vkc_device_t dev, uint64_t* compute_bytes, uint64_t* upload_bytes);
/* Host-side fault injection for the allocation error path (the reference
 * turns Vulkan allocation errors into RuntimeError, _vkarray.cc:32, 61-72):
 * the allocation request `after` requests from now (0 = the next one) fails
 * with VKC_ERR_OOM without calling CUDA; then injection switches itself
 * off.  after < 0 switches it off.  Touches no GPU. */
int vkc_inject_alloc_failure(int64_t after);

/* ---- fused elementwise kernels (no reference counterpart: vulkpy runs one
 * shader per op).  `source` is CUDA C defining
 *   extern "C" __global__ void <name>(P p)
 * with struct P { const float* in[8]; float* out[4]; unsigned long long n; };
 * it is compiled once per device with NVRTC for this GPU (-fmad=false) and
 * cached.  launch: in/out are 16-byte aligned device arrays of n floats. */
typedef struct vkc_kernel* vkc_kernel_t;
int vkc_jit_compile(vkc_device_t dev, const char* source, const char* name, vkc_kernel_t* kernel);
int vkc_jit_launch(vkc_device_t dev, vkc_kernel_t kernel, const float* const* in, int n_in,
                   float* const* out, int n_out, size_t n);

/* ---- CUDA graphs (no reference counterpart: vulkpy submits every op as
 * its own Vulkan job, _vkarray.cc:403-438) ---------------------------------
 * begin: start capturing the device's stream; every entry point called on
 * this thread is recorded instead of run (stream-ordered allocations become
 * graph memory nodes; uploads from the host are refused while capturing).
 * end: stop and instantiate; allocations still live at the end are re-made
 * at the same addresses on every launch.  launch: replay on the stream. */
typedef struct vkc_graph* vkc_graph_t;
/* Extra streams for independent work (e.g. one branch per model): create a
 * non-blocking stream on the device, and make `waiter` wait for everything
 * queued on `signaler` so far (an event record + wait; inside a capture this
 * becomes a graph dependency, so fork/join patterns capture as parallel
 * branches).  Route work to a stream with vkc_device_set_stream. */
int vkc_stream_create(vkc_device_t dev, void** stream);
int vkc_stream_destroy(vkc_device_t dev, void* stream);
int vkc_stream_wait(vkc_device_t dev, void* waiter, void* signaler);
int vkc_graph_begin(vkc_device_t dev);
int vkc_graph_end(vkc_device_t dev, vkc_graph_t* graph);
int vkc_graph_launch(vkc_graph_t graph);
int vkc_graph_destroy(vkc_graph_t graph);

/* ---- elementwise ---------------------------------- */
/* c[i] = a[i] op b[i] for i < n; c may alias a or b (in-place i*.comp twins).
 * vulkpy/vkarray.py:440-452 (_opVec/_opVec3), shaders add.comp:20-26 etc. */
int vkc_binary(vkc_device_t dev, int op, const float* a, const float* b, float* c, size_t n);
/* c[i] = a[i] op s  (op < VKC_RSUB), or s op' a[i] for VKC_RSUB/RDIV/RPOW.
 * vkarray.py:469-483 (_opVecScalar*), add_scalar.comp:19-24, rsub_scalar.comp. */
int vkc_binary_scalar(vkc_device_t dev, int op, const float* a, float s, float* c, size_t n);
/* c[i] = f(a[i]); c may alias a.  vkarray.py:680-1098, exp.comp:18-23 etc. */
int vkc_unary(vkc_device_t dev, int op, const float* a, float* c, size_t n);
/* d[i] = min(max(a[i], lo), hi) with lo/hi arrays (lo_arr/hi_arr non-NULL,
 * length n) or scalars.  vkarray.py:1110-1191, clamp{,_sv,_vs,_ss}.comp. */
int vkc_clamp(vkc_device_t dev, const float* a, const float* lo_arr, const float* hi_arr,
              float lo, float hi, float* d, size_t n);

/* ---- broadcasting --------------------------------- */
/* numpy broadcasting of a and b into c.  Shapes are given right-aligned and
 * already padded to `ndim` (<= 16) entries; a dim of 1 broadcasts.  c may
 * alias a when a has c's shape (in-place i*_broadcast.comp).
 * vkarray.py:499-519, 538-557; add_broadcast.comp:25-45, iadd_broadcast.comp:22-41. */
int vkc_broadcast_binary(vkc_device_t dev, int op,
                         const float* a, const int64_t* a_shape,
                         const float* b, const int64_t* b_shape,
                         float* c, const int64_t* c_shape, int ndim);
/* c = clamp(a, lo, hi) with every operand broadcast to c_shape; lo/hi NULL
 * means the scalar lo_s/hi_s.  Replaces clamp's broadcast_to copies (vkarray.py:1147-1160). */
int vkc_broadcast_clamp(vkc_device_t dev,
                        const float* a, const int64_t* a_shape,
                        const float* lo, const int64_t* lo_shape, float lo_s,
                        const float* hi, const int64_t* hi_shape, float hi_s,
                        float* c, const int64_t* c_shape, int ndim);
/* Explicit broadcast copy.  vkarray.py:1434-1474, broadcast.comp:25-44. */
int vkc_broadcast_to(vkc_device_t dev, const float* a, const int64_t* a_shape,
                     float* c, const int64_t* c_shape, int ndim);

/* ---- reductions -------------------------------------------- */
/* out[0] = reduce(a[0..n)) * scale (scale applies to SUM/PROD only; pass 1).
 * vkarray.py:1246-1274 (axis=None), sum.comp:18-30, sum_v1.3.comp:20-29. */
int vkc_reduce_all(vkc_device_t dev, int op, int precision, const float* a, size_t n,
                   float* out, float scale);
/* The same launches and result as vkc_reduce_all, bit for bit, for callers
 * that cannot allocate device memory during the call (a host that hands the
 * whole device heap to its own allocator, or a latency-critical path where
 * an allocation could block or fail).  No counterpart in the reference.  The block partials
 * live in a fixed 1 MiB device array inside the library, so n is limited to
 * 2^29 elements (larger n: VKC_ERR_INVALID).  The first call on a device
 * looks the array up (make it before capturing the stream); calls on one
 * device share the array, so calls that overlap on the GPU race.  Allocates
 * nothing: no cudaMalloc/cudaFree, no pool. */
int vkc_reduce_all_noalloc(vkc_device_t dev, int op, int precision, const float* a, size_t n,
                           float* out, float scale);
/* View a as [prev, axis, post]; out[i, j] = reduce_k a[i, k, j] * scale.
 * With rebroadcast != 0, out has a's shape and every k gets the result.
 * vkarray.py:1194-1244, sum_axis.comp:20-32, sum_axis_rebroadcast.comp:20-35. */
int vkc_reduce_axis(vkc_device_t dev, int op, const float* a, size_t prev, size_t axis,
                    size_t post, float* out, int rebroadcast, float scale);

/* ---- matmul ----------------------------------------------------- */
/* C[M,N] = A[M,K] @ B[K,N], row-major fp32 in and out.
 * vkarray.py:585-605, matmul.comp:23-33. */
int vkc_matmul(vkc_device_t dev, int precision, const float* a, const float* b, float* c,
               int64_t m, int64_t k, int64_t n);
/* General form used by the nn layers: C = alpha * op(A) @ op(B) + beta * C,
 * op(X) = X or X^T (trans flags), leading dimensions in elements. */
int vkc_gemm(vkc_device_t dev, int precision, int trans_a, int trans_b,
             int64_t m, int64_t n, int64_t k, float alpha,
             const float* a, int64_t lda, const float* b, int64_t ldb,
             float beta, float* c, int64_t ldc);

/* Tuning table of the tensor-core GEMM, keyed by precision and the log2 size
 * buckets of (m, n, k): the CTA tile width (tile_n = 128 or 256 columns of C
 * per 128-row tile) and the split-K count; splits = 0 removes an entry.  The
 * table written by vulkpy_gb300/autotune.py is loaded at import; shapes
 * without an entry use 256-wide tiles and an occupancy heuristic for splits.
 * get: the plan a shape will use.  tune_set/tune_get are the same with
 * tile_n = 256 / without it.  No reference counterpart (matmul.comp has no
 * tiling). */
int vkc_gemm_plan_set(int precision, int64_t m, int64_t n, int64_t k, int splits, int tile_n);
int vkc_gemm_plan_get(vkc_device_t dev, int precision, int64_t m, int64_t n, int64_t k, int* splits,
                      int* tile_n);
int vkc_gemm_tune_set(int precision, int64_t m, int64_t n, int64_t k, int splits);
int vkc_gemm_tune_get(vkc_device_t dev, int precision, int64_t m, int64_t n, int64_t k, int* splits);
int vkc_gemm_tune_clear(void);

/* ---- grouped (batched, uneven) GEMM and MLP-step pieces --------- */
/* No counterpart in the reference, which runs every Dense layer of every
 * model as its own job (nn/layers.py:94-141, batch_affine.comp:25-39,
 * _vkarray.cc:403-438).  One problem of a grouped call:
 *   C = act(alpha * op(A) op(B) + beta * C + bias), then, when relu_mask is
 *   not NULL, C *= max(sign(relu_mask), 0) elementwise (relu_mask has C's
 *   layout: the ReLU backward of layers.py:176-181 fused into the GEMM). */
typedef struct vkc_gemm_problem {
  int32_t ta, tb;           /* op(A) = A^T when ta, op(B) = B^T when tb */
  int64_t m, n, k;
  float alpha, beta;
  const float* a;
  int64_t lda;
  const float* b;
  int64_t ldb;
  float* c;
  int64_t ldc;
  const float* bias;        /* per column of C, may be NULL */
  int32_t act;              /* vkc_activation, applied before relu_mask */
  const float* relu_mask;   /* may be NULL */
} vkc_gemm_problem;
/* All `count` problems in persistent launches (128 problems per launch):
 * the output tiles of every problem form one work list, longest K first.
 * fp32: bit-identical to vkc_gemm per problem.  bf16x3: bit-identical to
 * vkc_gemm when that call does not split K; bf16: accumulated per 64-wide K
 * block in fp32 (at least as accurate as vkc_gemm's bf16). */
int vkc_gemm_grouped(vkc_device_t dev, int precision, const vkc_gemm_problem* problems, int count);
/* A parameter step fused into a grouped gradient GEMM: for every problem i
 * with updates[i].value not NULL, after C is stored (the gradient, kept),
 * value[r * ldc + c] += scale * C[r * ldc + c] -- the SGD step of
 * optimizers.py:24-60 with scale = float(-lr), in the arithmetic of
 * vkc_sgd_update_grouped, so the parameters equal a vkc_gemm_grouped call
 * followed by that update bit for bit.  C and the value are contiguous
 * m x n (ldc = n); such problems must be plain products (alpha 1, beta 0,
 * no bias, activation or mask) whose own operands are not the value.  Other
 * problems of the call may read the value as an operand and see it before
 * the step (dx = dy W beside W's step).  `updates` may be NULL (then this is
 * vkc_gemm_grouped).  The tensor-core path applies the step in the GEMM's
 * epilogue when its problems fit one launch (128); otherwise, and on the
 * fp32 path and for K = 0, one separate update runs after every product. */
typedef struct vkc_gemm_update {
  float* value;
  float scale;
} vkc_gemm_update;
int vkc_gemm_grouped_update(vkc_device_t dev, int precision, const vkc_gemm_problem* problems,
                            const vkc_gemm_update* updates, int count);
/* db[i][o] += sum_b dy[i][b, o] for every item (the bias gradient of
 * layers.py:125-128), b in order, one launch per 128 items; with
 * `overwrite` db[i][o] = the sum (equal to accumulating into a zeroed db). */
int vkc_colsum_grouped(vkc_device_t dev, const float* const* dy, float* const* db, const int64_t* batch,
                       const int64_t* cols, int count, int overwrite);
/* vkc_colsum_grouped, then value[i][o] += scale[i] * db[i][o] in the same
 * launch for every item whose value[i] is not NULL (the bias step of
 * optimizers.py:24-60, arithmetic as in vkc_sgd_update_grouped). */
int vkc_colsum_update_grouped(vkc_device_t dev, const float* const* dy, float* const* db, const int64_t* batch,
                              const int64_t* cols, int count, int overwrite, float* const* value,
                              const float* scale);
/* value[i] += (-lr) * grad[i] for every tensor (optimizers.py:24-60). */
int vkc_sgd_update_grouped(vkc_device_t dev, float* const* value, const float* const* grad, const int64_t* n,
                           double lr, int count);
/* Adam for `count` tensors with shared hyperparameters in one launch, each
 * with its own moments and running powers (double[3] as for
 * vkc_adam_update_dev); per tensor the result equals vkc_adam_update_dev's.
 * Replaces one AdamState.grad2diff + Parameter.update per tensor
 * (optimizers.py:221-253, parameters.py:88-95). */
int vkc_adam_update_grouped(vkc_device_t dev, float* const* value, const float* const* grad,
                            float* const* m, float* const* v, double* const* powers, const int64_t* n,
                            int count, double lr, double beta1, double beta2, double eps);
/* dst[i][0..n[i]) = v for every tensor: Sequence's zero_grad of every
 * parameter in one launch (parameters.py:81-86, models.py:47-49). */
int vkc_fill_f32_grouped(vkc_device_t dev, float* const* dst, const int64_t* n, float v, int count);
/* MSELoss with reduce="mean" for many models (losses.py:252-320 with
 * ReduceLoss 40-92): dx[i] = ((x - y) * 2) * float32(1/batch) (when dx is
 * not NULL) and loss[i] = mean over rows of sum over columns of (y - x)^2
 * (when loss is not NULL, at most 256 models; summation order differs from
 * the per-op path, the value agrees to rounding). */
int vkc_mse_grouped(vkc_device_t dev, const float* const* x, const float* const* y, float* const* dx,
                    const int64_t* batch, const int64_t* cols, float* loss, int count);

/* ---- gather ------------------------------------------------------ */
/* c[i] = a[idx[i]], i < n_idx.  An index >= n_a writes NaN and sets bit0 of
 * the device error word.  c must not overlap a.  Tables of >= 2^25 floats
 * gathered by >= 2^21 indices (16-byte aligned idx and c) take a binned
 * form: indices partitioned by table window in chunks of 4096, each window
 * read while it is in L2, values put back in order -- three launches and
 * scratch of 6 bytes per index (the direct kernel if that cannot be had).
 * vkarray.py:1476-1500, gather.comp:21-26. */
int vkc_gather(vkc_device_t dev, const float* a, size_t n_a, const uint32_t* idx,
               size_t n_idx, float* c);
/* Which form vkc_gather takes: 0 = by size (default), 1 = always the direct
 * kernel, 2 = the binned form whenever idx and c are 16-byte aligned and
 * n_idx < 2^32.  Both give the same values.  No reference counterpart. */
int vkc_set_gather_bins(int mode);
/* c[k, i, j] = a[i, min(idx[k], axis-1), j]; output [n_idx, prev, post].
 * vkarray.py:1501-1521, gather_axis.comp:24-43, U32Array.to_onehot 239-253. */
int vkc_gather_axis(vkc_device_t dev, const float* a, size_t prev, size_t axis, size_t post,
                    const uint32_t* idx, size_t n_idx, float* c);

/* ---- index reductions and permutations (no reference kernel) ---- */
/* The reference names argmax/argmin as missing (README.md:73) and its
 * training example computes them with numpy on the host
 * (example/02-nn.py:96).  numpy semantics: the first index of the extreme
 * value, the first NaN if any, -0.0 == +0.0.  out[0] = index; n < 2^32. */
int vkc_arg_reduce_all(vkc_device_t dev, int op, const float* a, size_t n, uint32_t* out);
/* out[p, q] = arg-extreme over k of a[p, k, q], k < axis < 2^32. */
int vkc_arg_reduce_axis(vkc_device_t dev, int op, const float* a, size_t prev, size_t axis, size_t post,
                        uint32_t* out);
/* out[0..n) = a pseudo-random permutation of 0..n-1, keyed by four uint32
 * drawn from the state stream (as vkc_xoshiro_u32 with n = 4): a 6-round
 * Feistel network on the smallest even-bit domain >= n, cycle-walked into
 * [0, n).  Replaces the host shuffle of example/02-nn.py:82 ("TODO:
 * Implement GPU shuffle()"); README.md:77 lists shuffle as missing. */
int vkc_xoshiro_permutation(vkc_device_t dev, uint32_t* state, uint32_t size, uint32_t* out, size_t n);

/* ---- xoshiro128++ PRNG ---------------------------------------- */
/* Fill state[4*size] (device) exactly like PRNG::Xoshiro128pp's constructor
 * (_vkarray.cc:643-675): four chained splitmix64 words, then state i is the
 * reference's jump() applied i times, computed in parallel on the GPU from
 * precomputed powers of the (linear, GF(2)) jump map. */
int vkc_xoshiro_seed(vkc_device_t dev, uint64_t seed, uint32_t size, uint32_t* state);
/* n outputs from `size` states with the reference's chunked layout:
 * out[k] = next^(k / size)(state[k % size]); states advance in place.
 * Replaces Xoshiro128pp::random (_vkarray.cc:697-717) and
 * prng_xoshiro128pp_{uint32,float}.comp:26-44.  One launch per call. */
int vkc_xoshiro_u32(vkc_device_t dev, uint32_t* state, uint32_t size, uint32_t* out, size_t n);
int vkc_xoshiro_f32(vkc_device_t dev, uint32_t* state, uint32_t size, float* out, size_t n);
/* Normal numbers: the uniform stream of vkc_xoshiro_f32 of length n (n even)
 * or n+1 (n odd) transformed pairwise by Box-Muller, fused in one launch when
 * `size` is even.  random.py:60-124, prng_{i,}box_muller.comp. */
int vkc_xoshiro_normal(vkc_device_t dev, uint32_t* state, uint32_t size, float* out, size_t n,
                       float mean, float stddev);
/* Box-Muller on an existing uniform buffer u[0..2*ceil(n/2)) into out[0..n)
 * (out may alias u).  prng_box_muller.comp:19-32, prng_ibox_muller.comp:16-27. */
int vkc_box_muller(vkc_device_t dev, const float* u, float* out, size_t n, float mean, float stddev);
/* out[i] = low + uint(float(high_incl - low + 1) * u_i) with u_i drawn from
 * the state stream (fused).  random.py:126-186, prng_randrange.comp:20-27. */
int vkc_xoshiro_randrange(vkc_device_t dev, uint32_t* state, uint32_t size, uint32_t* out,
                          size_t n, uint32_t low, uint32_t high_incl);

/* ---- nn fused kernels ---------------------------------------- */
/* y[b,o] = act(sum_i w[o,i] x[b,i] + bias[o]).  nn/layers.py:94-102, batch_affine.comp:25-39. */
int vkc_dense_forward(vkc_device_t dev, int precision, const float* x, const float* w,
                      const float* bias, float* y, int64_t batch, int64_t in_dim,
                      int64_t out_dim, int act);
/* A stack of Dense layers, y[l] = act[l](in_l W[l]^T + bias[l]) with in_0 = x
 * and in_l = y[l-1], dims[0..layers] the widths (layer l: dims[l] ->
 * dims[l+1]), the same results as vkc_dense_forward layer by layer bit for
 * bit (models.py:40-53 runs the layers one after the other).  On the
 * tensor-core path the operand pre-pass of layer l+1's input is written by
 * layer l's split-K reduction (or one pre-pass launch when it has none), and
 * the weights of layers 1.. are split on a side stream at the start: one
 * launch fewer on the chain per layer after the first.  bias[l] may be
 * NULL. */
int vkc_dense_stack_forward(vkc_device_t dev, int precision, int layers, const float* x, int64_t batch,
                            const int64_t* dims, const float* const* w, const float* const* bias,
                            const int* act, float* const* y);
/* Given dy (already multiplied by the activation derivative when act != NONE
 * is applied by the caller), accumulate dW += dy^T x, db += sum_b dy and write
 * dx = dy @ w (dx may be NULL).  nn/layers.py:104-141 without the (B,out,in)
 * temporary of layers.py:131-135. */
int vkc_dense_backward(vkc_device_t dev, int precision, const float* x, const float* w,
                       const float* dy, float* dx, float* dw, float* db,
                       int64_t batch, int64_t in_dim, int64_t out_dim);
/* An activation layer's backward followed by the preceding Dense layer's
 * (nn/layers.py:158-267 then 104-141): dy = act'(y) * dy_act with the
 * activation backward's float32 operations (act VKC_ACT_RELU or
 * VKC_ACT_SIGMOID, y the activation output), stored in dy [batch, out_dim];
 * then db += sum_b dy (rows in order), dW += dy^T x, dx = dy @ w (dx, dw, db
 * may be NULL).  The activation backward and the bias sum share one launch;
 * results equal vkc_activation_backward then vkc_dense_backward bit for bit. */
int vkc_dense_backward_act(vkc_device_t dev, int precision, const float* x, const float* w,
                           const float* dy_act, const float* y, int act, float* dy, float* dx,
                           float* dw, float* db, int64_t batch, int64_t in_dim, int64_t out_dim);
/* vkc_dense_backward_act (act VKC_ACT_RELU / VKC_ACT_SIGMOID) or, with act
 * VKC_ACT_NONE, vkc_dense_backward of dy_act (y and dy unused), with
 * accumulate == 0 writing dW and db instead of adding to them: the values
 * adding into zeroed gradients gives, without a zeroing pass.  The
 * reference zeroes every gradient before each backward (Sequence.train,
 * models.py:55-78, Parameter.zero_grad, parameters.py:81-86). */
int vkc_dense_backward_ex(vkc_device_t dev, int precision, const float* x, const float* w,
                          const float* dy_act, const float* y, int act, float* dy, float* dx,
                          float* dw, float* db, int64_t batch, int64_t in_dim, int64_t out_dim,
                          int accumulate);
/* vkc_dense_backward_ex with act VKC_ACT_NONE (dW, db from dy; accumulate as
 * there), with the backward of the activation below this layer fused into
 * the input-gradient GEMM: dx = (dy W) * act'(dx_y), dx_act VKC_ACT_RELU or
 * VKC_ACT_SIGMOID and dx_y that activation's output (batch x in_dim), in the
 * activation backward's float32 operations -- the dy of the Dense layer
 * below, so the results equal vkc_dense_backward_ex then
 * vkc_dense_backward_act's activation step bit for bit.  dx_act
 * VKC_ACT_NONE: plain dx.  The tensor-core path applies the derivative in
 * the GEMM's epilogue or split-K reduction (models.py:55-78 runs the two
 * layers' backward one after the other). */
int vkc_dense_backward_chain(vkc_device_t dev, int precision, const float* x, const float* w,
                             const float* dy, const float* dx_y, int dx_act, float* dx, float* dw,
                             float* db, int64_t batch, int64_t in_dim, int64_t out_dim, int accumulate);
/* Row softmax over the last axis of [rows, cols] (nn/layers.py:297-300). */
int vkc_softmax(vkc_device_t dev, const float* x, float* y, int64_t rows, int64_t cols);
/* loss_rows[r] = sum_c -y log(p + 1e-8) with p = softmax(x) when softmax != 0
 * (else p = x); nn_cross_entropy.comp:21-26, losses.py:140-176, 218-249. */
int vkc_cross_entropy(vkc_device_t dev, const float* x, const float* y, float* loss_rows,
                      float* p_out, int64_t rows, int64_t cols, int softmax);
/* The softmax-cross-entropy loss step of one batch in one launch instead
 * of three (losses.py:179-249 with ReduceLoss, losses.py:40-92): p_out =
 * softmax(x) per row, dx = (p - y) * grad_scale, and *loss = (sum over rows
 * of sum_c -y log(p + 1e-8)) * loss_scale, the rows added with the
 * arithmetic of vkc_reduce_axis over a (rows,) vector, so the results equal
 * vkc_cross_entropy + vkc_reduce_axis + vkc_softmax_ce_backward bit for bit.
 * rows 1..2048.  The last block of the launch adds up the rows (an arrival
 * counter of the device, back at zero after each call): calls on one device
 * must not run concurrently on different streams. */
int vkc_softmax_ce_fused(vkc_device_t dev, const float* x, const float* y, float* p_out, float* dx,
                         float* loss, int64_t rows, int64_t cols, float loss_scale, float grad_scale);
/* Adam step (optimizers.py:221-253) on n parameters, fused:
 * m = b1 m + (1-b1) g; v = b2 v + (1-b2) g^2;
 * value += -lr * (m / (1-b1t)) / (sqrt(v / (1-b2t)) + eps).  beta1t/beta2t
 * are the running powers after this step's update.  Hyper-parameters are
 * doubles (Python floats): each scalar is formed in double and rounded to
 * float32 exactly where the reference hands it to a float32 array op, so
 * the result is bit-identical to the reference's unfused chain. */
int vkc_adam_update(vkc_device_t dev, float* value, const float* grad, float* m, float* v,
                    size_t n, double lr, double beta1, double beta2, double eps,
                    double beta1t, double beta2t);
/* Adam with the running powers beta1^t, beta2^t kept on the device
 * (`powers` = double[3], start at {1, 1, 0}; the third slot is the kernel's
 * completion counter and is back at 0 after every call).  The update uses
 * beta1^t * beta1 and beta2^t * beta2 (in double), exactly as
 * AdamState.grad2diff advances them on the host, and the last block of the
 * same launch stores the advanced powers, so a captured step can be
 * replayed.  Same result as vkc_adam_update.  Calls on one `powers` buffer
 * must not overlap on the GPU. */
int vkc_adam_update_dev(vkc_device_t dev, float* value, const float* grad, float* m, float* v,
                        size_t n, double lr, double beta1, double beta2, double eps, double* powers);
/* dx = dy * f'(y) from the activation output y: ReLU dy * max(sign(y), 0)
 * (layers.py:187-210); Sigmoid and Softmax (diagonal) (1 - y) * y * dy
 * (layers.py:246-267, 302-323); same float32 op order as the reference. */
int vkc_activation_backward(vkc_device_t dev, int act, const float* y, const float* dy, float* dx,
                            size_t n);
/* Softmax cross entropy gradient (p - y) * scale (losses.py:229-249 with the
 * ReduceLoss scaling of losses.py:70-86); dx may alias p. */
int vkc_softmax_ce_backward(vkc_device_t dev, const float* p, const float* y, float* dx, size_t n,
                            float scale);
/* Float64 versions of vkc_dense_forward/backward, vkc_activation_backward,
 * vkc_cross_entropy and vkc_softmax_ce_backward: the same hand-written
 * math in double, for checking gradients against float64 finite
 * differences.  No reference counterpart (vulkpy is float32 only). */
int vkc_dense_forward_f64(vkc_device_t dev, const double* x, const double* w, const double* bias,
                          double* y, int64_t batch, int64_t in_dim, int64_t out_dim, int act);
int vkc_dense_backward_f64(vkc_device_t dev, const double* x, const double* w, const double* dy,
                           double* dx, double* dw, double* db, int64_t batch, int64_t in_dim,
                           int64_t out_dim);
int vkc_activation_backward_f64(vkc_device_t dev, int act, const double* y, const double* dy,
                                double* dx, size_t n);
int vkc_cross_entropy_f64(vkc_device_t dev, const double* x, const double* y, double* loss_rows,
                          double* p_out, int64_t rows, int64_t cols, int softmax);
int vkc_softmax_ce_backward_f64(vkc_device_t dev, const double* p, const double* y, double* dx,
                                size_t n, double scale);
/* Per-row loss, loss_rows[r] = sum_c term(x[r,c], y[r,c]) over [rows, cols]:
 * VKC_LOSS_CE -y log(x + 1e-8) (losses.py:95-176, nn_cross_entropy.comp:21-26);
 * VKC_LOSS_SCE the same of p = softmax(x), p stored in p_out when not NULL
 * (losses.py:179-249); VKC_LOSS_MSE (y - x)^2 (losses.py:252-320);
 * VKC_LOSS_HUBER 0.5 min(|y - x|, (y - x)^2) (losses.py:323-393).  The
 * batch reduction (ReduceLoss, losses.py:40-92) is the caller's. */
int vkc_loss_rows(vkc_device_t dev, int kind, const float* x, const float* y, float* loss_rows,
                  float* p_out, int64_t rows, int64_t cols);
/* Gradient of a weighted sum of losses, one pass over n elements:
 * dx = sum_j coeffs[j] * (grad_j * scales[j]), added in term order
 * (MixLoss, losses.py:396-458; one term is a single loss).  grad_j:
 * CE -y / (x + 1e-8) (nn_cross_entropy_backward.comp), SCE p - y
 * (losses.py:229-249, p from vkc_loss_rows), MSE 2 (x - y), Huber
 * clamp(x - y, -1, 1) as the reference (losses.py:376-393) or, with
 * huber_exact != 0, the derivative of its forward (x - y where
 * |x - y| <= 1, else 0.5 sign(x - y)).  scales[j] is the ReduceLoss
 * factor (1/batch for a mean, losses.py:70-86).  nterms 1..8; the term
 * tables are host memory.  float32 operations in the reference's order. */
int vkc_loss_backward(vkc_device_t dev, int nterms, const int* kinds, const double* coeffs,
                      const double* scales, int huber_exact, const float* x, const float* y,
                      const float* p, float* dx, size_t n);
/* Softmax backward with the full Jacobian: dx = y * (dy - sum_c dy y) per
 * row of [rows, cols].  The reference's Softmax.backward keeps only the
 * diagonal, dy y (1 - y) (layers.py:302-323; vkc_activation_backward with
 * VKC_ACT_SIGMOID reproduces it). */
int vkc_softmax_backward(vkc_device_t dev, const float* y, const float* dy, float* dx, int64_t rows,
                         int64_t cols);
/* Standalone ReLU max(x, 0) (layers.py:158-185) and Sigmoid
 * 1 / (1 + exp(0 - x)) (layers.py:213-244, its four float32 array ops). */
int vkc_activation_forward(vkc_device_t dev, int act, const float* x, float* y, size_t n);
/* Float64 versions of the five entry points above, for finite-difference
 * gradient checks; vkc_softmax_f64 is vkc_softmax in double.  No reference
 * counterpart (vulkpy is float32 only). */
int vkc_loss_rows_f64(vkc_device_t dev, int kind, const double* x, const double* y,
                      double* loss_rows, double* p_out, int64_t rows, int64_t cols);
int vkc_loss_backward_f64(vkc_device_t dev, int nterms, const int* kinds, const double* coeffs,
                          const double* scales, int huber_exact, const double* x, const double* y,
                          const double* p, double* dx, size_t n);
int vkc_softmax_backward_f64(vkc_device_t dev, const double* y, const double* dy, double* dx,
                             int64_t rows, int64_t cols);
int vkc_activation_forward_f64(vkc_device_t dev, int act, const double* x, double* y, size_t n);
int vkc_softmax_f64(vkc_device_t dev, const double* x, double* y, int64_t rows, int64_t cols);
/* value += (-lr) * grad (optimizers.py:39-52). */
int vkc_sgd_update(vkc_device_t dev, float* value, const float* grad, size_t n, double lr);
/* h += g^2; value += (g / (sqrt(h) + eps)) * (-lr)  (optimizers.py:120-139). */
int vkc_adagrad_update(vkc_device_t dev, float* value, const float* grad, float* h, size_t n,
                       double lr, double eps);

#ifdef __cplusplus
}
#endif
#endif /* VULKPY_GB300_H */
