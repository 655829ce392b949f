/* pdt.h -- C ABI of the GB300 primal-dual TV/TGV^2 engine (libpdt.so).
 *
 * The reference (VLOGroup/primal-dual-toolbox) exposes C++ class templates and a boost.python module;
 * this header is the plain-C boundary those surfaces sit on here. Every entry point names the reference
 * interface it replaces (file:line inside the reference project). All functions return a pdt_status;
 * on failure pdt_last_error() returns a thread-local message that mirrors the text of the reference's
 * IuException at the same throw site.
 *
 * Conventions
 *   - Sizes are given in ImageUtilities order, fastest dimension first: an image is {W (phase-encode),
 *     H (frequency-encode)}, Cartesian k-space is {W, H, coils}. A numpy array of shape (C, H, W) in C
 *     order has exactly this memory layout.
 *   - Complex data is interleaved float pairs (complex64 / float2).
 *   - `is_device` = 1: pointers are device pointers on the current device; 0: host pointers (pinned or
 *     pageable). The caller owns every buffer it passes; handles own constants and solver state.
 *   - `stream` is a cudaStream_t (NULL = the legacy default stream). Calls enqueue work on `stream`
 *     and return when host buffers may be reused; pdt_opt_solve with a NULL stream returns after the
 *     solve has finished (the reference's solve() is synchronous through its timer).
 *   - One handle is used by one thread at a time.
 */
#ifndef PDT_H
#define PDT_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define PDT_API __attribute__((visibility("default")))
#else
#define PDT_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pdt_status {
  PDT_OK = 0,
  PDT_ERR_INVALID_ARGUMENT = 1, /* null handle / pointer, unknown enum value, bad ndim */
  PDT_ERR_SIZE = 2,             /* IU_SIZE_CHECK failures (e.g. mricartesianoperator.cu:177-179) */
  PDT_ERR_CONSTANTS = 3,        /* constant count / index / type (operatorbase.h:241-256, 266-287, 493-502) */
  PDT_ERR_CONFIG = 4,           /* OpConfig count or parse (operatorbase.h:219-228, 404-480) */
  PDT_ERR_STATE = 5,            /* "No operator is set!", "No noisy data is set!" (tgvmrioptimizer.cu:96-110) */
  PDT_ERR_CUDA = 6,             /* a CUDA runtime error */
  PDT_ERR_UNSUPPORTED = 7,      /* a size or kind this build does not handle */
  PDT_ERR_NUMERIC = 8,          /* non-finite values detected */
  PDT_ERR_TIMEOUT = 9,          /* a bounded device wait gave up */
  PDT_ERR_ALLOC = 10            /* device or pinned allocation failed */
} pdt_status;

typedef enum pdt_dtype {
  PDT_F32 = 0, /* float  (reference floatX = float, python/pyDenoising.cpp:26-29) */
  PDT_C64 = 1  /* float2 (reference complexX, python/pyMriReconstruction.cpp:39-42) */
} pdt_dtype;

typedef enum pdt_op_kind {
  PDT_OP_CARTESIAN = 0,         /* MriCartesianOperator          (mricartesianoperator.h:31-70) */
  PDT_OP_CARTESIAN_ROOS = 1,    /* MriCartesianRemoveROOSOperator (mricartesianoperator.h:72-118) */
  PDT_OP_SAMPLING = 2,          /* MriSamplingOperator           (mrisamplingoperator.h:30-66) */
  PDT_OP_RADIAL = 3,            /* MriRadialOperator             (mriradialoperator.h:35-95) */
  PDT_OP_RADIAL_SINGLECOIL = 4  /* MriRadialSinglecoilOperator   (mriradialoperator.h:97-155) */
} pdt_op_kind;

typedef enum pdt_opt_kind {
  PDT_OPT_TV = 0,      /* TvOptimizer         (tvoptimizer.h:47-121) */
  PDT_OPT_TGV = 1,     /* TgvOptimizer        (tgvoptimizer.h:70-142) */
  PDT_OPT_TV_OP = 2,   /* TvOptimizerWithOp   (tvoptimizerwithop.h:30-100) */
  PDT_OPT_TGV_OP = 3,  /* TgvOptimizerWithOp  (tgvoptimizerwithop.h:30-113) */
  PDT_OPT_TGV_MRI = 4  /* TgvMriOptimizer     (tgvmrioptimizer.h:73-150) */
} pdt_opt_kind;

/* One OpConfig entry (operatorbase.h:52-151: std::map<std::string, std::string>). */
typedef struct pdt_kv {
  const char* key;
  const char* value;
} pdt_kv;

/* Union of TvParameters (tvoptimizer.h:31-45), TgvParameters (tgvoptimizer.h:34-66) and
 * TgvMriParameters (tgvmrioptimizer.h:32-66); fields an optimizer does not use are ignored.
 * Defaults as in the reference constructors: alpha0 = alpha1 = lambda = reduction = 1,
 * max_iter = 1, check = 100. */
typedef struct pdt_params {
  double alpha0;
  double alpha1;
  double lambda;
  double reduction;
  uint32_t max_iter;
  uint32_t check;
} pdt_params;

typedef struct pdt_op pdt_op;
typedef struct pdt_opt pdt_opt;

/* ---- library ------------------------------------------------------------------------------------ */
PDT_API const char* pdt_last_error(void);  /* replaces IuException::what() across the ABI */
PDT_API int pdt_version(void);
/* Number of CUDA kernels this library has launched since it was loaded (graph replays count every
 * kernel node). Used by benchmarks to prove the native path ran. */
PDT_API uint64_t pdt_launch_count(void);
PDT_API pdt_status pdt_host_alloc(size_t bytes, void** out); /* pinned host memory for fast H2D/D2H */
PDT_API pdt_status pdt_host_free(void* p);
PDT_API pdt_status pdt_stream_synchronize(void* stream);

/* ---- operators (OperatorBase<InputType, OutputType>, operatorbase.h:196-507) ---------------------- */
/* Constructor. Cartesian / sampling operators take no config (ncfg = 0); radial operators need exactly
 * the four keys osf, sector_width, kernel_width, img_dim (mriradialoperator.cu:28-35). */
PDT_API pdt_status pdt_op_create(pdt_op_kind kind, const pdt_kv* cfg, int ncfg, pdt_op** out);
/* Releases the caller's reference; an optimizer that was given the operator keeps it alive
 * (the reference shares it through std::shared_ptr, tgvmrioptimizer.h:121). */
PDT_API pdt_status pdt_op_destroy(pdt_op* op);
/* OperatorBase::addConstant (operatorbase.h:238-257): positional constants, copied to the device.
 * Cartesian: #0 coil sensitivities C64 {W,H,C}, #1 mask F32 {W,H}. Sampling: #0 mask F32 {W,H}.
 * Radial: #0 trajectory F32 {Ns,2}, #1 dcf F32 {Ns,1}, #2 coil sensitivities C64 {N,N,C} (multi-coil). */
PDT_API pdt_status pdt_op_add_constant(pdt_op* op, pdt_dtype dtype, int ndim, const int64_t* size, const void* data,
                               int is_device);
/* Replaces constant `idx` with one of the same type and rank, ordered on `stream` (NULL: the legacy
 * default stream, synchronised before returning). No counterpart in the reference, whose constants can
 * only be appended; it lets one operator serve a sequence of slices without reallocation. The device
 * buffer is kept when the size is unchanged. An F32 constant (mask, trajectory, density weights) equal
 * to the current one is a no-op; a different one waits for the work already queued on `stream`, then
 * rebuilds the operator's tables (given on the device, it is first read back, waiting for `stream`). */
PDT_API pdt_status pdt_op_replace_constant(pdt_op* op, int idx, pdt_dtype dtype, int ndim, const int64_t* size,
                                           const void* data, int is_device, void* stream);
/* OperatorBase::getInputSize / getOutputSize (operatorbase.h:328-340). */
PDT_API pdt_status pdt_op_input_size(pdt_op* op, int out_ndim, const int64_t* out_size, int* in_ndim, int64_t* in_size);
PDT_API pdt_status pdt_op_output_size(pdt_op* op, int in_ndim, const int64_t* in_size, int* out_ndim, int64_t* out_size);
/* OperatorBase::forward / adjoint (operatorbase.h:297-312): constant-count and size checks, then
 * executeForward / executeAdjoint. src and dst are both device or both host buffers. */
PDT_API pdt_status pdt_op_forward(pdt_op* op, const void* src, int src_ndim, const int64_t* src_size, void* dst,
                          int dst_ndim, const int64_t* dst_size, int is_device, void* stream);
PDT_API pdt_status pdt_op_adjoint(pdt_op* op, const void* src, int src_ndim, const int64_t* src_size, void* dst,
                          int dst_ndim, const int64_t* dst_size, int is_device, void* stream);
/* OperatorBase::print (operatorbase.h:343-351), e.g. "MriCartesianOperator: Added constants: (2/2)". */
PDT_API pdt_status pdt_op_describe(pdt_op* op, char* buf, size_t len);
/* No reference counterpart: the kernel configuration the operator's autotuner picked (launch shapes timed
 * with CUDA events at set-up and cached per problem shape), as text. */
PDT_API pdt_status pdt_op_tuning(pdt_op* op, char* buf, size_t len);
/* adjointnessCheck (mricartesianoperator.cu:267-282 and siblings): random u, p (seeded), returns
 * <Au, p> and <u, A^H p> accumulated in double. */
PDT_API pdt_status pdt_op_adjointness(pdt_op* op, uint64_t seed, double out[4]);

/* ---- optimizers --------------------------------------------------------------------------------- */
/* dtype: PDT_F32 for the real denoising optimizers (*_2f), PDT_C64 for complex ones. */
PDT_API pdt_status pdt_opt_create(pdt_opt_kind kind, pdt_dtype dtype, pdt_opt** out);
PDT_API pdt_status pdt_opt_destroy(pdt_opt* opt);
/* getParameters() (tgvmrioptimizer.h:109-112): read and write the parameter struct. */
PDT_API pdt_status pdt_opt_get_params(pdt_opt* opt, pdt_params* out);
PDT_API pdt_status pdt_opt_set_params(pdt_opt* opt, const pdt_params* params);
/* setOperator (tgvmrioptimizer.cu:55-60). */
PDT_API pdt_status pdt_opt_set_operator(pdt_opt* opt, pdt_op* op);
/* setNoisyData (tgvmrioptimizer.cu:81-91): copies f to the device and resets the k-space dual r to 0. */
PDT_API pdt_status pdt_opt_set_noisy_data(pdt_opt* opt, const void* f, int ndim, const int64_t* size, int is_device,
                                  void* stream);
/* setInput0 (tgvmrioptimizer.cu:62-79): u = u-bar = input, v = v-bar = p = q = 0. */
PDT_API pdt_status pdt_opt_set_input0(pdt_opt* opt, const void* u0, int ndim, const int64_t* size, int is_device,
                              void* stream);
/* solve (tgvmrioptimizer.cu:93-203, tvoptimizer.cu:76-125, tgvoptimizer.cu:80-141, ...): runs
 * max_iter + 1 iterations from the current state (u0 = A^H f or f when no state is set). The
 * with-operator solvers check every new u and v for NaN and Inf on the device; with a NULL stream the
 * call returns PDT_ERR_NUMERIC when one appeared (the state then holds the non-finite iterate). */
PDT_API pdt_status pdt_opt_solve(pdt_opt* opt, int verbose, void* stream);
/* No counterpart in the reference, whose with-operator solvers fix tau = 1/16 (TGV-MRI) or 1/8 and
 * sigma = 1/8 (tgvmrioptimizer.cu:132-134, t*optimizerwithop.cu): the primal and dual step sizes of the
 * following solves of a with-operator optimizer; 0 restores the reference's value. Convergence needs
 * tau * sigma * |K|^2 < 1 for the solver's whole linear operator (about 13 for TGV with an operator of
 * norm 1). The reference's steps stay the default. */
PDT_API pdt_status pdt_opt_set_steps(pdt_opt* opt, double tau, double sigma);
/* No counterpart in the reference: the non-finite check of solves enqueued on an explicit stream. Waits
 * for `stream`, returns PDT_ERR_NUMERIC if a NaN or Inf appeared in u or v since the last check (and
 * clears the flag), else PDT_OK. */
PDT_API pdt_status pdt_opt_status(pdt_opt* opt, void* stream);
/* getResult (tgvmrioptimizer.cu:48-52): size query, then a copy of u into dst. */
PDT_API pdt_status pdt_opt_result_size(pdt_opt* opt, int* ndim, int64_t* size);
PDT_API pdt_status pdt_opt_get_result(pdt_opt* opt, void* dst, int is_device, void* stream);
/* No reference counterpart (the reference only prints the whole solve time, tgvmrioptimizer.cu:202):
 * runs `iters` further iterations launch by launch with a CUDA event after every kernel phase on
 * `stream` and returns each phase's mean duration in ms, phase names comma-separated in `names`.
 * The iterations advance the optimizer state exactly like solve(). */
PDT_API pdt_status pdt_opt_profile(pdt_opt* opt, int iters, void* stream, int max_phases, int* nphases, char* names,
                                   size_t names_len, double* ms);

/* ---- FP64 metrics and state access (no counterpart in the reference, which reports no energies) ----- */
/* setInput0 with the second TGV primal as well: u = u-bar = u0; v = v-bar = v0 (two planes vx then vy,
 * each the size of u0; v0 may be NULL); p = q = 0. */
PDT_API pdt_status pdt_opt_set_input0_uv(pdt_opt* opt, const void* u0, const void* v0, int ndim, const int64_t* size,
                                         int is_device, void* stream);
/* Copies one state plane: 0 u, 1 u-bar, 2 vx, 3 vy, 4 v-bar x, 5 v-bar y, 6 px, 7 py, 8 qxx, 9 qyy, 10 qxy
 * (each the size of u), or 11 the k-space dual r of a with-operator optimizer (the size of the noisy data,
 * in its layout; entries on phase-encode lines the mask never samples are not held and read as 0).
 * The reference keeps this state in TgvMriOptimizer's members u_, u__, v_, v__, p_, q_, r_
 * (tgvmrioptimizer.h:121-140) and has no accessor for it. */
PDT_API pdt_status pdt_opt_get_field(pdt_opt* opt, int field, void* dst, int is_device, void* stream);
/* Replaces one state plane (the fields of pdt_opt_get_field): planes 0-10 need an existing state
 * (setInput0 or a solve first), r needs the operator and the noisy data. The next solve() continues
 * from the new state, so exporting every field and importing it into a fresh optimizer resumes a solve
 * exactly. No counterpart in the reference, whose setInput0 / setNoisyData reset v, p, q and r to 0
 * (tgvmrioptimizer.cu:62-91). */
PDT_API pdt_status pdt_opt_set_field(pdt_opt* opt, int field, const void* src, int is_device, void* stream);
/* Energy of the current state accumulated in FP64: out = {total, data, first-order, second-order} --
 * 1/2 ||K u - f||^2 + alpha1 sum |grad u - v| + alpha0 sum |eps(v)| (TGV-MRI at its final alpha); the
 * TGV / TV with-operator optimizers weight the data term 1 / (2 lambda) (their r-prox), the denoising
 * optimizers lambda / 2 ||u - f||^2. */
PDT_API pdt_status pdt_opt_energy(pdt_opt* opt, void* stream, double out[4]);
/* Primal-dual gap of a with-operator optimizer (TGV-MRI, TGV / TV with operator) in FP64:
 * out = {gap, primal, dual, |div- p - K^H r|_2, |p + div_h- q|_2, |K^H r|_2} with primal the energy above,
 * dual = -Re<f, r> - lambda/2 |r|^2 (lambda = 1 for TGV-MRI; the k-space dual r continued by its limit
 * -f / lambda on phase-encode lines that are never sampled), and the two residuals of the dual
 * constraints K^H r = div- p and p = -div_h- q (0 for TV). gap -> 0 and both residuals -> 0 at the
 * saddle point. */
PDT_API pdt_status pdt_opt_gap(pdt_opt* opt, void* stream, double out[6]);
/* Operator norm ||K|| by `iters` power iterations on K^H K (FP64 norms). */
PDT_API pdt_status pdt_op_norm(pdt_op* op, int iters, uint64_t seed, double* out);
/* sum |a - b|^2 of two device arrays (b may be NULL) accumulated in FP64. */
PDT_API pdt_status pdt_dist2(pdt_dtype dtype, const void* a, const void* b, size_t n, void* stream, double* out);

/* ---- learned warm start (no counterpart in the reference) --------------------------------------- */
/* A residual CNN (8 convolutions, 32 channels, 3 x 3, BF16 weights and activations, FP32 accumulation)
 * mapping the zero-filled image u0 = A^H f to an initial (u, v) for the TGV^2 solvers. All image
 * pointers are device pointers: u0, u [B][H][W] complex64; v [B][2][H][W] complex64 (vx then vy).
 * Training minimises the mean squared error to target solutions (ut, vt), scaled per image by max|u0|. */
typedef struct pdt_cnn pdt_cnn;
PDT_API pdt_status pdt_cnn_create(uint64_t seed, pdt_cnn** out);
PDT_API pdt_status pdt_cnn_destroy(pdt_cnn* c);
PDT_API pdt_status pdt_cnn_num_params(pdt_cnn* c, size_t* n);
PDT_API pdt_status pdt_cnn_get_params(pdt_cnn* c, float* dst, size_t n);  /* host FP32 */
PDT_API pdt_status pdt_cnn_set_params(pdt_cnn* c, const float* src, size_t n);
PDT_API pdt_status pdt_cnn_get_grads(pdt_cnn* c, float* dst, size_t n);   /* gradients of the last step */
/* One forward + backward pass; with lr > 0 also one Adam step. *loss = mean over pixels of the summed
 * squared error of the six output channels. */
PDT_API pdt_status pdt_cnn_train_step(pdt_cnn* c, const void* u0, const void* ut, const void* vt, int B, int H,
                                      int W, float lr, void* stream, double* loss);
PDT_API pdt_status pdt_cnn_predict(pdt_cnn* c, const void* u0, int B, int H, int W, void* u, void* v, void* stream);

/* ---- batched solves ------------------------------------------------------------------------------ */
/* No counterpart in the reference (which solves one reconstruction per call): a batch advances many
 * independent optimizers together -- uneven sizes, coil counts, masks and iteration counts -- as parallel
 * branches of one captured CUDA graph, equivalent to calling pdt_opt_solve on each. Every optimizer
 * needs its own operator; optimizers must outlive the batch. */
typedef struct pdt_batch pdt_batch;
PDT_API pdt_status pdt_batch_create(pdt_batch** out);
PDT_API pdt_status pdt_batch_destroy(pdt_batch* b);
PDT_API pdt_status pdt_batch_add(pdt_batch* b, pdt_opt* opt);
PDT_API pdt_status pdt_batch_solve(pdt_batch* b, int verbose, void* stream);

/* ---- test hook (no counterpart in the reference) ------------------------------------------------- */
/* Every wait of the tensor-core kernels on an mbarrier is bounded (200 ms); a kernel that gives up
 * records an error word, waits (bounded) for its own copies and MMAs in flight, frees its tensor memory
 * and returns, and the next synchronous call raises PDT_ERR_TIMEOUT. With on != 0 those kernels
 * withhold one arrival (an operand barrier of the Cartesian tensor-core row passes; the first tile's
 * MMA commit of block 0 of a tensor-core convolution), so that tests can run the give-up path; 0
 * restores normal operation. Call it only while none of those kernels run. */
PDT_API pdt_status pdt_debug_drop_arrival(int on);

/* ---- allocation-free entry point ---------------------------------------------------------------- */
/* No counterpart in the reference. The Cartesian forward operator (MriCartesianOperator, or with
 * roos = 1 MriCartesianRemoveROOSOperator) for callers that cannot allocate device memory: code inside
 * another framework's memory pool or under a fixed device-memory budget, real-time loops that must not
 * enter the allocator, plugins whose host owns every allocation. All pointers are device pointers the
 * caller owns: sens {W,H,C} complex64, mask {W,H} float, img {W,H} or {W,H/2} (roos) complex64, kspace
 * {W,H,C} complex64 (every element is written). The scratch is a 32 MiB static device array (plus a
 * 64 KiB twiddle table) that every GPU loading libpdt.so holds until exit; C * W * image_rows * 8 bytes
 * must fit in it and W, H must be at most 4096, otherwise PDT_ERR_UNSUPPORTED. The first call on a
 * device resolves the array's address (cudaGetSymbolAddress), so make that first call before any stream
 * capture. Calls share the arrays: calls that overlap on the GPU race and must be serialised by the
 * caller. */
PDT_API pdt_status pdt_cartesian_forward_noalloc(int roos, const void* sens, const void* mask, int W, int H, int C,
                                                 const void* img, void* kspace, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PDT_H */
