/*
 * libxm-gb300 extensions to the libxm C API.
 *
 * Everything declared in xm.h keeps the reference's behaviour (void return,
 * fatal exit on error).  This header adds what a GB300 engine needs beyond
 * that: status-code variants of the hot-path operations, the precision
 * mode, per-call statistics and the hand-written contraction adjoint.
 * Every function here is new; none replaces a reference symbol.
 */
#ifndef XMG_H_INCLUDED
#define XMG_H_INCLUDED

#include "tensor.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes returned by the xmg_* functions. */
#define XMG_OK        0
#define XMG_EINVAL    1   /* bad argument (indices, block structure, ...) */
#define XMG_ENOMEM    2   /* host or device allocation failed             */
#define XMG_ECUDA     3   /* CUDA runtime / kernel error                   */
#define XMG_EIO       4   /* pagefile read/write failed                    */
#define XMG_ETIMEOUT  5   /* a bounded device wait gave up                 */
#define XMG_ENOTSUP   6   /* combination not supported                     */

/* Message of the last failing xmg_* call on this thread. */
const char *xmg_last_error(void);

/* Precision of double / double complex contractions.
 *   XMG_PREC_FP64  - plain FP64 grouped GEMM on the FP64 pipe.
 *   XMG_PREC_EMU64 - split-precision emulated FP64: 6 signed 8-bit slices
 *                    per operand as bf16 on tcgen05 tensor cores, exact
 *                    FP32 partial sums drained into 64-bit integers, FP64
 *                    only for scaling and the alpha*AB + beta*C fold.
 *   XMG_PREC_AUTO  - EMU64 where it applies (power-of-two block-pair
 *                    factors), FP64 elsewhere.  Default.
 * float uses a compensated bf16 split in EMU modes and FP32 FMA in FP64
 * mode; complex types decompose into real products.  The environment
 * variable XMG_PRECISION=fp64|emu64|auto sets the initial mode. */
#define XMG_PREC_FP64  0
#define XMG_PREC_EMU64 1
#define XMG_PREC_AUTO  2
int xmg_set_precision(int mode);
int xmg_get_precision(void);

/* Status-code forms of the xm.h operations: same arguments and semantics,
 * but errors return XMG_* instead of exiting. */
int xmg_contract(xm_scalar_t alpha, const xm_tensor_t *a, const xm_tensor_t *b,
    xm_scalar_t beta, xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc);
int xmg_add(xm_scalar_t alpha, xm_tensor_t *a, xm_scalar_t beta,
    const xm_tensor_t *b, const char *idxa, const char *idxb);
int xmg_set(xm_tensor_t *a, xm_scalar_t x);

/* Useful (symmetry-reduced) flops of a contraction: 2*m*n*k summed over
 * every canonical output block and surviving merged block pair, times 4
 * for complex types.  Exactly the GEMM work the reference issues. */
double xmg_contract_flops(const xm_tensor_t *a, const xm_tensor_t *b,
    const xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc);

/* Merged block-pair structure of a contraction without running it:
 * cb(cblock, re, im, m, n, k) once per surviving pair, cblock being the
 * position in the canonical block list of c and (re, im) the pair factor
 * s_a * s_b after merging.  Needs no device. */
typedef void (*xmg_pair_cb)(size_t cblock, double re, double im, long m,
    long n, long k);
int xmg_contract_pairs(const xm_tensor_t *a, const xm_tensor_t *b,
    const xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc, xmg_pair_cb cb);

/* The split-precision GEMM's work list for one policy (0-2, 6), built and
 * checked on the host without a device: out = {items, members, items with
 * more than one member, 1 if every invariant the kernel relies on holds}.
 * For tests and tuning studies. */
int xmg_work_list_check(const xm_tensor_t *a, const xm_tensor_t *b,
    const xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc, int policy, long long out[4]);

/* The out-of-core batch plans, cut on the host without a device from the
 * whole plan, for b's blocks (in the streamed path's order: file order,
 * or the output blocks' with XMG_STREAM_ORDER=output) in the
 * streamed path's batches of at most `region` bytes, or, with region <= 0,
 * in nbatch equal runs: out = {batches, pairs over all batches, work-list
 * items of `policy` over all batches, 1 if every block lies aligned inside
 * its batch's region after the previous one, every pair of the whole plan
 * is in exactly one batch, in its order, with its views, the flops add up,
 * every batch's work list holds its invariants and no block of c is
 * written back before the last batch that feeds it}.  For tests. */
int xmg_batch_plan_check(const xm_tensor_t *a, const xm_tensor_t *b,
    const xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc, int nbatch, long long region, int policy,
    long long out[4]);

/* The copies the staging path makes for a list of n blocks (host address
 * h[i], bytes sz[i], device address dst[i]): one per run of blocks that
 * follow one another on both sides with only alignment padding between;
 * start[q] = the first block of run q (start holds n entries).  Returns
 * the number of runs.  For tests. */
size_t xmg_copy_runs(const uint64_t *h, const uint64_t *sz,
    const uint64_t *dst, size_t n, size_t *start);

/* The batches the streamed path cuts for b's distinct blocks of sizes
 * sz[0 .. n - 1], in that order: for a host-memory b (host != 0, the
 * XMG_HOST_* schedule) or a pagefile b beyond the staging budget
 * (XMG_STAGE_BATCHES equal batches), each at most `region` bytes with its
 * blocks 256-byte aligned; batch k holds blocks bstart[k] .. bstart[k + 1]
 * - 1 (bstart holds n + 1 entries).  Returns the number of batches, 0
 * when a block exceeds the region.  For tests. */
size_t xmg_stream_batches(const uint64_t *sz, size_t n, size_t region,
    int host, size_t *bstart);

/* Statistics of the last xm_contract / xmg_contract on this process. */
typedef struct {
	double flops;            /* useful flops (see xmg_contract_flops) */
	double ms_plan;          /* host planning, wall clock */
	double ms_device;        /* device time of the contraction */
	double ms_split;         /* of which: operand split / unfold kernels */
	double ms_gemm;          /* of which: grouped GEMM kernel(s) */
	long long n_cblocks;     /* canonical output blocks */
	long long n_pairs;       /* merged block pairs issued */
	long long slice_bytes;   /* bytes of staged operand slices */
	int precision_used;      /* XMG_PREC_FP64 or XMG_PREC_EMU64 */
	int gemm_launches;       /* kernels launched for the GEMM phase */
	long long stage_bytes;   /* out-of-core: b bytes streamed into HBM */
	int stage_batches;       /* out-of-core: batches (0: in-core) */
	int gemm_policy;         /* work-list policy of the split-precision
	                            GEMM (last batch), -1 if none ran */
	double ms_stage_wait;    /* out-of-core: host wait for staging beyond
	                            the overlapped compute, wall clock */
} xmg_stats_t;
int xmg_get_last_stats(xmg_stats_t *out);

/* Out-of-core contractions.  When the pagefile blocks of b that a
 * contraction reads exceed `budget` bytes, b is streamed through HBM in
 * about XMG_STAGE_BATCHES (default 8) equal batches of at most `region`
 * bytes: two device regions alternate, each batch is copied on a side
 * stream while the previous batch is contracted (c accumulates over the
 * batches; beta is applied once).  Where the device reads pageable host
 * memory through the host's page tables (a coherent CPU-GPU link) the
 * copies read the pagefile's blocks straight from a read-only mapping of
 * the file, else reader threads read them into pinned chunks first
 * (XMG_STAGE_MMAP=0 / 1 forces either).  a and c are staged whole; a's
 * split-precision operands are prepared once per call, by the first
 * batch, for all batches (XMG_STREAM_SHARE_A=0: in every batch).  Each
 * block of c goes back to the host as soon as the last batch that feeds
 * it has run, while later batches run (XMG_STREAM_CWRITE=0: all of c
 * after the last batch; with reader threads staging b, always after the
 * last batch).  b's blocks are batched in file order, or in the order of
 * the output blocks they feed with XMG_STREAM_ORDER=output (each batch
 * then feeds a range of c's blocks, which go back early).  Defaults: 180
 * GB and 32 GB, or XMG_STAGE_BUDGET_GB / XMG_STAGE_REGION_GB; 0 keeps the
 * current value. */
int xmg_set_staging(size_t budget, size_t region);

/* Hand-written adjoint of c = alpha * a * b over the index strings.  Given
 * dc (same structure as c), accumulates into the canonical blocks of da
 * and db (same structures as a and b):
 *     da += d<L>/d(canonical a),  db += d<L>/d(canonical b)
 * for L = sum over all blocks of dc o c (the xm_dot pairing), i.e. the
 * contractions dc*b and a*dc projected onto canonical blocks with every
 * derivative block's permutation and scalar folded back.  Either of da, db
 * may be NULL.  Every canonical block of a (b) must be canonical in da
 * (db).  When the block tables of a, b and dc are consistent with the
 * contraction (each derivative block's permutation and scalar carry the
 * contraction over, checked block by block), each gradient is one
 * contraction at the canonical positions times a per-block multiplicity;
 * otherwise it is computed at every nonzero position and folded back
 * (XMG_ADJOINT_EVERY=1 forces that form).  Returns XMG_* status. */
int xm_contract_adjoint(xm_scalar_t alpha, const xm_tensor_t *a,
    const xm_tensor_t *b, const xm_tensor_t *dc, xm_tensor_t *da,
    xm_tensor_t *db, const char *idxa, const char *idxb, const char *idxc);

/* Host-only: the structural checks of xm_contract_adjoint for these
 * tensors, without a device.  mode[0] (a's gradient) and mode[1] (b's):
 * 1 = canonical positions with per-block factors, 2 = every nonzero
 * position.  fa, fb (may be NULL): for the first form, the factor of each
 * block of a (b) in linear block order (index 0 fastest) as re, im pairs
 * (2 * number of blocks doubles; zero off the canonical blocks).  Releases
 * the adjoint's kept intermediates.  Returns XMG_* status. */
int xmg_adjoint_plan_check(const xm_tensor_t *a, const xm_tensor_t *b,
    const xm_tensor_t *dc, const char *idxa, const char *idxb,
    const char *idxc, int mode[2], double *fa, double *fb);

/* For tensors in GPU memory the adjoint keeps its intermediates (the
 * checks' outcome, W and the gradient tensors) and, through the plan
 * cache, the device plans of its two contractions while a, b and dc keep
 * their block structures, so that repeated calls neither plan nor
 * allocate.  This frees them (xmg_plan_cache_clear does too). */
void xmg_adjoint_release(void);

/* Allocation-free dot product.  No counterpart in the reference: it is an
 * addition for callers that cannot allocate memory at the point where they
 * need the value -- typically a host program whose own pool already holds
 * the GPU memory it may use (so any cudaMalloc would fail), or a solver
 * evaluating a norm every iteration of a tight loop, where the regular
 * xm_dot's first-use device allocations would stall it.  The value of
 * xm_dot(a, b, idxa, idxb), written to *result: the same block pairing and
 * factors, summed in another order (double types agree to rounding; float
 * types round each block's contribution and the running sum to float as
 * xm_dot does, and agree to float rounding).  The tensors must live in GPU
 * memory (allocator created with path NULL).  It calls no cudaMalloc,
 * cudaFree or host allocator: its task table, per-CTA partial sums and
 * running result live in one static device array of about 270 KiB that
 * the engine's GPU holds from the engine's initialisation (the first call
 * of this library that needs the GPU, which also looks up the array's
 * device address) until exit.  Limits: blocks of at most
 * XMG_NOALLOC_MAX_CTAS * XMG_NOALLOC_ELEMS_PER_CTA elements (larger ones
 * are rejected with XMG_EINVAL), tasks run in batches of
 * XMG_NOALLOC_MAX_TASKS.  Calls share the array: calls that overlap on
 * the GPU race.  Returns XMG_* status (XMG_EINVAL for NULL arguments). */
#define XMG_NOALLOC_MAX_TASKS      64
#define XMG_NOALLOC_MAX_CTAS       16384
#define XMG_NOALLOC_ELEMS_PER_CTA  2048
int xmg_dot_noalloc(const xm_tensor_t *a, const xm_tensor_t *b,
    const char *idxa, const char *idxb, xm_scalar_t *result);

/* Wait for all device work of the engine. */
int xmg_synchronize(void);

/* Free and total bytes of the engine's device (cudaMemGetInfo). */
int xmg_device_memory(size_t *free_bytes, size_t *total_bytes);

/* Opt-in tile-aware autosplit (no counterpart in the reference, whose
 * xm_block_space_autosplit is unchanged): every dimension is cut into about
 * dim / target parts, each a whole multiple of quantum (the last one also
 * takes the remainder below a quantum), so that the contraction's tiles
 * (N widths in multiples of 16, 128-row M tiles) carry less padding.
 * The block space must not be split yet. */
int xmg_block_space_autosplit_tiles(xm_block_space_t *bs, size_t target,
    size_t quantum);

/* Failure-detection self-test (no counterpart in the reference): one
 * thread block waits on a barrier that nothing arrives at, through the
 * bounded-wait path of the GEMM pipelines, gives up after timeout_us and
 * returns; the expected result is XMG_ETIMEOUT with the device still
 * usable.  Nothing faults or hangs. */
int xmg_selftest_bounded_wait(unsigned timeout_us);

/* xmg_contract keeps a device plan (metadata, work lists and a CUDA graph
 * of the launch sequence) for its most recent contractions over GPU-
 * resident tensors and replays it while the tensors' block tables are
 * unchanged; XMG_PLAN_CACHE=<n> sets the number kept (0 disables, at most
 * 16).  This frees every cached plan. */
void xmg_plan_cache_clear(void);

/* Device-time measurement on the engine's stream: start records an event,
 * stop records another, waits for it and returns the elapsed milliseconds
 * (negative on error). */
int xmg_timer_start(void);
double xmg_timer_stop(void);

/* Number of engine kernels launched since the library was loaded. */
long long xmg_kernel_launches(void);

/* Page-locked host buffers for fast block transfers (NULL on failure). */
void *xmg_host_alloc(size_t bytes);
void xmg_host_free(void *p);

/* An allocator whose blocks live in page-locked host memory, the
 * counterpart of the reference's RAM allocator (xm_allocator_create(NULL)
 * in the reference, alloc.c:233-239; here that call gives GPU memory).
 * Handles are host addresses; xm_allocator_read/write and the block
 * read/write calls are plain memory copies.  xm_contract streams the
 * operands of such tensors through HBM on every call: a's blocks (and c's
 * when beta != 0) and b's first batch are copied in, then each further
 * batch of b is copied on a side stream while the previous batch is
 * contracted, and c is copied back before the call returns (block by
 * block once final, as for the pagefile).  The batches
 * (about XMG_HOST_BATCHES of them, default 8, at most the staging region
 * each) grow by a factor XMG_HOST_GROWTH (default 1.45) from one to the
 * next up to the middle and shrink again toward the end
 * (XMG_HOST_SHAPE=geometric: grow to the end), so that the first copy,
 * which nothing overlaps, and the last batch's kernels, which nothing
 * overlaps where the host link is the slower side, are short.  The
 * streamed plan of the last such contraction (batches, HBM regions, the
 * device plans and their graphs) is kept while the tensors' block
 * structures and the call's arguments stay the same (XMG_STREAM_CACHE=0
 * disables that; xmg_plan_cache_clear releases it).  Element-wise
 * operations stage the blocks they touch.  NULL if the engine cannot
 * start. */
xm_allocator_t *xmg_allocator_create_host(void);

/* Write (read) n blocks in one call: blks[i] from (into) the host buffer
 * bufs[i], of xm_tensor_get_block_bytes bytes each.  For tensors in GPU
 * memory the copies are queued back to back (one cudaMemcpyAsync per
 * block) and waited for once; buffers may be reused on return, as after
 * xm_tensor_write_block.  Same rules as the one-block calls (canonical
 * blocks only for writes, no zero blocks for reads), reported as
 * XMG_EINVAL before any data moves.  Returns XMG_* status. */
int xmg_tensor_write_blocks(xm_tensor_t *t, size_t n, const xm_dim_t *blks,
    const void *const *bufs);
int xmg_tensor_read_blocks(const xm_tensor_t *t, size_t n,
    const xm_dim_t *blks, void *const *bufs);

/* The engine runs on device ordinal $XMG_DEVICE (default 0), chosen at
 * the first call that needs the GPU. */

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* XMG_H_INCLUDED */
