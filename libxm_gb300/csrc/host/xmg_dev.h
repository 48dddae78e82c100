/*
 * Interface between the libxm-gb300 C host layer and its CUDA kernels.
 * Plain C types only; every function returns an XMG_* status code.
 */
#ifndef XMG_DEV_H
#define XMG_DEV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- runtime: device, stream, HBM arena ---------------------------- */
int xmgd_init(void);
int xmgd_alloc(size_t bytes, uint64_t *dptr);
int xmgd_free(uint64_t dptr);
int xmgd_h2d(uint64_t dst, const void *src, size_t bytes);
int xmgd_d2h(void *dst, uint64_t src, size_t bytes);
int xmgd_d2d(uint64_t dst, uint64_t src, size_t bytes);
int xmgd_sync(void);
int xmgd_is_device_ptr(const void *p);
/* Engine-owned grow-only device scratch, one buffer per slot. */
#define XMGD_SCRATCH_SLOTS 16
int xmgd_scratch(int slot, size_t bytes, uint64_t *dptr);
/* Pinned host staging buffer (grow-only). */
int xmgd_pinned(size_t bytes, void **hptr);
/* Page-locked host memory for host-allocator blocks (on the GPU's
 * nearest NUMA node where the system has several). */
int xmgd_host_alloc(size_t bytes, void **hptr);
void xmgd_host_free(void *p);
/* Asynchronous copies on the engine stream (xmgd_sync waits). */
int xmgd_h2d_async(uint64_t dst, const void *src, size_t bytes);
int xmgd_d2h_async(void *dst, uint64_t src, size_t bytes);
/* Out-of-core staging on the side stream: pinned chunk buffers in
 * XMGD_SIDE_SLOTS slots (two per reader thread); side_copy sends chunk
 * `slot` to dst asynchronously, side_fetch fills it from src, side_wait
 * blocks until that slot's last copy is done (the buffer may then be
 * reused), side_sync drains the side stream.  Distinct slots may be used
 * from distinct threads. */
#define XMGD_SIDE_SLOTS 32
int xmgd_bind_thread(void);
int xmgd_side_chunk(int slot, size_t bytes, void **hptr);
int xmgd_side_copy(int slot, uint64_t dst, size_t bytes);
int xmgd_side_fetch(int slot, uint64_t src, size_t bytes);
int xmgd_side_wait(int slot);
int xmgd_side_sync(void);
/* Copies between page-locked host memory and HBM on the side stream,
 * without a chunk slot (host-allocator blocks); xmgd_side_sync waits. */
int xmgd_side_put(uint64_t dst, const void *src, size_t bytes);
/* the device reads pageable host memory through the host's page tables
 * (then side_put also takes pageable sources, at the link's rate) */
int xmgd_pageable_direct(void);
int xmgd_side_get(void *dst, uint64_t src, size_t bytes);
size_t xmgd_arena_bytes_in_use(void);

/* ---- permuted element-wise ops over blocks -------------------------- */
enum {
	XMGD_OP_SET = 0,    /* dst = alpha                               */
	XMGD_OP_COPY,       /* dst = alpha * src   (with type conversion) */
	XMGD_OP_SCALE,      /* dst = alpha * dst                          */
	XMGD_OP_AXPY,       /* dst = alpha * dst + beta * src             */
	XMGD_OP_MUL,        /* dst = (alpha * dst) * src                  */
	XMGD_OP_DIV,        /* dst = dst / (alpha * src)                  */
	XMGD_OP_DOT,        /* partial[task] += dst * src  (no store)     */
};

/* One block-sized task.  The iteration space has ndim dimensions of the
 * given sizes; element (d_0..d_{n-1}) lives at dst + sum d_k*dst_stride[k]
 * and src + sum d_k*src_stride[k] (strides in elements).  Dimension 0 must
 * have dst_stride 1 for coalesced stores. */
typedef struct {
	uint64_t dst, src;
	int32_t ndim, op;
	int32_t size[8];
	int64_t dst_stride[8], src_stride[8];
	double alpha[2], beta[2];
} xmgd_ptask_t;

/* dtype/stype: xm_scalar_type_t values.  For XMGD_OP_DOT the per-task dot
 * products (complex: re, im) are written to dots[2*ntasks] (host). */
/* A batch uploaded once into a device buffer owned by the caller (release
 * with xmgd_free) and launched any number of times, also under stream
 * capture. */
typedef struct {
	uint64_t dbuf;               /* tasks + schedule metadata (xmgd_free) */
	int ntasks;
	int64_t begin[6];            /* CTA range of each schedule */
	int64_t slab_smem;           /* dynamic shared memory of the slab
	                                schedule's launch */
} xmgd_ptask_batch_t;
int xmgd_ptask_stage(const xmgd_ptask_t *tasks, int ntasks, int stype,
    xmgd_ptask_batch_t *b);
int xmgd_ptask_launch(int dtype, int stype, const xmgd_ptask_batch_t *b);
int xmgd_ptasks(int dtype, int stype, const xmgd_ptask_t *tasks, int ntasks,
    double *dots);

/* ---- block-sparse contraction -------------------------------------- */

/* One canonical output block.  Its m x n matrix view has element (i, j)
 * at c_ptr + crow[i] + ccol[j]; i runs over the output dimensions shared
 * with operand A, j over those shared with B. */
typedef struct {
	uint64_t c_ptr;
	int32_t m, n;
	int32_t crow, ccol;          /* offsets into the int32 table pool */
	int32_t first_pair, npairs;
	int32_t eA, eB;              /* exponent-table offsets (emulation) */
} xmgd_cblock_t;

/* One merged block pair: C += al * A^T B with A (k x m) and B (k x n),
 * A(k, i) at a_ptr + arow[k] + acol[i] and likewise for B. */
typedef struct {
	uint64_t a_ptr, b_ptr;
	int32_t k;
	int32_t arow, acol, brow, bcol;
	int32_t aview, bview;        /* operand-view ids (emulation) */
	int32_t esign, eshift;       /* pair factor = esign * 2^eshift when
	                                it is a signed power of two */
	double al[2];
} xmgd_pair_t;

/* A distinct unfolded operand (block data + permutation + masks). */
typedef struct {
	uint64_t ptr;
	int32_t k, mn;               /* rows (contracted), cols (free) */
	int32_t rowtab, coltab;      /* table-pool offsets */
	int32_t exptab;              /* exponent-table offset (per column) */
	int32_t n_rt, n_ks;          /* 128-row tiles, 16-wide K steps */
	int32_t kfast;               /* rows (K) unit-stride in memory */
	int32_t cplx;                /* complex elements: realified K */
	int32_t khp;                 /* complex: K per half, padded to 16 */
	int32_t kcontig;             /* rows (K) contiguous: row offset k is
	                                row offset 0 + k for every k */
	uint64_t slices;             /* device address of the tiled slices */
} xmgd_view_t;

typedef struct {
	int dtype;                   /* xm_scalar_type_t */
	int precision;               /* XMG_PREC_* */
	double alpha[2], beta[2];
	int ncblocks, npairs, nviews_a, nviews_b;
	const xmgd_cblock_t *cblocks;
	const xmgd_pair_t *pairs;
	xmgd_view_t *views_a, *views_b;
	const int32_t *tabs;         /* offset-table pool */
	int64_t ntabs;
	int32_t nexp_a, nexp_b;      /* exponent-table sizes */
	double flops;                /* useful flops (reference counting) */
	const uint8_t *emulatable;   /* per cblock: every pair factor +-2^t */
	int precision_used;          /* out: XMG_PREC_FP64 / XMG_PREC_EMU64 */
	int one_shot;                /* the plan runs once (an out-of-core
	                                batch): no graphs, no tuning runs */
	/* a's split-precision operands shared by the batches of a streamed
	 * contraction: 0 none; 1 this plan prepares them for all of a's views
	 * (exponent table a_E, slices in a_slices at a_off[v] for view v,
	 * Inf/NaN flag a_flag); 2 this plan uses them as prepared */
	int a_mode;
	uint64_t a_slices, a_E, a_flag;
	const int64_t *a_off;
} xmgd_contract_t;

/* bytes of one operand view's split-precision slices in a contraction of
 * scalar type dtype (0 when the type has no split-precision form) */
int64_t xmgd_emu_view_bytes(const xmgd_view_t *v, int dtype);

int xmgd_contract(xmgd_contract_t *plan);
/* the split-precision work list of one policy, built and checked on the
 * host: {items, members, stacked items, invariants hold} */
int xmgd_work_list_check(const xmgd_contract_t *p, int policy, long long out[4]);

/* Reusable device plan of one contraction: the uploaded metadata, operand
 * views and work lists, and the whole launch sequence captured once as a
 * CUDA graph.  Built from a host plan (whose arrays may be freed right
 * after), replayed by xmgd_plan_run. */
typedef struct xmgd_plan xmgd_plan_t;
int xmgd_plan_create(const xmgd_contract_t *p, xmgd_plan_t **out);
int xmgd_plan_run(xmgd_plan_t *dp, int *precision_used);
void xmgd_plan_free(xmgd_plan_t *dp);
/* 1 when the plan prepares a shared a side (a_mode 1 and a
 * split-precision part that took it) */
int xmgd_plan_a_shared(const xmgd_plan_t *dp);

/* Timing of the last xmgd_contract, milliseconds (device events). */
typedef struct {
	double ms_total, ms_split, ms_gemm;
	int64_t slice_bytes;
	int32_t gemm_launches, gemm_items;
	int32_t gemm_policy;         /* split-precision work list, -1: none */
} xmgd_timing_t;
void xmgd_last_timing(xmgd_timing_t *t);

#ifdef __cplusplus
}
#endif

#endif /* XMG_DEV_H */
