/*
 * hsmu_gb.h -- C ABI of the GB300 (sm_103a) HSMU SpGEMM engine, C = A * B.
 *
 * CSR in, CSR out: int32 row pointers and column indices, FP64 values,
 * zero-based, columns strictly increasing within each row.  All matrix
 * arrays passed to the compute entry points live in device memory of the
 * current CUDA device.  No torch or CUDA types appear in the signatures:
 * streams are passed as `void *` (a cudaStream_t, NULL = legacy default).
 *
 * Every function returns an hsmu_status (0 = success); no C++ exception
 * crosses this boundary.  The C++ compatibility layer in hsmu_nhc_compat.h
 * maps non-zero codes to std::exception as the reference's CHECK_ERROR does.
 *
 * Reference interfaces replaced (paths relative to the HSMU-SpGEMM project):
 *   hsmu_spgemm          <- void NHC_spgemm(compressed_bin*, NHC_bin*, NHC_CSR *A,
 *                           NHC_CSR *B, NHC_CSR *C, NHC_mask_matrix*)
 *                           src/NHC_spgemm.cuh:7, whose compressed branch is
 *                           compressed_NHC_spgemm, src/compressed/compressed_NHC_spgemm.cu:22
 *   hsmu_handle_create   <- setup(), src/loading.cuh:51-84 (streams, scratch, scan storage)
 *   hsmu_handle_destroy  <- realse_compressed_bin / free_bin, src/loading.cuh:106-130,166-173
 *   hsmu_csr_free        <- free_C_matrix, src/loading.cuh:151-165
 *   hsmu_btiles_build    <- Initialize_compressed_mask64_matrix,
 *                           src/compressed/compressed_mask64.cuh:343-424
 *   hsmu_btiles_free     <- realse_NHC_tile, src/loading.cuh:95-105
 *   hsmu_strerror        <- (none: the reference prints and throws, inc/cuda_comm.h:16-29)
 */
#ifndef HSMU_GB_H
#define HSMU_GB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HSMU_ABI_VERSION 1

typedef enum hsmu_status {
    HSMU_OK = 0,
    HSMU_ERR_INVALID = 1,      /* bad argument, shape mismatch, NULL pointer */
    HSMU_ERR_ALLOC = 2,        /* device or host allocation failed */
    HSMU_ERR_CUDA = 3,         /* a CUDA runtime call or kernel launch failed */
    HSMU_ERR_OVERFLOW = 4,     /* nnz(C) or a scratch size does not fit int32 */
    HSMU_ERR_UNSORTED = 5,     /* validation: columns not strictly increasing / out of range */
    HSMU_ERR_INTERNAL = 6,     /* a device-side consistency check failed */
    HSMU_ERR_TIMEOUT = 7,      /* a bounded device-side wait gave up */
    HSMU_ERR_NO_DEVICE = 8,    /* no usable sm_103 device */
    HSMU_ERR_UNSUPPORTED = 9,  /* kept for ABI stability; no call returns it */
    HSMU_ERR_CAPACITY = 10     /* hsmu_spgemm_host: output buffers too small (C->nnz = needed size) */
} hsmu_status;

/* CSR matrix descriptor.  row_ptr has M+1 entries, col/val have nnz entries.
 * `owned` = 1 when the arrays were allocated by this library (output of
 * hsmu_spgemm); hsmu_csr_free releases exactly those. */
typedef struct hsmu_csr {
    int32_t M;
    int32_t N;
    int32_t nnz;
    int32_t owned;
    int32_t *row_ptr;
    int32_t *col;
    double *val;
} hsmu_csr;

/* B converted to 64-column bit tiles (the reference's compressed mask64
 * format, one u64 per non-empty 64-column tile of a row):
 *   tile_ptr[M+1]  tiles of row k are tile_ptr[k] .. tile_ptr[k+1]-1
 *   tile_col[T]    tile index (column >> 6), strictly increasing per row
 *   mask[T]        bit b set  <=> column tile_col*64 + b is present
 *   tile_off[T]    CSR offset of the tile's first entry in B
 * The same tiles may be reused for every product with the same B. */
typedef struct hsmu_btiles {
    int32_t M;
    int32_t N;
    int32_t ntiles;
    int32_t reserved;
    int32_t *tile_ptr;
    int32_t *tile_col;
    uint64_t *mask;
    int32_t *tile_off;
} hsmu_btiles;

/* Options; a NULL pointer means all defaults (zero-initialise to get them). */
#define HSMU_ARITH_RN 0
#define HSMU_ARITH_FMA 1
#define HSMU_ARITH_IMUL 2
typedef struct hsmu_opts {
    int32_t validate;     /* 1: check A and B are canonical CSR before computing */
    int32_t arith;        /* how each product is accumulated, c <- c + a*b:
                           * HSMU_ARITH_RN (0, default): product rounded, then added -- the
                           *   reference's arithmetic (atomicAdd(.., aval * bval),
                           *   src/compressed/compressed_Cval.cuh:60-61);
                           * HSMU_ARITH_FMA (1): one fused multiply-add per product (one
                           *   rounding instead of two, half the FP64 instructions);
                           * HSMU_ARITH_IMUL (2): as RN, with the product formed exactly on the
                           *   integer pipe.
                           * In every mode products are added in A-row order, so results are
                           * deterministic; RN and IMUL give identical bits. */
    int32_t window_cap;   /* 0: default slots per numeric window (<= 4096) */
    int32_t panels;       /* hsmu_spgemm_host: row panels of the copy pipeline (0: one per 32 MB
                           * of output; at most 8).  Sizes shrink from the first panel when the
                           * compute takes longer than the copy back; when the copy is the longer
                           * part they double from the first panel to the middle and halve
                           * towards the last.  The panels run in the order that keeps the host
                           * link busy soonest (the least compute first) */
    int32_t wait_polls;   /* test hook, 0 in normal use.  > 0: every bounded device wait of the call
                           * gives up after this many polls instead of its default limit (the value
                           * pass's wait for a window's column copy polls without blocking; the batch's
                           * grid barriers spin this many times) and the call reports
                           * HSMU_ERR_TIMEOUT.  A wait that gives up still lets its own copy land
                           * before the kernel returns; the handle stays usable.  For hsmu_batch_create
                           * it applies to every launch of the batch. */
    int32_t no_tile_store; /* 1: the count pass keeps no C tiles of the large rows, and the structure
                           * pass repeats their OR walk over B's tiles (same output; less scratch) */
    int32_t learned_always; /* test hook, 0 in normal use.  1: hsmu_spgemm_learned never hands the
                           * product to the plain path (it uses its prediction whatever the rows) */
    int32_t reserved;
} hsmu_opts;

/* Per-call statistics (filled by hsmu_spgemm when stats != NULL). */
typedef struct hsmu_stats {
    uint64_t products;       /* intermediate products sum nnz(B(k,:)) over A entries */
    int64_t nnz_c;
    int64_t ntiles_b;
    int64_t windows;         /* numeric work items */
    float ms_convert;        /* B -> tiles */
    float ms_symbolic;       /* bounds, binning, exact count, scan */
    float ms_alloc;          /* output allocation (includes the one host read of nnz) */
    float ms_structure;      /* column emission */
    float ms_numeric;        /* value accumulation */
    float ms_total;
    int32_t launches;        /* kernels this call launched */
    int32_t routed;          /* learned path: 1 when it handed the product to the plain path */
    int64_t spec_capacity;   /* learned path: entries of the speculative slots */
    int64_t fallback_rows;   /* learned path: rows that exceeded their slot and were redone */
} hsmu_stats;

typedef struct hsmu_handle_s *hsmu_handle;

const char *hsmu_strerror(int status);
int hsmu_abi_version(void);

/* Library context for the current device: scratch pool, events, cached
 * device properties.  One handle per host thread (not reentrant). */
int hsmu_handle_create(hsmu_handle *out);
int hsmu_handle_destroy(hsmu_handle h);

/* C = A * B.  A, B: device CSR (A->N == B->M).  On success C->M = A->M,
 * C->N = B->N, C->nnz is set and C->row_ptr/col/val are new device arrays
 * owned by the library (free with hsmu_csr_free).  Columns of every C row
 * are sorted ascending; entries whose products cancel to 0.0 are kept.
 * Values: each product a_ik*b_kj is rounded to double, then added to the
 * entry in the order of A(i,:)'s storage (bit-identical run to run).
 * Stream-ordered on `stream`; returns after one host read of nnz(C) and
 * leaves the remaining kernels queued on `stream`. */
int hsmu_spgemm(hsmu_handle h, const hsmu_csr *A, const hsmu_csr *B, hsmu_csr *C,
                const hsmu_opts *opts, void *stream, hsmu_stats *stats);

/* Same, with B already converted by hsmu_btiles_build (B tiles reused). */
int hsmu_spgemm_tiled(hsmu_handle h, const hsmu_csr *A, const hsmu_csr *B,
                      const hsmu_btiles *Bt, hsmu_csr *C, const hsmu_opts *opts,
                      void *stream, hsmu_stats *stats);

/* C = A * B with A, B and C in HOST memory: the whole sequence a reference
 * caller runs around NHC_spgemm -- HtD_value_col_ptr(&A), HtD_value_col_ptr(&B)
 * (src/test.cu:67-68, src/loading.cuh:86-94), NHC_spgemm (src/test.cu:71)
 * and the copy of C back to the host -- as one pipelined call.  The index
 * arrays go up first and the symbolic pass starts on them while the values
 * are copied on a second stream; C is then computed in row panels and each
 * finished panel is copied back on a third stream while the next one is
 * computed.  Results are identical to hsmu_spgemm + hsmu_csr_download.
 *   A, B: host arrays; when A and B are the same arrays they are copied once.
 *   C:    in:  row_ptr (A->M + 1 entries), col and val of capacity C->nnz;
 *         out: M, N, nnz, and the three arrays filled; owned = 0.
 * HSMU_ERR_CAPACITY: C->nnz < nnz(C); C->nnz and C->row_ptr then hold the
 * product's, col/val are untouched -- call again with larger arrays.
 * Host arrays must be page-locked (cudaHostAlloc / cudaHostRegister) for the
 * copies to overlap; pageable memory gives the same result, serialised.
 * Blocks until C is in host memory.  In stats, ms_structure covers the panels'
 * kernels (with the copies they hide) and ms_numeric the last copies. */
int hsmu_spgemm_host(hsmu_handle h, const hsmu_csr *A, const hsmu_csr *B, hsmu_csr *C,
                     const hsmu_opts *opts, void *stream, hsmu_stats *stats);

int hsmu_btiles_build(hsmu_handle h, const hsmu_csr *B, hsmu_btiles *out, void *stream);

/* CSR with 64-bit row pointers, for products with more than INT32_MAX
 * entries.  The reference's index type is int throughout (index_t,
 * inc/NHC_spgemm.h:13; NHC_CSR::nnz, :77), which caps C at 2^31 - 1 entries
 * (hsmu_spgemm reports such products with HSMU_ERR_OVERFLOW). */
typedef struct hsmu_csr64 {
    int32_t M;
    int32_t N;
    int64_t nnz;
    int32_t owned;
    int32_t reserved;
    int64_t *row_ptr; /* [M+1] */
    int32_t *col;     /* [nnz] */
    double *val;      /* [nnz] */
} hsmu_csr64;

/* C = A * B on the device with C in hsmu_csr64 form (row pointers int64,
 * library-owned: free with hsmu_csr64_free).  Same results as hsmu_spgemm.
 * The exact nnz of every row comes first; the rows of A are then processed
 * in panels whose entries fit int32 (at most max_panel_nnz each, 0 = INT32_MAX;
 * a row with more entries than the cap is a panel of its own), each written
 * straight into its place in C.  B's tiles are built once for all panels.
 * Synchronizes `stream` before returning. */
int hsmu_spgemm64(hsmu_handle h, const hsmu_csr *A, const hsmu_csr *B, hsmu_csr64 *C, int64_t max_panel_nnz,
                  const hsmu_opts *opts, void *stream);
int hsmu_csr64_free(hsmu_csr64 *C);
/* hsmu_csr_download for an hsmu_csr64 (row_ptr[M+1] int64, col/val[nnz]) */
int hsmu_csr64_download(const hsmu_csr64 *C, int64_t *row_ptr, int32_t *col, double *val, void *stream);

/* At = A^T on the device, every row of At in ascending column order (a stable
 * radix sort of A's entries by column).  At is owned by the library
 * (hsmu_csr_free).  A must be canonical CSR.  Replaces the host transpose the
 * reference runs before an A*A^T product: csr2csc, src/mmio_highlevel.h:194,
 * called from src/test.cu:40-56. */
int hsmu_csr_transpose(hsmu_handle h, const hsmu_csr *A, hsmu_csr *At, void *stream);
int hsmu_btiles_free(hsmu_btiles *t);

/* B -> 64-column bit tiles into caller-owned arrays, allocating nothing.
 * No counterpart in the reference (its conversion always allocates).  For
 * callers that cannot allocate device memory -- their memory is owned by
 * their own pool or a fixed budget that forbids cudaMalloc/cudaFree on the
 * compute path.  The caller passes B (device CSR) and the outputs:
 * tile_ptr[B->M + 1] and tile_col/mask/tile_off with room for B->nnz
 * entries (the tile count is tile_ptr[B->M] afterwards, at most B->nnz).
 * The scan's scratch is a static ~64 KB device array inside the library,
 * which limits B to 2^24 rows (larger B -> HSMU_ERR_OVERFLOW).  The first
 * call on each device looks up that array's address (make it before any
 * stream capture).  Calls share the array: calls that overlap on the GPU
 * race, so serialise them.  Checks B's columns (HSMU_ERR_UNSORTED) and
 * synchronizes `stream` before returning.  No handle needed. */
int hsmu_btiles_build_noalloc(const hsmu_csr *B, int32_t *tile_ptr, int32_t *tile_col, uint64_t *mask,
                              int32_t *tile_off, void *stream);

/* Releases the arrays of a library-owned CSR (owned == 1) and zeroes it. */
int hsmu_csr_free(hsmu_csr *C);

/* Copies a device CSR into caller-provided host buffers (pinned or pageable):
 * row_ptr[M+1], col[nnz], val[nnz].  Stream-ordered; synchronizes `stream`
 * before returning. */
int hsmu_csr_download(const hsmu_csr *C, int32_t *row_ptr, int32_t *col, double *val, void *stream);

/* ---- Learned row scheduler ----------------------------------------------
 * hsmu_spgemm_learned computes the same C as hsmu_spgemm (bit for bit) but
 * replaces the exact symbolic count pass with a prediction: a 3-layer FP32
 * MLP (4 -> 32 -> 32 -> 1) maps each row's features (log2(1+x) of A-row nnz,
 * intermediate products, longest referenced B row, column span) to log2 of
 * its nnz; each row gets a slot of min(products, N, 2^(prediction + margin))
 * entries, the structure pass writes into the slot and finds the exact count,
 * rows that overflow are redone after the scan.  params: HSMU_MLP_FLOATS
 * device floats (W1[32][4] b1[32] W2[32][32] b2[32] W3[32] b3, then mu[4]
 * sd[4] ymu ysd).  No counterpart in the reference.
 * hsmu_row_features / hsmu_row_nnz produce training data (features, and
 * labels from the engine's own exact symbolic pass); hsmu_mlp_forward /
 * hsmu_mlp_grad / hsmu_mlp_adam are the inference and training kernels
 * (grad adds to `grad` and `loss`; adam applies grad * scale). */
#define HSMU_MLP_FLOATS 1259
typedef struct hsmu_mlp {
    const float *params;
    float margin;
    int32_t reserved;
} hsmu_mlp;
int hsmu_spgemm_learned(hsmu_handle h, const hsmu_csr *A, const hsmu_csr *B, hsmu_csr *C, const hsmu_mlp *model,
                        const hsmu_opts *opts, void *stream, hsmu_stats *stats);
int hsmu_row_features(hsmu_handle h, const hsmu_csr *A, const hsmu_csr *B, float *feat, int64_t *products,
                      void *stream);
int hsmu_row_nnz(hsmu_handle h, const hsmu_csr *A, const hsmu_csr *B, int32_t *nnz, void *stream);
int hsmu_mlp_forward(const float *params, const float *feat, int n, float *out, void *stream);
int hsmu_mlp_grad(const float *params, const float *feat, const float *target, int n, float *grad, float *loss,
                  void *stream);
int hsmu_mlp_adam(float *params, const float *grad, float *m, float *v, float lr, float scale, int step,
                  void *stream);

/* ---- Batched persistent engine ------------------------------------------
 * Many independent products in ONE cooperative persistent launch, with no
 * host synchronisation inside and outputs in one preallocated pool:
 *   HSMU_BATCH_PRODUCT : C_p = A[p] * B[p]
 *   HSMU_BATCH_GALERKIN: C_p = Pt[p] * (A[p] * B[p])   (B = prolongator P, Pt = P^T)
 * No counterpart in the reference, which runs products one by one
 * (src/NHC_spgemm.cuh:7 per product).  hsmu_batch_create sizes the pool with
 * one device pass and one host read; execute / graph_launch only enqueue
 * work (graph_launch captures the launch in a CUDA graph on first use and
 * replays it).  Results (hsmu_batch_result) are descriptors into the pool
 * (owned = 0) valid until hsmu_batch_destroy.  Rows of any width are taken:
 * rows of more than 512 entries or a column span of more than 512 64-column
 * tiles are written one column window at a time by a wide-row phase of the
 * same launch.  A product whose entries exceed INT32_MAX reports
 * HSMU_ERR_OVERFLOW. */
#define HSMU_BATCH_PRODUCT 0
#define HSMU_BATCH_GALERKIN 1
typedef struct hsmu_batch_s *hsmu_batch;
int hsmu_batch_create(hsmu_handle h, int kind, int n, const hsmu_csr *A, const hsmu_csr *B, const hsmu_csr *Pt,
                      const hsmu_opts *opts, hsmu_batch *out, void *stream);
int hsmu_batch_execute(hsmu_batch b, void *stream);
int hsmu_batch_graph_launch(hsmu_batch b, void *stream);
/* synchronizes `stream`; maps the device-side error bits to a status */
int hsmu_batch_status(hsmu_batch b, void *stream);
int hsmu_batch_result(hsmu_batch b, int p, hsmu_csr *C);
/* tiny: products threshold of the thread-per-row class (0..32); grid: blocks (0 = keep) */
int hsmu_batch_set_params(hsmu_batch b, int tiny, int grid);
/* times the parameter candidates on this batch and keeps the fastest */
int hsmu_batch_autotune(hsmu_batch b, void *stream, int *best_tiny, int *best_grid, float *best_ms);
int hsmu_batch_destroy(hsmu_batch b);

/* ---- Synthetic AMG operators generated on the device (workload inputs) ---
 * 7-point Poisson matrix of a side^3 grid (6 on the diagonal, -1 off it, natural
 * ordering) and the piecewise-constant 2x2x2 aggregation prolongator P (fine x
 * ceil(side/2)^3, weight 1) with its transpose.  Outputs are library-owned
 * (free with hsmu_csr_free).  No counterpart in the reference. */
int hsmu_gen_poisson7(int side, hsmu_csr *A, void *stream);
int hsmu_gen_aggregation(int side, hsmu_csr *P, hsmu_csr *Pt, void *stream);

/* Diagnostic: checks the numeric phase's integer-pipe FP64 multiply against
 * the FP64 pipe's multiply on n generated operand pairs (all bit patterns,
 * values in (-1,1), short significands with frequent ties) and stores the
 * number of results that differ in any bit (expected 0).  No reference
 * counterpart: the reference multiplies on the FP64 pipe only. */
int hsmu_selftest_dmul(uint64_t n, uint64_t seed, uint64_t *mismatches, void *stream);

/* Measures the device's FP64 pipe: every thread of a full grid runs
 * independent chains of rounded multiplies and adds (the two operations a
 * product costs in the value pass) for `iters` steps; stores FP64 lane
 * operations per second (timed with CUDA events on `stream`).  The
 * denominator of the value pass's FP64 roofline.  No reference counterpart. */
int hsmu_probe_fp64_rate(int iters, double *lane_ops_per_s, void *stream);

/* Test hook for the failure paths: the nth device allocation the library makes
 * from now on (1 = the next one, counted across all calls and threads) fails
 * as if the device were out of memory, so the call that makes it returns
 * HSMU_ERR_ALLOC after releasing what it holds.  0 disarms the hook.
 * No reference counterpart (the reference throws on a failed cudaMalloc,
 * inc/cuda_comm.h:16-29). */
int hsmu_debug_fail_alloc(int64_t nth);

/* Test hook: the row panels hsmu_spgemm_host would use for a product with C's
 * row pointers row_ptr (M + 1 entries), `products` intermediate products,
 * chunk_products[c] = the products of rows 64c .. 64c+63 (ceil(M / 64)
 * entries; NULL: the panels run in row order) and hsmu_opts.panels = panels.
 * Writes the number of panels np (at most 8) to *n_panels, their row bounds
 * to cut[0..np] (panel q = rows cut[q] .. cut[q+1]-1) and the order they run
 * in to order[0..np-1]; cut needs 9 entries, order 8.  Host-only: no device
 * call.  No reference counterpart (the reference computes C whole in one
 * NHC_spgemm call, src/test.cu:71). */
int hsmu_debug_plan_panels(int32_t M, const int32_t *row_ptr, int64_t products, const int64_t *chunk_products,
                           int32_t panels, int32_t *n_panels, int32_t *cut, int32_t *order);

#ifdef __cplusplus
}
#endif
#endif /* HSMU_GB_H */
