// Batched persistent engine: many independent SpGEMMs (C_p = A_p * B_p) or
// AMG Galerkin triple products (C_p = Pt_p * (A_p * P_p)) in ONE launch.
//
// The reference runs each product separately, with ~10 blocking host round
// trips and several cudaMalloc calls per product
// (src/compressed/compressed_NHC_spgemm.cu:22-248); for hundreds of small
// products that overhead, not the arithmetic, sets the time.  Here all rows of
// all products form one flattened row space, cut into tiles of 32 rows that
// never span two products, and a single cooperative, persistent kernel takes
// every row in ONE pass:
//   * a warp computes its tile's rows (thread per row with a sorted list in
//     shared memory; warp per row with a dense tile table for rows with more
//     products), so the tile's entry count is known;
//   * one atomic on the product's allocation counter gives the tile a
//     contiguous block of the product's region of the output pool (regions
//     sized by the products' nnz bounds when the batch is made), and the rows
//     are written there, compact, with no count pass and no wait on any other
//     tile.
// The intermediate A*P of a Galerkin product is read in that form (every row
// has a start and an end); the second product (Pt * (AP)) runs the same way
// after one grid barrier.  The last product is put in row order at the end:
// a device-wide scan of the tile counts gives every tile its place in its
// product, and each tile is copied there as one block with its row pointers.
// No host synchronisation happens inside; the launch is captured once in a
// CUDA graph and replayed.
//
// Wide rows (more than B_FUSE_CAP entries, or a column span of more than
// SPAN_T tiles) are counted by their tile's warp one column window at a time
// and listed; after the tiles, a wide-row phase of the same launch gives each
// listed row to a warp, which writes it window by window (windows of whole
// tiles with fewer than B_FUSE_CAP entries).
//
// Grid barriers spin on a generation counter with an iteration limit: a
// barrier that gives up sets an error bit (HSMU_ERR_TIMEOUT) and every block
// returns, so a fault in one block can never hang the GPU.
//
// Tuning: the thread-per-row product limit (`tiny`) and the grid size are
// parameters of the launch; hsmu_batch_autotune times the candidates on the
// actual batch and keeps the fastest.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <new>
#include <vector>

#include "hsmu_gb.h"
#include "hsmu_kernels.h"
#include "hsmu_rowops.cuh"

namespace hsmu {

constexpr int B_FUSE_CAP = 512;           // entries of a row (or a column window) written from one table
constexpr int SUB_NNZ = B_FUSE_CAP - 64;  // window cut: tiles whose first entry lies in one block of SUB_NNZ
constexpr int TILE_ROWS = WARP;           // rows per tile (one warp)
constexpr int WIDE_LIST = 1 << 16;        // listed wide rows per round (more are written in place)
constexpr unsigned long long SPIN_LIMIT = 1ull << 25;
enum BatchErr : int { BERR_TIMEOUT = 16, BERR_CAPACITY = 64, BERR_INTERNAL = 128 };

struct BOp {  // one CSR operand on the device; row k is rp[k] .. re[k]-1
    int M, N;
    const int *rp;
    const int *re;
    const int *col;
    const double *val;
};

// A round: one product of every entry of the batch (one round for plain products;
// two for Galerkin entries, A*P and then Pt*(AP)).
struct BRound {
    int nprod;
    const BOp *A;            // left operand per product
    const BOp *B;            // right operand per product (unused when b_from_prev)
    int b_from_prev;         // B_p = C_p of the previous round
    int last;                // the round whose output is returned (put in row order)
    const long long *row0;   // [nprod+1] flattened row offsets
    const long long *rpo;    // [nprod+1] offsets of each product's row pointers in rp_pool / rs / re
    const long long *tile0;  // [nprod+1] offsets of each product's tiles
    const long long *reg;    // [nprod+1] each product's region of the pools
    long long R, T;          // rows, tiles
    unsigned long long *alloc;  // [nprod] entries handed out in each region (zeroed before every launch)
    int *nwide;              // wide rows listed (zeroed before every launch)
    long long *wide;         // [2*WIDE_LIST] (flattened row, pool offset) of listed wide rows
    int *col_pool;           // [reg[nprod]] rows as the tiles wrote them
    double *val_pool;
    // intermediate rounds: every row's start and end in its region
    int *rs, *re;            // [rpo[nprod]]
    // the last round: tile counts and places, then the output in row order
    int *tbase, *tcnt;       // [T] a tile's block in its region, its entry count
    long long *tex;          // [T+1] exclusive scan of tcnt over all tiles of the round
    int *rp_pool;            // [rpo[nprod]] row pointers, 0-based within the product (row counts before)
    int *out_col;            // [reg[nprod]]
    double *out_val;
};

struct GridBar {
    unsigned count;
    unsigned gen;
};

struct BParams {
    BRound rnd[2];
    int nrounds;
    int tiny;              // products limit of the thread-per-row path
    long long *bsum;       // [gridDim.x + 1] block sums of the tile-count scan
    GridBar *bar;
    int *err;
    int arith;             // hsmu_opts.arith of the batch
    unsigned long long spin_limit;  // polls of a grid barrier before it gives up
};

// grid-wide barrier; false (every block returns) when a wait gave up or any
// error bit is set, so no later phase reads what an unfinished phase left
__device__ bool grid_sync(GridBar *gb, int *err, unsigned long long spin_limit) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        volatile unsigned *vgen = &gb->gen;
        const unsigned g = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(&gb->count, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(&gb->count, 0u);
            __threadfence();
            atomicAdd(&gb->gen, 1u);
        } else {
            unsigned long long it = 0;
            while (*vgen == g) {
                if (++it > spin_limit) {
                    atomicOr(err, BERR_TIMEOUT);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        if (*(volatile int *)err) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// product owning flattened index i of an ascending offset array (off[lo] <= i < off[lo+1])
__device__ __forceinline__ int find_prod(const long long *off, int n, long long i) {
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= i) lo = mid; else hi = mid;
    }
    return lo;
}

// the B operand of product p in round r (C of the previous round for Galerkin)
__device__ __forceinline__ BOp b_operand(const BParams &P, int r, int p) {
    const BRound &R = P.rnd[r];
    if (!R.b_from_prev) return R.B[p];
    const BRound &Q = P.rnd[r - 1];
    const long long base = __ldg(Q.reg + p), ro = __ldg(Q.rpo + p);
    BOp b;
    b.M = (int)(__ldg(Q.row0 + p + 1) - __ldg(Q.row0 + p));
    b.N = -1;  // not needed by the row routines
    b.rp = Q.rs + ro;
    b.re = Q.re + ro;
    b.col = Q.col_pool + base;
    b.val = Q.val_pool + base;
    return b;
}

constexpr int BW = 8;  // warps per block (launch uses BW*32 threads)

struct BWarpSmem {
    union {
        struct {
            unsigned long long msk[SPAN_T];
            int base[SPAN_T];
            double acc[B_FUSE_CAP];
        } w;
        struct {
            int cols[TINY_MAX * WARP];
            double acc[TINY_MAX * WARP];
        } t;
    };
};

// exclusive prefix of the masks' popcounts into base[0..span); returns the total
__device__ __forceinline__ int mask_prefix(const unsigned long long *msk, int span, int *base) {
    const int lane = lane_id();
    const int per = (span + WARP - 1) / WARP;
    const int lo = min(span, lane * per), hi = min(span, lo + per);
    int sum = 0;
    for (int t = lo; t < hi; t++) sum += popc64(msk[t]);
    const int incl = warp_incl_scan(sum);
    int run = incl - sum;
    for (int t = lo; t < hi; t++) {
        base[t] = run;
        run += popc64(msk[t]);
    }
    __syncwarp();
    return __shfl_sync(FULL, incl, WARP - 1);
}

// first index in [lo, hi) with base[idx] >= key (base ascending, shared memory)
__device__ __forceinline__ int smem_lower_bound(const int *base, int lo, int hi, int key) {
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (base[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Entry count of a row that fails the thread path (warp-wide).  Rows of span
// <= SPAN_T tiles take one pass over their products; wider ones one pass per
// SPAN_T-tile column window.  `wide` is set for rows that the warp-row fill
// cannot write in one table (more than B_FUSE_CAP entries or a wide span).
template <bool NC>
__device__ int big_row_count(int a_lo, int a_hi, const BOp &A, const BOp &B, BWarpSmem &S, bool &wide, bool &bad) {
    int cmin, cmax, prod;
    warp_row_extent<NC>(a_lo, a_hi, A.col, B.rp, B.re, B.col, cmin, cmax, prod);
    wide = false;
    if (cmax < 0) return 0;
    const int t_lo = cmin >> 6, t_hi = cmax >> 6;
    if (t_hi - t_lo < SPAN_T) {
        const int span = t_hi - t_lo + 1;
        if (!warp_row_masks<NC>(a_lo, a_hi, A.col, B.rp, B.re, B.col, t_lo, span, S.w.msk)) bad = true;
        const int c = warp_mask_count(S.w.msk, span);
        __syncwarp();
        wide = c > B_FUSE_CAP;
        return c;
    }
    wide = true;
    long long c = 0;
    for (int c0 = t_lo; c0 <= t_hi; c0 += SPAN_T) {
        const int span = min(SPAN_T, t_hi - c0 + 1);
        if (!warp_row_masks<NC, true>(a_lo, a_hi, A.col, B.rp, B.re, B.col, c0, span, S.w.msk)) bad = true;
        c += warp_mask_count(S.w.msk, span);
        __syncwarp();
    }
    if (c > INT_MAX) bad = true;
    return (int)c;
}

// Writes a wide row of `nnz` entries at out_col/out_val (warp-wide): one
// SPAN_T-tile column window at a time, each cut into windows of whole tiles
// whose first entries lie in one block of SUB_NNZ entries (fewer than
// B_FUSE_CAP entries each), written by the warp-row fill on clipped B rows.
template <int AR, bool NC>
__device__ bool wide_row_fill(int a_lo, int a_hi, const BOp &A, const BOp &B, BWarpSmem &S, int nnz,
                              int *__restrict__ out_col, double *__restrict__ out_val) {
    int cmin, cmax, prod;
    warp_row_extent<NC>(a_lo, a_hi, A.col, B.rp, B.re, B.col, cmin, cmax, prod);
    if (cmax < 0) return nnz == 0;
    const int t_lo = cmin >> 6, t_hi = cmax >> 6;
    long long done = 0;
    for (int c0 = t_lo; c0 <= t_hi; c0 += SPAN_T) {
        const int span = min(SPAN_T, t_hi - c0 + 1);
        if (!warp_row_masks<NC, true>(a_lo, a_hi, A.col, B.rp, B.re, B.col, c0, span, S.w.msk)) return false;
        const int total = mask_prefix(S.w.msk, span, S.w.base);
        if (done + total > nnz) return false;
        int s0 = 0;
        for (int w0 = 0; w0 < total; w0 += SUB_NNZ) {
            // tiles [s0, s1): base in [w0, w0 + SUB_NNZ); base[s0..) is read before the
            // fill below rewrites base[s0..s1) with the window's own offsets
            const int s1 = smem_lower_bound(S.w.base, s0, span, w0 + SUB_NNZ);
            const int first = s0 < span ? S.w.base[s0] : total;
            const int n = (s1 < span ? S.w.base[s1] : total) - first;
            __syncwarp();
            if (n > 0 && !warp_row_fill<AR, NC, true>(a_lo, a_hi, A.col, A.val, B.rp, B.re, B.col, B.val, c0 + s0,
                                                      s1 - s0, S.w.msk + s0, S.w.base + s0, S.w.acc, n,
                                                      out_col + done + first, out_val + done + first))
                return false;
            s0 = s1;
        }
        done += total;
    }
    return done == nnz;
}

enum RowKind { RK_THREAD = 0, RK_WARP = 1, RK_WIDE = 2 };

// All tiles of round r, tile t by global warp t mod (warps in the grid).  A
// tile's rows are computed, the tile takes a block of its product's region
// (one atomic) and the rows are written there in row order.
template <int AR, bool NC>
__device__ void phase_tiles(const BParams &P, int r, BWarpSmem &S) {
    const BRound &R = P.rnd[r];
    const int lane = lane_id();
    const long long nw = (long long)gridDim.x * BW;
    const long long gw = (long long)blockIdx.x * BW + (threadIdx.x >> 5);
    int p = gw < R.T ? find_prod(R.tile0, R.nprod, gw) : 0;
    for (long long t = gw; t < R.T; t += nw) {
        while (__ldg(R.tile0 + p + 1) <= t) p++;
        const long long tfirst = __ldg(R.tile0 + p), prow0 = __ldg(R.row0 + p);
        const int M = (int)(__ldg(R.row0 + p + 1) - prow0);
        const int li = (int)(t - tfirst) * TILE_ROWS + lane;
        const bool valid = li < M;
        const BOp A = R.A[p];
        const BOp B = b_operand(P, r, p);
        const int a_lo = valid ? ldx<true>(A.rp + li) : 0, a_hi = valid ? ldx<true>(A.rp + li + 1) : 0;
        // thread path: the row's list is built in shared memory; rows with more
        // than `tiny` products give up (nothing written) and go to the warp
        int cnt = tiny_row_build<AR, NC>(a_lo, a_hi, A.col, A.val, B.rp, B.re, B.col, B.val, S.t.cols + lane,
                                         S.t.acc + lane, WARP, P.tiny);
        int kind = RK_THREAD;
        if (cnt < 0) kind = RK_WARP;
        unsigned bigs = __ballot_sync(FULL, kind != RK_THREAD);
        const bool had_big = bigs != 0;
        bool bad = false;
        while (bigs) {  // counts of the other rows, one row at a time (the lists are lost)
            const int src = __ffs(bigs) - 1;
            bigs &= bigs - 1;
            const int lo = __shfl_sync(FULL, a_lo, src), hi = __shfl_sync(FULL, a_hi, src);
            bool wide;
            const int c = big_row_count<NC>(lo, hi, A, B, S, wide, bad);
            if (lane == src) {
                cnt = c;
                kind = wide ? RK_WIDE : RK_WARP;
            }
        }
        if (!valid) cnt = 0;
        const int incl = warp_incl_scan(cnt);
        const int agg = __shfl_sync(FULL, incl, WARP - 1);
        unsigned long long tb = 0;
        if (lane == 0 && agg) tb = atomicAdd(R.alloc + p, (unsigned long long)agg);
        tb = __shfl_sync(FULL, tb, 0);
        const long long region = __ldg(R.reg + p + 1) - __ldg(R.reg + p);
        if ((long long)tb + agg > region) {
            if (lane == 0) atomicOr(P.err, BERR_CAPACITY);
            continue;
        }
        const int off = (int)tb + incl - cnt;  // within the region
        const long long ro = __ldg(R.rpo + p);
        if (R.last) {
            if (valid) R.rp_pool[ro + li] = cnt;
            if (lane == 0) {
                R.tbase[t] = (int)tb;
                R.tcnt[t] = agg;
            }
        } else if (valid) {
            R.rs[ro + li] = off;
            R.re[ro + li] = off + cnt;
        }
        const long long base = __ldg(R.reg + p);
        int *ocol = R.col_pool + base;
        double *oval = R.val_pool + base;
        if (!had_big) {
            if (valid) tiny_row_write(S.t.cols + lane, S.t.acc + lane, WARP, cnt, ocol + off, oval + off);
            continue;
        }
        // a tile with other rows: thread rows are built again, then the others one at a time
        if (valid && kind == RK_THREAD) {
            if (tiny_row_build<AR, NC>(a_lo, a_hi, A.col, A.val, B.rp, B.re, B.col, B.val, S.t.cols + lane,
                                       S.t.acc + lane, WARP, P.tiny) == cnt)
                tiny_row_write(S.t.cols + lane, S.t.acc + lane, WARP, cnt, ocol + off, oval + off);
            else
                bad = true;
        }
        __syncwarp();
        unsigned warps = __ballot_sync(FULL, valid && kind == RK_WARP);
        while (warps) {
            const int src = __ffs(warps) - 1;
            warps &= warps - 1;
            const int lo = __shfl_sync(FULL, a_lo, src), hi = __shfl_sync(FULL, a_hi, src);
            const int n = __shfl_sync(FULL, cnt, src), o = __shfl_sync(FULL, off, src);
            if (n == 0) continue;
            int cmin, cmax, prod;
            warp_row_extent<NC>(lo, hi, A.col, B.rp, B.re, B.col, cmin, cmax, prod);
            const int t0 = cmin >> 6, span = (cmax >> 6) - t0 + 1;
            if (span > SPAN_T || !warp_row_masks<NC>(lo, hi, A.col, B.rp, B.re, B.col, t0, span, S.w.msk) ||
                !warp_row_fill<AR, NC>(lo, hi, A.col, A.val, B.rp, B.re, B.col, B.val, t0, span, S.w.msk, S.w.base,
                                       S.w.acc, n, ocol + o, oval + o))
                bad = true;
            __syncwarp();
        }
        unsigned wides = __ballot_sync(FULL, valid && kind == RK_WIDE);
        while (wides) {
            const int src = __ffs(wides) - 1;
            wides &= wides - 1;
            const int o = __shfl_sync(FULL, off, src);
            int slot = 0;
            if (lane == 0) slot = atomicAdd(R.nwide, 1);
            slot = __shfl_sync(FULL, slot, 0);
            if (slot < WIDE_LIST) {  // written in the wide-row phase
                if (lane == 0) {
                    R.wide[2 * slot] = prow0 + (t - tfirst) * TILE_ROWS + src;
                    R.wide[2 * slot + 1] = base + o;
                }
                continue;
            }
            const int lo = __shfl_sync(FULL, a_lo, src), hi = __shfl_sync(FULL, a_hi, src);
            const int n = __shfl_sync(FULL, cnt, src);
            if (!wide_row_fill<AR, NC>(lo, hi, A, B, S, n, ocol + o, oval + o)) bad = true;
            __syncwarp();
        }
        if (__any_sync(FULL, bad) && lane == 0) atomicOr(P.err, BERR_INTERNAL);
    }
}

// the listed wide rows of round r, one per warp (after a grid barrier: every
// row's count is stored)
template <int AR, bool NC>
__device__ void phase_wide(const BParams &P, int r, BWarpSmem &S, int n) {
    const BRound &R = P.rnd[r];
    const long long nw = (long long)gridDim.x * BW;
    for (long long e = (long long)blockIdx.x * BW + (threadIdx.x >> 5); e < n; e += nw) {
        const long long i = ldx<false>(R.wide + 2 * e), o = ldx<false>(R.wide + 2 * e + 1);
        const int p = find_prod(R.row0, R.nprod, i);
        const int li = (int)(i - __ldg(R.row0 + p));
        const long long ro = __ldg(R.rpo + p);
        const BOp A = R.A[p];
        const BOp B = b_operand(P, r, p);
        const int nnz = R.last ? ldx<false>(R.rp_pool + ro + li) : ldx<false>(R.re + ro + li) - ldx<false>(R.rs + ro + li);
        if (!wide_row_fill<AR, NC>(ldx<true>(A.rp + li), ldx<true>(A.rp + li + 1), A, B, S, nnz, R.col_pool + o,
                                   R.val_pool + o) &&
            lane_id() == 0)
            atomicOr(P.err, BERR_INTERNAL);
        __syncwarp();
    }
}

// block sums of the last round's tile counts (first step of a device-wide
// exclusive scan of tcnt into tex; the blocks take equal ranges of tiles)
__device__ void scan_block_sums(const BParams &P, const BRound &R) {
    __shared__ long long s_tmp[BW + 1];
    const long long per = (R.T + gridDim.x - 1) / gridDim.x;
    const long long lo = min((long long)blockIdx.x * per, R.T), hi = min(lo + per, R.T);
    long long v = 0;
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) v += ldx<false>(R.tcnt + i);
    long long tot;
    block_excl_sum<BW * 32>(v, s_tmp, tot);
    if (threadIdx.x == 0) P.bsum[blockIdx.x] = tot;
}

// block 0: exclusive scan of the block sums
__device__ void scan_top(const BParams &P, const BRound &R) {
    __shared__ long long s_tmp[BW + 1];
    if (blockIdx.x != 0) return;
    long long carry = 0;
    for (int b0 = 0; b0 < (int)gridDim.x; b0 += blockDim.x) {
        const int b = b0 + threadIdx.x;
        const long long x = b < (int)gridDim.x ? ldx<false>(P.bsum + b) : 0;
        long long t2;
        const long long ex = block_excl_sum<BW * 32>(x, s_tmp, t2);
        if (b < (int)gridDim.x) P.bsum[b] = ex + carry;
        carry += t2;
    }
    if (threadIdx.x == 0) R.tex[R.T] = carry;
}

// the block's range of tiles scanned from its block sum, SCAN_RUN tiles per thread
__device__ void scan_blocks(const BParams &P, const BRound &R) {
    __shared__ long long s_tmp[BW + 1];
    constexpr int SCAN_RUN = 16;
    const long long per = (R.T + gridDim.x - 1) / gridDim.x;
    const long long lo = min((long long)blockIdx.x * per, R.T), hi = min(lo + per, R.T);
    long long run = ldx<false>(P.bsum + blockIdx.x);
    for (long long b = lo; b < hi; b += (long long)blockDim.x * SCAN_RUN) {
        const long long i0 = b + (long long)threadIdx.x * SCAN_RUN;
        int x[SCAN_RUN];
        long long sum = 0;
#pragma unroll
        for (int u = 0; u < SCAN_RUN; u++) {
            x[u] = i0 + u < hi ? ldx<false>(R.tcnt + i0 + u) : 0;
            sum += x[u];
        }
        long long t2;
        long long e = run + block_excl_sum<BW * 32>(sum, s_tmp, t2);
#pragma unroll
        for (int u = 0; u < SCAN_RUN; u++) {
            if (i0 + u < hi) R.tex[i0 + u] = e;
            e += x[u];
        }
        run += t2;
    }
}

// the last round in row order: every tile's block copied to its place in the
// product (scanned tile counts) and its rows' pointers written
__device__ void phase_place(const BParams &P, const BRound &R) {
    const int lane = lane_id();
    const long long nw = (long long)gridDim.x * BW;
    const long long gw = (long long)blockIdx.x * BW + (threadIdx.x >> 5);
    int p = gw < R.T ? find_prod(R.tile0, R.nprod, gw) : 0;
    for (long long t = gw; t < R.T; t += nw) {
        while (__ldg(R.tile0 + p + 1) <= t) p++;
        const long long tfirst = __ldg(R.tile0 + p);
        const int M = (int)(__ldg(R.row0 + p + 1) - __ldg(R.row0 + p));
        const int li = (int)(t - tfirst) * TILE_ROWS + lane;
        const long long ro = __ldg(R.rpo + p), base = __ldg(R.reg + p);
        const long long dst = ldx<false>(R.tex + t) - ldx<false>(R.tex + tfirst);  // within the product
        const int n = ldx<false>(R.tcnt + t);
        const int src = ldx<false>(R.tbase + t);
        const int c = li < M ? ldx<false>(R.rp_pool + ro + li) : 0;
        const int incl = warp_incl_scan(c);
        if (li < M) {
            R.rp_pool[ro + li] = (int)dst + incl - c;
            if (li == M - 1) R.rp_pool[ro + M] = (int)dst + incl;
        }
        const int *sc = R.col_pool + base + src;
        const double *sv = R.val_pool + base + src;
        int *dc = R.out_col + base + dst;
        double *dv = R.out_val + base + dst;
        for (int q = lane; q < n; q += WARP) {
            dc[q] = ldx<false>(sc + q);
            dv[q] = ldx<false>(sv + q);
        }
    }
}

template <int AR>
__global__ void __launch_bounds__(BW * 32, 2) k_batch(BParams P) {
    extern __shared__ unsigned long long s_dyn[];
    BWarpSmem &S = reinterpret_cast<BWarpSmem *>(s_dyn)[threadIdx.x >> 5];
    for (int r = 0; r < P.nrounds; r++) {
        // the first product reads only the caller's operands (read-only path); the second
        // reads the first one's output through L2
        if (r == 0) phase_tiles<AR, true>(P, r, S);
        else phase_tiles<AR, false>(P, r, S);
        if (!grid_sync(P.bar, P.err, P.spin_limit)) return;
        const BRound &R = P.rnd[r];
        const int nwide = min(*(volatile int *)R.nwide, WIDE_LIST);
        if (nwide > 0) {
            if (r == 0) phase_wide<AR, true>(P, r, S, nwide);
            else phase_wide<AR, false>(P, r, S, nwide);
        }
        if (!R.last) {
            if (nwide > 0 && !grid_sync(P.bar, P.err, P.spin_limit)) return;
            continue;
        }
        scan_block_sums(P, R);
        if (!grid_sync(P.bar, P.err, P.spin_limit)) return;
        scan_top(P, R);
        if (!grid_sync(P.bar, P.err, P.spin_limit)) return;
        scan_blocks(P, R);
        if (!grid_sync(P.bar, P.err, P.spin_limit)) return;
        phase_place(P, R);
    }
}

// ---------------------------------------------------------------- sizing
// per row of the first product: products and the bound min(products, N) on its nnz,
// summed per product; `rowbound` keeps the uncapped products of each row for
// the second product's bound
__device__ __forceinline__ void add_per_product(unsigned long long *pbound, int p, unsigned long long v) {
    const int p0 = __shfl_sync(FULL, p, 0);
    if (__all_sync(FULL, p == p0)) {
        v = warp_sum(v);
        if (lane_id() == 0 && v) atomicAdd(pbound + p0, v);
    } else if (v) {
        atomicAdd(pbound + p, v);
    }
}

__global__ void k_batch_bound(const BOp *A, const BOp *B, const long long *row0, int nprod, long long R,
                              long long *rowbound, unsigned long long *pbound) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    // every lane runs the same number of iterations (the warp-wide sums below)
    for (long long i0 = blockIdx.x * (long long)blockDim.x; i0 < R; i0 += stride) {
        const long long i = i0 + threadIdx.x;
        int p = 0;
        unsigned long long bnd = 0;
        if (i < R) {
            p = find_prod(row0, nprod, i);
            const BOp a = A[p], b = B[p];
            const int li = (int)(i - row0[p]);
            long long prod = 0;
            for (int q = a.rp[li]; q < a.rp[li + 1]; q++) {
                const int k = a.col[q];
                prod += b.rp[k + 1] - b.rp[k];
            }
            if (rowbound) rowbound[i] = prod;
            bnd = (unsigned long long)(prod < b.N ? prod : b.N);
        }
        add_per_product(pbound, p, bnd);
    }
}

// bound of a row of Pt * (A*P): the sum over its entries of the A*P row bounds, capped by N
__global__ void k_batch_bound2(const BOp *Pt, const long long *row0_2, const long long *row0_1, int nprod,
                               long long R, const long long *rowbound1, const int *ncols,
                               unsigned long long *pbound) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i0 = blockIdx.x * (long long)blockDim.x; i0 < R; i0 += stride) {
        const long long i = i0 + threadIdx.x;
        int p = 0;
        unsigned long long bnd = 0;
        if (i < R) {
            p = find_prod(row0_2, nprod, i);
            const BOp a = Pt[p];
            const int li = (int)(i - row0_2[p]);
            long long prod = 0;
            for (int q = a.rp[li]; q < a.rp[li + 1]; q++)
                prod += min(rowbound1[row0_1[p] + a.col[q]], (long long)ncols[p]);
            bnd = (unsigned long long)(prod < ncols[p] ? prod : ncols[p]);
        }
        add_per_product(pbound, p, bnd);
    }
}

}  // namespace hsmu

using namespace hsmu;

struct hsmu_batch_s {
    int kind, nprod;
    int nsm, grid, threads, tiny, arith;
    size_t smem;
    BParams P;
    std::vector<void *> allocs;
    std::vector<long long> row0[2], rpo[2], reg[2];
    std::vector<int> ncol[2];
    void *reset;          // zeroed before every launch: barrier, error word, wide-row counters, tile status
    size_t reset_bytes;
    cudaGraph_t graph;
    cudaGraphExec_t gexec;
};

namespace {

template <class T>
cudaError_t balloc(hsmu_batch_s *b, T **p, size_t n) {
    *p = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess) b->allocs.push_back(*p);
    return e;
}

template <class T>
cudaError_t bupload(hsmu_batch_s *b, T **p, const std::vector<T> &h) {
    cudaError_t e = balloc(b, p, h.size());
    if (e == cudaSuccess) e = cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    return e;
}

int launch_batch(hsmu_batch_s *b, cudaStream_t st) {
    if (cudaMemsetAsync(b->reset, 0, b->reset_bytes, st) != cudaSuccess) return HSMU_ERR_CUDA;
    b->P.tiny = b->tiny;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(b->grid);
    cfg.blockDim = dim3(b->threads);
    cfg.dynamicSmemBytes = b->smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = b->arith == AR_IMUL  ? cudaLaunchKernelEx(&cfg, k_batch<AR_IMUL>, b->P)
                    : b->arith == AR_FMA ? cudaLaunchKernelEx(&cfg, k_batch<AR_FMA>, b->P)
                                         : cudaLaunchKernelEx(&cfg, k_batch<AR_RN>, b->P);
    return e == cudaSuccess ? HSMU_OK : HSMU_ERR_CUDA;
}

int configure_batch(hsmu_batch_s *b, int dev) {
    b->threads = BW * 32;
    b->smem = BW * sizeof(BWarpSmem);
    for (auto k : {k_batch<AR_RN>, k_batch<AR_FMA>, k_batch<AR_IMUL>})
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem) != cudaSuccess)
            return HSMU_ERR_CUDA;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<AR_RN>, b->threads, b->smem) != cudaSuccess ||
        per_sm < 1)
        return HSMU_ERR_CUDA;
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop) return HSMU_ERR_NO_DEVICE;
    b->grid = b->nsm * per_sm;
    return HSMU_OK;
}

}  // namespace

extern "C" {

int hsmu_batch_create(hsmu_handle h, int kind, int n, const hsmu_csr *A, const hsmu_csr *B, const hsmu_csr *Pt,
                      const hsmu_opts *opts, hsmu_batch *out, void *stream) {
    if (!h || !out || n <= 0 || !A || !B) return HSMU_ERR_INVALID;
    if (kind != HSMU_BATCH_PRODUCT && kind != HSMU_BATCH_GALERKIN) return HSMU_ERR_INVALID;
    if (kind == HSMU_BATCH_GALERKIN && !Pt) return HSMU_ERR_INVALID;
    if (opts && (opts->arith < HSMU_ARITH_RN || opts->arith > HSMU_ARITH_IMUL)) return HSMU_ERR_INVALID;
    *out = nullptr;
    for (int p = 0; p < n; p++) {
        if (A[p].N != B[p].M || !A[p].row_ptr || !B[p].row_ptr) return HSMU_ERR_INVALID;
        if (kind == HSMU_BATCH_GALERKIN && (Pt[p].N != A[p].M || !Pt[p].row_ptr)) return HSMU_ERR_INVALID;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    hsmu_batch_s *b = new (std::nothrow) hsmu_batch_s();
    if (!b) return HSMU_ERR_ALLOC;
    b->kind = kind;
    b->nprod = n;
    b->arith = opts ? opts->arith : AR_RN;
    // test hook: barriers and look-backs that give up after opts->wait_polls polls
    b->P.spin_limit = (opts && opts->wait_polls > 0) ? (unsigned long long)opts->wait_polls : SPIN_LIMIT;
    b->tiny = TINY_MAX;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, dev);
    int rc = configure_batch(b, dev);
    const int nr = kind == HSMU_BATCH_GALERKIN ? 2 : 1;
    long long *rowbound = nullptr;
    int *dncol = nullptr;
    unsigned long long *dpb = nullptr;
    std::vector<unsigned long long> hpb;
    std::vector<long long> tiles[2];
    std::vector<BOp> hA(n), hB(n);
    if (rc) goto fail;
    b->P.nrounds = nr;
    // operand tables, row, row-pointer and tile offsets
    for (int r = 0; r < nr; r++) {
        const hsmu_csr *L = (r == 0) ? A : Pt;
        b->row0[r].assign(n + 1, 0);
        b->rpo[r].assign(n + 1, 0);
        tiles[r].assign(n + 1, 0);
        b->ncol[r].assign(n, 0);
        for (int p = 0; p < n; p++) {
            b->row0[r][p + 1] = b->row0[r][p] + L[p].M;
            b->rpo[r][p + 1] = b->rpo[r][p] + L[p].M + 1;
            tiles[r][p + 1] = tiles[r][p] + (L[p].M + TILE_ROWS - 1) / TILE_ROWS;
            b->ncol[r][p] = B[p].N;
        }
        for (int p = 0; p < n; p++) {
            hA[p] = BOp{L[p].M, L[p].N, L[p].row_ptr, L[p].row_ptr + 1, L[p].col, L[p].val};
            hB[p] = BOp{B[p].M, B[p].N, B[p].row_ptr, B[p].row_ptr + 1, B[p].col, B[p].val};
        }
        BRound &R = b->P.rnd[r];
        BOp *dA = nullptr, *dB = nullptr;
        long long *drow0 = nullptr, *drpo = nullptr, *dtile0 = nullptr;
        if (bupload(b, &dA, hA) || bupload(b, &dB, hB) || bupload(b, &drow0, b->row0[r]) ||
            bupload(b, &drpo, b->rpo[r]) || bupload(b, &dtile0, tiles[r])) {
            rc = HSMU_ERR_ALLOC;
            goto fail;
        }
        R.nprod = n;
        R.A = dA;
        R.B = (r == 0) ? dB : nullptr;
        R.b_from_prev = r > 0;
        R.row0 = drow0;
        R.rpo = drpo;
        R.tile0 = dtile0;
        R.R = b->row0[r][n];
        R.T = tiles[r][n];
    }
    // nnz bound of every product (one sizing pass and one host read): min(products, N) per row of
    // the first product; for Galerkin, per row of the second the sum of its A*P rows' bounds
    if (balloc(b, &dpb, (size_t)n * nr) || (nr == 2 && balloc(b, &rowbound, (size_t)b->P.rnd[0].R))) {
        rc = HSMU_ERR_ALLOC;
        goto fail;
    }
    cudaMemsetAsync(dpb, 0, sizeof(unsigned long long) * n * nr, st);
    k_batch_bound<<<b->nsm * 8, 256, 0, st>>>(b->P.rnd[0].A, b->P.rnd[0].B, b->P.rnd[0].row0, n, b->P.rnd[0].R,
                                              rowbound, dpb);
    if (nr == 2) {
        if (bupload(b, &dncol, b->ncol[1])) {
            rc = HSMU_ERR_ALLOC;
            goto fail;
        }
        k_batch_bound2<<<b->nsm * 8, 256, 0, st>>>(b->P.rnd[1].A, b->P.rnd[1].row0, b->P.rnd[0].row0, n,
                                                   b->P.rnd[1].R, rowbound, dncol, dpb + n);
    }
    hpb.assign((size_t)n * nr, 0);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(hpb.data(), dpb, sizeof(unsigned long long) * n * nr, cudaMemcpyDeviceToHost, st) ||
        cudaStreamSynchronize(st)) {
        rc = HSMU_ERR_CUDA;
        goto fail;
    }
    for (void *q : {(void *)rowbound, (void *)dpb, (void *)dncol}) {  // only needed for sizing
        if (!q) continue;
        cudaFree(q);
        b->allocs.erase(std::find(b->allocs.begin(), b->allocs.end(), q));
    }
    // output regions (a product's entries are indexed by int: its region is capped there; a
    // product that needs more reports HSMU_ERR_OVERFLOW), pools, row starts / row pointers
    for (int r = 0; r < nr; r++) {
        BRound &R = b->P.rnd[r];
        R.last = r == nr - 1;
        b->reg[r].assign(n + 1, 0);
        for (int p = 0; p < n; p++)
            b->reg[r][p + 1] = b->reg[r][p] + (long long)std::min<unsigned long long>(hpb[(size_t)r * n + p], INT_MAX);
        const size_t cap = (size_t)b->reg[r][n], nrp = (size_t)b->rpo[r][n];
        long long *dreg = nullptr;
        if (bupload(b, &dreg, b->reg[r]) || balloc(b, &R.col_pool, cap) || balloc(b, &R.val_pool, cap) ||
            balloc(b, &R.wide, 2 * (size_t)WIDE_LIST)) {
            rc = HSMU_ERR_ALLOC;
            goto fail;
        }
        R.reg = dreg;
        if (!R.last) {
            if (balloc(b, &R.rs, nrp) || balloc(b, &R.re, nrp)) {
                rc = HSMU_ERR_ALLOC;
                goto fail;
            }
            continue;
        }
        if (balloc(b, &R.tbase, (size_t)R.T) || balloc(b, &R.tcnt, (size_t)R.T) || balloc(b, &R.tex, (size_t)R.T + 1) ||
            balloc(b, &R.rp_pool, nrp) || balloc(b, &R.out_col, cap) || balloc(b, &R.out_val, cap)) {
            rc = HSMU_ERR_ALLOC;
            goto fail;
        }
        // row pointers of products without rows are never written by a tile
        if (cudaMemset(R.rp_pool, 0, sizeof(int) * nrp) != cudaSuccess) {
            rc = HSMU_ERR_CUDA;
            goto fail;
        }
    }
    {
        int per_sm = 0;  // the scan's block sums, for the largest grid a launch can have
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<AR_RN>, b->threads, b->smem);
        if (balloc(b, &b->P.bsum, (size_t)b->nsm * per_sm + 1)) {
            rc = HSMU_ERR_ALLOC;
            goto fail;
        }
    }
    // the block zeroed before every launch: barrier, error word, wide-row counters, allocation counters
    {
        size_t o = 0;
        const size_t o_bar = o;
        o += sizeof(GridBar);
        const size_t o_err = o;
        o += sizeof(int);
        const size_t o_nwide = o;
        o += 2 * sizeof(int);
        o = (o + 15) & ~size_t(15);
        size_t o_alloc[2] = {0, 0};
        for (int r = 0; r < nr; r++) {
            o_alloc[r] = o;
            o += sizeof(unsigned long long) * (size_t)n;
        }
        unsigned char *rb = nullptr;
        if (balloc(b, &rb, o)) {
            rc = HSMU_ERR_ALLOC;
            goto fail;
        }
        b->reset = rb;
        b->reset_bytes = o;
        b->P.bar = reinterpret_cast<GridBar *>(rb + o_bar);
        b->P.err = reinterpret_cast<int *>(rb + o_err);
        for (int r = 0; r < nr; r++) {
            b->P.rnd[r].nwide = reinterpret_cast<int *>(rb + o_nwide) + r;
            b->P.rnd[r].alloc = reinterpret_cast<unsigned long long *>(rb + o_alloc[r]);
        }
    }
    b->P.arith = b->arith;
    *out = b;
    return HSMU_OK;
fail:
    hsmu_batch_destroy(b);
    return rc;
}

int hsmu_batch_execute(hsmu_batch b, void *stream) {
    if (!b) return HSMU_ERR_INVALID;
    return launch_batch(b, static_cast<cudaStream_t>(stream));
}

int hsmu_batch_graph_launch(hsmu_batch b, void *stream) {
    if (!b) return HSMU_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (!b->gexec) {
        cudaStream_t cap;
        if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return HSMU_ERR_CUDA;
        int rc = HSMU_OK;
        if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = HSMU_ERR_CUDA;
        if (!rc) rc = launch_batch(b, cap);
        cudaGraph_t g = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(cap, &g);
        if (!rc && ee != cudaSuccess) rc = HSMU_ERR_CUDA;
        if (!rc && cudaGraphInstantiate(&b->gexec, g, 0) != cudaSuccess) rc = HSMU_ERR_CUDA;
        if (g) b->graph = g;
        cudaStreamDestroy(cap);
        if (rc) {
            cudaGetLastError();
            return rc;
        }
    }
    return cudaGraphLaunch(b->gexec, st) == cudaSuccess ? HSMU_OK : HSMU_ERR_CUDA;
}

int hsmu_batch_status(hsmu_batch b, void *stream) {
    if (!b) return HSMU_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int err = 0;
    if (cudaMemcpyAsync(&err, b->P.err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return HSMU_ERR_CUDA;
    if (err & BERR_TIMEOUT) return HSMU_ERR_TIMEOUT;
    if (err & BERR_CAPACITY) return HSMU_ERR_OVERFLOW;
    if (err) return HSMU_ERR_INTERNAL;
    return HSMU_OK;
}

int hsmu_batch_result(hsmu_batch b, int p, hsmu_csr *C) {
    if (!b || !C || p < 0 || p >= b->nprod) return HSMU_ERR_INVALID;
    const int r = b->P.nrounds - 1;
    const BRound &R = b->P.rnd[r];
    const int M = (int)(b->row0[r][p + 1] - b->row0[r][p]);
    int nnz = 0;
    if (cudaMemcpy(&nnz, R.rp_pool + b->rpo[r][p] + M, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return HSMU_ERR_CUDA;
    C->M = M;
    C->N = b->ncol[r][p];
    C->nnz = nnz;
    C->owned = 0;
    C->row_ptr = R.rp_pool + b->rpo[r][p];
    C->col = R.out_col + b->reg[r][p];
    C->val = R.out_val + b->reg[r][p];
    return HSMU_OK;
}

int hsmu_batch_set_params(hsmu_batch b, int tiny, int grid) {
    if (!b || tiny < 0 || tiny > TINY_MAX || grid < 0) return HSMU_ERR_INVALID;
    b->tiny = tiny;
    if (grid > 0) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<AR_RN>, b->threads, b->smem);
        if (grid > b->nsm * per_sm) return HSMU_ERR_INVALID;  // cooperative launch needs all blocks resident
        b->grid = grid;
    }
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    return HSMU_OK;
}

int hsmu_batch_autotune(hsmu_batch b, void *stream, int *best_tiny, int *best_grid, float *best_ms) {
    if (!b) return HSMU_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<AR_RN>, b->threads, b->smem);
    const int tinies[] = {8, 16, 32};
    std::vector<int> grids = {b->nsm * per_sm};
    if (per_sm > 1) grids.push_back(b->nsm);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int bt = b->tiny, bg = b->grid, rc = HSMU_OK;
    for (int t : tinies)
        for (int g : grids) {
            if ((rc = hsmu_batch_set_params(b, t, g))) break;
            if ((rc = launch_batch(b, st))) break;  // warm-up
            cudaEventRecord(e0, st);
            for (int k = 0; k < 2 && !rc; k++) rc = launch_batch(b, st);
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) != cudaSuccess) rc = HSMU_ERR_CUDA;
            if (rc) break;
            if ((rc = hsmu_batch_status(b, st))) break;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            ms *= 0.5f;
            if (ms < best) {
                best = ms;
                bt = t;
                bg = g;
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    rc = hsmu_batch_set_params(b, bt, bg);
    if (best_tiny) *best_tiny = bt;
    if (best_grid) *best_grid = bg;
    if (best_ms) *best_ms = best;
    return rc;
}

int hsmu_batch_destroy(hsmu_batch b) {
    if (!b) return HSMU_OK;
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (void *p : b->allocs) cudaFree(p);
    delete b;
    return HSMU_OK;
}

}  // extern "C"
