// Shared definitions for the GB300 HSMU SpGEMM kernels (sm_103a).
//
// Data layout in HBM (all arrays are plain device allocations):
//   A, B, C   int32 row_ptr / col, FP64 val (canonical CSR, sorted columns)
//   B tiles   tile_ptr[K+1], tile_col[T], mask[T] (u64), tile_off[T]
//   rows      per A row: products (i64), tile bound (i64), first/last C tile
//   bins      NBIN slabs of M row ids (row classes for the symbolic and
//             structure kernels)
//   windows   numeric work items {row, first slot, slot count, first tile}
//   ctl       one small control block of counters / totals / error bits
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <climits>

namespace hsmu {

constexpr int WARP = 32;
constexpr unsigned FULL = 0xffffffffu;

// A C row whose tile span is at most SPAN_T tiles is handled by one warp
// with a dense per-tile table in shared memory (symbolic / structure).
constexpr int SPAN_T = 512;
// Numeric windows: consecutive tiles of one C row with
//   < WIN_CAP slots (cut where the tile's first slot crosses a multiple of WIN_CUT),
//   <= WIN_TCAP tiles (cut where the tile's rank in the row crosses a multiple of WIN_TCAP),
//   a tile span of <= WIN_SPAN tiles (cut at multiples of WIN_SPAN from the row's first tile),
// so that the numeric kernel's two-level tile table (occupancy bitmap of
// WIN_SPAN bits + WIN_TCAP rank-ordered masks) and accumulator fit one warp.
constexpr int WIN_CAP = 1024;
constexpr int WIN_CUT = WIN_CAP - 64;
constexpr int WIN_TCAP = 256;
constexpr int WIN_SPAN = 4096;
constexpr int WIN_OCCW = WIN_SPAN / 64;
// Tiles per chunk of the CTA (large-row) kernels.
constexpr int DCH_COUNT = 4096;   // count pass: 8 B per tile  -> 32 KB (6 CTAs per SM)
constexpr int DCH_STRUCT = 4096;  // structure pass: 12 B per tile -> 48 KB (4 CTAs per SM)

// Row classes
enum RowBin : int {
    BIN_DS = 0,    // tile span <= SPAN_T : one warp, dense span table
    BIN_L = 1,     // wider rows          : one CTA, dense chunked table
    BIN_TINY = 2,  // <= TINY_MAX products: one thread, sorted insertion list
    NBIN = 3
};

// device error bits (ctl->err)
enum DevErr : int {
    DERR_UNSORTED = 1,
    DERR_INTERNAL = 2,
    DERR_CAPACITY = 4,
    DERR_OVERFLOW = 8,
    DERR_TIMEOUT = 16  // a bounded wait (an asynchronous copy) ran out
};

struct Window {
    int row;   // C row
    int s0;    // first slot of the window, relative to the row's first entry
    int cnt;   // number of slots
    int t0;    // tile id of the first slot's column
    int redo;  // 1 when emitted by the redo pass of the learned path
    int li;    // rows with a tile list: the window's first tile in the tile store, else -1
    int nt;    // rows with a tile list: tiles of the window (set with cnt before the value pass)
};

// warp-class rows with at most this many entries get their values in the
// fused structure kernel; wider ones go through numeric windows
constexpr int FUSE_CAP = 512;

// Row hand-out of a kernel that gives each CTA one row at a time: a CTA starts
// on row first + blockIdx.x and thread 0 draws its next one from `next` while
// the current row runs.  Costs of the large rows spread over orders of
// magnitude, so a fixed stride leaves a few CTAs running long after the rest.
// The pair resets itself (the last CTA to run out of rows zeroes it), so
// consecutive launches on one stream -- row panels -- need no reset between.
struct RowCounter {
    int next;
    int done;
};
enum RowCounterId : int { ROWS_COUNT_L = 0, ROWS_STRUCT_LS = 1, ROWS_STRUCT_L = 2 };

struct Ctl {
    unsigned long long products;     // sum of intermediate products
    unsigned long long win_bound;    // upper bound on the number of windows
    long long nnz;                   // exact nnz(C) (after the scan)
    int bin_count[NBIN];
    int win_count;                   // windows emitted by the structure pass
    int win_next;                    // dynamic work counter of the numeric pass
    int err;
    int ntiles;                      // B tiles (after the B conversion scan)
    int fallback;                    // learned path: rows that did not fit their slot
    int wide_rows;                   // warp-class rows with more than FUSE_CAP entries (need windows)
    long long binned;                // rows in the bins (total of the bin scan)
    unsigned long long cur_bound;    // bound on sum over windows of the row's A entries: large-class
                                     // rows (bounds pass) + warp rows above FUSE_CAP (count pass)
    unsigned long long cur_bound_ds; // same for every warp row with more than FUSE_CAP products
                                     // (bounds pass; for paths without a count pass)
    long long store_tiles;           // arena entries the large rows' lists may take (count pass)
    long long span_tiles;            // sum of the large rows' tile spans (bounds pass): a bound on it
    long long store_used;            // arena entries reserved by the count pass
    unsigned long long wide_ds_prod; // products of warp-class rows with more than FUSE_CAP products
    unsigned long long pred_wide_prod;  // learned path: products of warp-class rows predicted
                                     // above FUSE_CAP entries
    long long win_listed;            // windows of the rows with a tile list (scan total)
    RowCounter rows[3];              // row hand-out of the kernels that give a CTA one row at a time
};

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ int lane_id() { return threadIdx.x & (WARP - 1); }

// thread 0: the CTA's next row (first: the launch's first row)
__device__ __forceinline__ int draw_row(RowCounter *c, int first) {
    return first + (int)gridDim.x + atomicAdd(&c->next, 1);
}
// all threads: the CTA's next row, drawn by thread 0 when the current one is done
// (s_slot: a shared int of the kernel's own)
__device__ __forceinline__ int next_row_sync(RowCounter *c, int first, int *s_slot) {
    if (threadIdx.x == 0) *s_slot = draw_row(c, first);
    __syncthreads();
    const int r = *s_slot;
    __syncthreads();
    return r;
}
// thread 0, once per CTA after its last draw (every CTA of the launch, also one
// that had no row)
__device__ __forceinline__ void rows_done(RowCounter *c) {
    __threadfence();
    if (atomicAdd(&c->done, 1) == (int)gridDim.x - 1) {
        c->next = 0;
        c->done = 0;
    }
}

__device__ __forceinline__ unsigned lanemask_le() { return lanemask_lt() | (1u << lane_id()); }

template <class T>
__device__ __forceinline__ T warp_incl_scan(T v) {
    const int lane = lane_id();
#pragma unroll
    for (int d = 1; d < WARP; d <<= 1) {
        T o = __shfl_up_sync(FULL, v, d);
        if (lane >= d) v += o;
    }
    return v;
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(FULL, v, d);
    return v;
}

__device__ __forceinline__ int popc64(unsigned long long x) { return __popcll(x); }

// Load through the read-only path (NC: data constant for the whole launch) or
// through L2 only (!NC: data written earlier in the same launch by other
// blocks, e.g. the first product of a batched Galerkin triple product).
template <bool NC, class T>
__device__ __forceinline__ T ldx(const T *p) {
    if (NC) return __ldg(p);
    return __ldcg(p);
}

// number of set bits of m strictly below bit b (0 <= b < 64)
__device__ __forceinline__ int rank64(unsigned long long m, int b) {
    return __popcll(m & ((1ull << b) - 1ull));
}

// slot of column j in a tile whose column mask is m and whose first column
// sits at slot base, or -1 when bit (j & 63) of m is clear: the shift moves
// bit (j & 63) to bit 63, so the sign tests membership and the popcount of
// the shifted mask counts the set bits up to and including it
__device__ __forceinline__ int tile_slot(unsigned long long m, int base, int j) {
    const unsigned long long sh = m << (~j & 63);
    return (long long)sh < 0 ? base + __popcll(sh) - 1 : -1;
}

// position of the (r+1)-th lowest set bit of m (0 <= r < popc(m)): the
// largest p with popc(m & ((1 << p) - 1)) <= r, by halving steps
__device__ __forceinline__ int nth_set_bit(unsigned m, int r) {
    int p = 0;
#pragma unroll
    for (int w = 16; w > 0; w >>= 1)
        if (__popc(m & ((1u << (p + w)) - 1u)) <= r) p += w;
    return p;
}

// first index in [lo, hi) with a[idx] >= key (a sorted ascending)
__device__ __forceinline__ int lower_bound_i32(const int *__restrict__ a, int lo, int hi, int key) {
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (__ldg(a + mid) < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// the same, loading as ldx<NC> (for arrays written earlier in the same launch)
template <bool NC>
__device__ __forceinline__ int lower_bound_x(const int *a, int lo, int hi, int key) {
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (ldx<NC>(a + mid) < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// first index in [lo, hi) with a[idx] > key, searching forward from lo by
// doubling steps (cheap when the answer is close to lo)
__device__ __forceinline__ int gallop_gt(const int *__restrict__ a, int lo, int hi, int key) {
    if (lo >= hi || __ldg(a + lo) > key) return lo;
    int prev = lo, step = 1;
    while (prev + step < hi && __ldg(a + prev + step) <= key) {
        prev += step;
        step <<= 1;
    }
    const int l = prev + 1, h = min(prev + step, hi);
    return lower_bound_i32(a, l, h, key + 1);
}

__device__ __forceinline__ void set_err(int *err, int bit) { atomicOr(err, bit); }

// ---- 1-D bulk copies global -> shared memory (cp.async.bulk, the TMA unit)
// completing on an mbarrier.  Source and destination 16-byte aligned, size a
// multiple of 16 bytes.
__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// one thread: order this warp's earlier shared-memory accesses before the
// copy's writes, arm the barrier for `bytes` and start the copy
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// the same for two copies completing one barrier phase
__device__ __forceinline__ void bulk_g2s2(void *dst1, const void *src1, unsigned bytes1, void *dst2, const void *src2,
                                          unsigned bytes2, unsigned long long *bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes1 + bytes2)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst1)),
                 "l"(src1), "r"(bytes1), "r"(smem_u32(bar))
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst2)),
                 "l"(src2), "r"(bytes2), "r"(smem_u32(bar))
                 : "memory");
}

// wait until the barrier's phase `parity` has completed, at most `limit`
// polls (each poll may suspend the thread for a bounded time); false if the
// limit ran out
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity, int limit) {
    for (int it = 0; it < limit; it++) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// at most `polls` non-blocking tests of the barrier's phase `parity`
// (mbarrier.test_wait never suspends the thread); false if it has not completed
__device__ __forceinline__ bool mbar_poll(unsigned long long *bar, unsigned parity, int polls) {
    for (int it = 0; it < polls; it++) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// OR of a 64-bit mask into shared memory as 32-bit atomics on its halves.
// The SM executes 32-bit shared atomics natively; the 64-bit form measured
// 2-4x slower on GB300 when lanes of a warp hit the same word.
__device__ __forceinline__ void smem_or64(unsigned long long *p, unsigned long long v) {
    unsigned *q = reinterpret_cast<unsigned *>(p);
    const unsigned lo = (unsigned)v, hi = (unsigned)(v >> 32);
    if (lo) atomicOr(q, lo);
    if (hi) atomicOr(q + 1, hi);
}

// set bit b (0..63) of a 64-bit shared word: one 32-bit atomic
__device__ __forceinline__ void smem_setbit64(unsigned long long *p, int b) {
    atomicOr(reinterpret_cast<unsigned *>(p) + (b >> 5), 1u << (b & 31));
}

// Lanes hold keys in non-decreasing lane order (runs of equal keys) and a
// 64-bit value each; returns, on the first lane of every run, the OR over
// the run (other lanes: partial values).  Invalid lanes must carry a key
// that no valid lane has.
__device__ __forceinline__ unsigned long long warp_run_or(int key, unsigned long long v) {
    const int lane = threadIdx.x & (WARP - 1);
#pragma unroll
    for (int d = 1; d < WARP; d <<= 1) {
        const unsigned long long o = __shfl_down_sync(FULL, v, d);
        const int k = __shfl_down_sync(FULL, key, d);
        if (lane + d < WARP && k == key) v |= o;
    }
    return v;
}

}  // namespace hsmu
