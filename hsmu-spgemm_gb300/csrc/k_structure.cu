// Stage 5a: C column structure and numeric work items (windows).
//
// GB300 counterpart of h_get_Ccol_from_Ctile / k_formccol_shared_for_many_rows
// (src/compressed/compressed_Ccol_symbolic.cuh:1-63,119-389), which expands
// each C tile mask into columns with __ffsll and then rank-sorts every row in
// O(n^2).  Here the row's tiles are rebuilt in a dense per-tile table
// indexed by tile id, so they are already in column order: an exclusive scan
// of the tile popcounts gives every tile's first slot and the columns are
// written sorted, with no sort at all.
//
// The same pass cuts every row into numeric windows: consecutive tiles whose
// first slot lies in the same WIN_CUT-slot block and whose tile ids lie in the
// same WIN_TCAP-tile block.  A window therefore holds < WIN_CAP slots and spans
// <= WIN_TCAP tiles, which bounds the numeric kernel's shared memory, and long
// rows are split across many warps and SMs (the reference sends rows with
// more than 4096 nnz to one CTA of the spECK dense accumulator,
// src/compressed/compressed_Cval.cuh:300-365).
//
// Rows of the warp class (tile span <= SPAN_T) with at most FUSE_CAP entries
// -- every row of the stencil and Laplacian workloads -- are finished in the
// same warp: the dense tile table that produced the columns is exactly the
// slot lookup of the value phase (slot = base[t] + popc(mask[t] below j)),
// so the products are accumulated right away and the values written with no
// window, no second walk over A and no re-read of C's columns.
//
// Output modes (RowOut): PLAIN writes every row at its final place (exact
// counts came from the symbolic pass); SPEC (learned scheduler) writes every
// row into a speculative slot sized by the predicted nnz, records the exact
// count it finds and flags rows that did not fit; REDO runs PLAIN on the
// flagged rows once the exact counts have been scanned.  Window offsets are
// row-relative so they stay valid whichever buffer the columns were written to.
#include "hsmu_block.cuh"
#include "hsmu_kernels.h"
#include "hsmu_products.cuh"
#include "hsmu_rowops.cuh"
#include "hsmu_tilelist.cuh"

namespace hsmu {

// Columns of a tile table (msk[t], first slot base[t], 0 <= t < len) written
// by the warps of a block: 32-tile groups go round-robin to the warps, a lane
// takes one tile of its group and writes the tile's columns lowest bit first;
// a group takes as many steps as its fullest tile has columns.
__device__ __forceinline__ void block_emit_tiles(const unsigned long long *msk, const int *base, int len, int warp,
                                                 int nwarps, int cb0, int *__restrict__ out) {
    const int lane = lane_id();
    for (int tb = warp * WARP; tb < len; tb += nwarps * WARP) {
        const int t = tb + lane;
        unsigned long long m = t < len ? msk[t] : 0ull;
        int *o = out + (t < len ? base[t] : 0);
        const int cb = cb0 + (t << 6);
        const int n = (int)__reduce_max_sync(FULL, (unsigned)popc64(m));
        for (int k = 0; k < n; k++) {
            if (m) {
                *o++ = cb + (__ffsll((long long)m) - 1);
                m &= m - 1ull;
            }
        }
    }
}

// Columns of the tiles lo..hi-1 of a tile table, one thread walking its tiles
// (rows of the warp class: few entries per tile, the tiles split evenly).
template <class BaseT>
__device__ __forceinline__ void emit_tiles(const unsigned long long *msk, const BaseT *base, int lo, int hi, int cb0,
                                           int *__restrict__ out) {
    for (int t = lo; t < hi; t++) {
        unsigned long long m = msk[t];
        int p = base[t];
        const int cb = cb0 + (t << 6);
        while (m) {
            out[p++] = cb + (__ffsll((long long)m) - 1);
            m &= m - 1ull;
        }
    }
}

// positions [b0, b1) of a bin (rows in ascending order) that hold the panel's rows lo <= i < hi
__device__ __forceinline__ void bin_slice(const int *rows, int n, const RowOut &o, int M, int &b0, int &b1) {
    b0 = o.lo > 0 ? lower_bound_i32(rows, 0, n, o.lo) : 0;
    b1 = o.hi < M ? lower_bound_i32(rows, b0, n, o.hi) : n;
}

// rows outside the panel, and in REDO mode rows that fitted their slots, are left alone
__device__ __forceinline__ bool skip_row(const RowOut &o, int i) {
    return i < o.lo || i >= o.hi || (o.mode == OUT_REDO && o.flag[i] != ROW_OVERFLOW);
}

__device__ __forceinline__ long long out_base(const RowOut &o, int i) {
    return o.mode == OUT_SPEC ? o.soff[i] : (long long)o.crp[i];
}
__device__ __forceinline__ int out_limit(const RowOut &o, int i) {
    return o.mode == OUT_SPEC ? (int)(o.soff[i + 1] - o.soff[i]) : o.crp[i + 1] - o.crp[i];
}

constexpr int SDS_WARPS = 4;
constexpr int SDS_CTAS_PER_SM = 6;
constexpr int SDS_WL = 64;     // > max windows of one DS row (slot cuts + tile cuts + 1)
static_assert(SPAN_T * 64 / WIN_CUT + SPAN_T / WIN_TCAP + 1 < SDS_WL, "window list of a warp row");

struct SdsSmem {
    unsigned long long msk[SPAN_T];
    unsigned short base[SPAN_T];  // slots of a warp row: at most SPAN_T * 64 = 32768
    unsigned short wl[SDS_WL];
    unsigned short wt[SDS_WL];
    double acc[FUSE_CAP];
};
static_assert(SDS_WARPS * sizeof(SdsSmem) * SDS_CTAS_PER_SM <= 227 * 1024, "CTAs per SM fit in shared memory");

template <int AR>
__global__ void __launch_bounds__(SDS_WARPS * 32, SDS_CTAS_PER_SM)
    k_struct_ds(int M, const int *__restrict__ arp, const int *__restrict__ acol, const double *__restrict__ aval,
                const int *__restrict__ brp, const int *__restrict__ bcol, const double *__restrict__ bval,
                const int *__restrict__ tptr, const int *__restrict__ tcol,
                const unsigned long long *__restrict__ tmask, RowInfo ri, RowOut out, Window *__restrict__ win,
                long long win_cap, Ctl *ctl) {
    extern __shared__ unsigned long long s_dyn[];
    const int lane = lane_id(), w = threadIdx.x >> 5;
    SdsSmem &S = reinterpret_cast<SdsSmem *>(s_dyn)[w];
    const int *rows = ri.bins + (size_t)BIN_DS * M;
    int b0, b1;
    bin_slice(rows, ctl->bin_count[BIN_DS], out, M, b0, b1);
    int *__restrict__ ccol = out.ccol;
    double *__restrict__ cval = out.cval;
    for (int r = b0 + blockIdx.x * SDS_WARPS + w; r < b1; r += gridDim.x * SDS_WARPS) {
        const int i = rows[r];
        if (skip_row(out, i)) continue;
        const int t0 = ri.tmin[i];
        const int span = ri.tmax[i] - t0 + 1;
        const long long rowbase = out_base(out, i);
        const int limit = out_limit(out, i);
        for (int t = lane; t < span; t += WARP) S.msk[t] = 0ull;
        __syncwarp();
        bool bad = false;
        warp_or_tiles<false>(arp[i], arp[i + 1], 0, WARP, acol, tptr, tcol, tmask, t0, span, S.msk, bad);
        if (__any_sync(FULL, bad)) {
            if (lane == 0) {
                set_err(&ctl->err, DERR_INTERNAL);
                if (out.mode == OUT_SPEC) {
                    out.cnnz[i] = 0;
                    out.flag[i] = ROW_OVERFLOW;
                }
            }
            __syncwarp();
            continue;
        }
        __syncwarp();
        const int per = (span + WARP - 1) / WARP;
        const int lo = min(span, lane * per), hi = min(span, lo + per);
        int sum = 0;
        for (int t = lo; t < hi; t++) sum += popc64(S.msk[t]);
        const int incl = warp_incl_scan(sum);
        const int total = __shfl_sync(FULL, incl, WARP - 1);
        const int nnz = total;
        if (out.mode == OUT_SPEC) {
            if (lane == 0) {
                out.cnnz[i] = total;
                out.flag[i] = total > limit ? ROW_OVERFLOW : (total <= FUSE_CAP ? ROW_VALUES : ROW_COLUMNS);
                if (total > limit) atomicAdd(&ctl->fallback, 1);
            }
            if (total > limit) {
                __syncwarp();
                continue;
            }
        } else if (total != limit) {
            if (lane == 0) set_err(&ctl->err, DERR_INTERNAL);
            __syncwarp();
            continue;
        }
        // window key of a tile: its first slot's WIN_CUT block and its WIN_TCAP block of
        // the row's span (a window then has < WIN_CAP slots and spans <= WIN_TCAP tiles)
        auto wkey = [](int base, int t) { return ((base / WIN_CUT) << 8) | (t / WIN_TCAP); };
        int run = incl - sum;
        int lastkey = -1;
        for (int t = lo; t < hi; t++) {
            const unsigned long long m = S.msk[t];
            S.base[t] = (unsigned short)run;
            if (m) {
                lastkey = wkey(run, t);
                run += popc64(m);
            }
        }
        __syncwarp();
        if (nnz <= FUSE_CAP) {
            // ---- fused values: columns, then products through the same dense table
            for (int q = lane; q < nnz; q += WARP) S.acc[q] = 0.0;
            emit_tiles(S.msk, S.base, lo, hi, t0 << 6, ccol + rowbase);
            __syncwarp();
            auto seg = [&](int p, int k, int &elo, int &ehi) {
                elo = __ldg(brp + k);
                ehi = __ldg(brp + k + 1);
            };
            auto lookup = [&](int j) -> int {
                const int t = (j >> 6) - t0;
                if ((unsigned)t >= (unsigned)span) return -1;
                return tile_slot(S.msk[t], S.base[t], j);
            };
            bool vbad = false;
            warp_accumulate<AR>(arp[i], arp[i + 1], acol, aval, brp, bcol, bval, seg, lookup, S.acc, vbad);
            __syncwarp();
            for (int q = lane; q < nnz; q += WARP) cval[rowbase + q] = S.acc[q];
            if (__any_sync(FULL, vbad) && lane == 0) set_err(&ctl->err, DERR_INTERNAL);
            __syncwarp();
            continue;
        }
        int carry = __shfl_up_sync(FULL, warp_incl_max(lastkey), 1);
        if (lane == 0) carry = -1;
        int nst = 0;
        {
            int kk = carry;
            for (int t = lo; t < hi; t++)
                if (S.msk[t]) {
                    const int key = wkey(S.base[t], t);
                    if (key != kk) nst++;
                    kk = key;
                }
        }
        const int st_incl = warp_incl_scan(nst);
        const int nwin = __shfl_sync(FULL, st_incl, WARP - 1);
        {
            int pos = st_incl - nst, kk = carry;
            for (int t = lo; t < hi; t++)
                if (S.msk[t]) {
                    const int key = wkey(S.base[t], t);
                    if (key != kk) {
                        S.wl[pos] = S.base[t];
                        S.wt[pos] = (unsigned short)t;
                        pos++;
                    }
                    kk = key;
                }
        }
        __syncwarp();
        int wbase = 0;
        if (lane == 0) wbase = atomicAdd(&ctl->win_count, nwin);
        wbase = __shfl_sync(FULL, wbase, 0);
        if ((long long)wbase + nwin > win_cap) {
            if (lane == 0) set_err(&ctl->err, DERR_CAPACITY);
        } else {
            for (int j = lane; j < nwin; j += WARP) {
                const int s0 = S.wl[j];
                const int e = (j + 1 < nwin) ? S.wl[j + 1] : total;
                win[wbase + j] = Window{i, s0, e - s0, t0 + S.wt[j], out.mode == OUT_REDO, -1, 0};
            }
        }
        emit_tiles(S.msk, S.base, lo, hi, t0 << 6, ccol + rowbase);
        __syncwarp();
    }
}

constexpr int SL_THREADS = 512;  // 16 warps per wide row, 3 CTAs per SM (40 registers)
// > max windows in one chunk: DCH*64/WIN_CUT (slot cuts) + DCH/WIN_TCAP (rank cuts) + DCH/WIN_SPAN + 1
constexpr int SL_WL = 512;
constexpr int SL_PER = DCH_STRUCT / SL_THREADS;
static_assert(DCH_STRUCT % WIN_SPAN == 0, "chunks must start on window span boundaries");
static_assert(DCH_STRUCT * 64 / WIN_CUT + DCH_STRUCT / WIN_TCAP + DCH_STRUCT / WIN_SPAN + 1 < SL_WL, "window list");

// packed window key of a tile: (first slot / WIN_CUT, rank / WIN_TCAP, chunk-relative tile / WIN_SPAN)
__device__ __forceinline__ long long win_key(int base, int rank, int t) {
    return ((long long)(base / WIN_CUT) << 32) | ((long long)(rank / WIN_TCAP) << 8) | (long long)(t / WIN_SPAN);
}

struct SlSmem {
    unsigned long long msk[DCH_STRUCT];
    int base[DCH_STRUCT];
    int wl[SL_WL];
    int wt[SL_WL];
};

// stored: nullable per-row tile-list counts of the tile store; rows that have a
// list (>= 0) are built by k_struct_ls (or, learned path, by the count kernel)
// and skipped here
__global__ void __launch_bounds__(SL_THREADS, 3) k_struct_l(int M, const int *__restrict__ arp,
                                                         const int *__restrict__ acol,
                                                         const int *__restrict__ tptr,
                                                         const int *__restrict__ tcol,
                                                         const unsigned long long *__restrict__ tmask, RowInfo ri,
                                                         RowOut out, Window *__restrict__ win, long long win_cap,
                                                         const int *__restrict__ stored, Ctl *ctl) {
    extern __shared__ unsigned long long s_dyn[];
    SlSmem &S = *reinterpret_cast<SlSmem *>(s_dyn);
    // warp totals of the three block scans of a chunk (one array each: one barrier per scan)
    __shared__ long long s_w0[SL_THREADS / 32], s_w1[SL_THREADS / 32];
    __shared__ int s_w2[SL_THREADS / 32];
    __shared__ int s_wbase, s_next;
    constexpr int NWARP = SL_THREADS / 32;
    const int w = threadIdx.x >> 5;
    const int *rows = ri.bins + (size_t)BIN_L * M;
    int b0, b1;
    bin_slice(rows, ctl->bin_count[BIN_L], out, M, b0, b1);
    int *__restrict__ ccol = out.ccol;
    // one row at a time from a counter (RowCounter)
    for (int r = b0 + blockIdx.x; r < b1; r = next_row_sync(&ctl->rows[ROWS_STRUCT_L], b0, &s_next)) {
        const int i = rows[r];
        if (skip_row(out, i) || (stored && stored[i] >= 0)) continue;
        const int tmin = ri.tmin[i], tmax = ri.tmax[i];
        const int a_lo = arp[i], a_hi = arp[i + 1];
        const long long rowbase = out_base(out, i);
        const int nnz = out_limit(out, i);  // exact (PLAIN/REDO) or capacity (SPEC)
        const bool one_chunk = (tmax - tmin + 1) <= DCH_STRUCT;
        int run_row = 0, tiles_row = 0;
        for (int c0 = tmin; c0 <= tmax; c0 += DCH_STRUCT) {
            const int c1 = min(c0 + DCH_STRUCT, tmax + 1);
            const int len = c1 - c0;
            for (int t = threadIdx.x; t < len; t += SL_THREADS) S.msk[t] = 0ull;
            __syncthreads();
            bool bad = false;
            if (one_chunk)
                warp_or_tiles<false, true>(a_lo, a_hi, w * WARP, NWARP * WARP, acol, tptr, tcol, tmask, c0, len, S.msk, bad);
            else
                warp_or_tiles<true, true>(a_lo, a_hi, w * WARP, NWARP * WARP, acol, tptr, tcol, tmask, c0, len, S.msk, bad);
            if (bad) set_err(&ctl->err, DERR_INTERNAL);
            __syncthreads();
            const int lo = min(len, (int)threadIdx.x * SL_PER), hi = min(len, lo + SL_PER);
            int sum = 0, ntl = 0;
            for (int t = lo; t < hi; t++) {
                const unsigned long long m = S.msk[t];
                sum += popc64(m);
                ntl += m != 0ull;
            }
            // one scan of (slots, non-empty tiles) packed into 64 bits
            long long packed_total;
            const long long packed = block_excl_sum1<SL_THREADS>(((long long)sum << 32) | ntl, s_w0, packed_total);
            const int chunk_total = (int)(packed_total >> 32), chunk_tiles = (int)(packed_total & 0xffffffffll);
            int run = (int)(packed >> 32) + run_row;
            int rank = (int)(packed & 0xffffffffll) + tiles_row;
            // window key: (first slot / WIN_CUT, tile rank / WIN_TCAP, tile / WIN_SPAN),
            // packed so that it is non-decreasing along the row
            long long lastkey = -1;
            for (int t = lo; t < hi; t++) {
                const unsigned long long m = S.msk[t];
                S.base[t] = run;
                if (m) {
                    lastkey = win_key(run, rank, t);
                    run += popc64(m);
                    rank++;
                }
            }
            const long long carry = block_excl_max1<SL_THREADS>(lastkey, s_w1, -1ll);
            int nst = 0;
            {
                long long kk = carry;
                int rk = rank - ntl;
                for (int t = lo; t < hi; t++)
                    if (S.msk[t]) {
                        const long long key = win_key(S.base[t], rk++, t);
                        if (key != kk) nst++;
                        kk = key;
                    }
            }
            int nwin;
            int pos = block_excl_sum1<SL_THREADS>(nst, s_w2, nwin);
            {
                long long kk = carry;
                int rk = rank - ntl;
                for (int t = lo; t < hi; t++)
                    if (S.msk[t]) {
                        const long long key = win_key(S.base[t], rk++, t);
                        if (key != kk) {
                            if (pos < SL_WL) {
                                S.wl[pos] = S.base[t];
                                S.wt[pos] = t;
                            }
                            pos++;
                        }
                        kk = key;
                    }
            }
            if (threadIdx.x == 0)
                s_wbase = (nwin <= SL_WL && !(out.mode == OUT_SPEC && run_row + chunk_total > nnz))
                              ? atomicAdd(&ctl->win_count, nwin)
                              : -1;
            __syncthreads();
            const int wbase = s_wbase;
            const int chunk_end = run_row + chunk_total;
            if (chunk_end > nnz && out.mode == OUT_SPEC) {
                // does not fit its speculative slot: keep counting, write nothing more
            } else if (wbase < 0 || (long long)wbase + nwin > win_cap || chunk_end > nnz) {
                if (threadIdx.x == 0) set_err(&ctl->err, wbase < 0 || chunk_end <= nnz ? DERR_CAPACITY : DERR_INTERNAL);
            } else {
                for (int j = threadIdx.x; j < nwin; j += SL_THREADS) {
                    const int s0 = S.wl[j];
                    const int e = (j + 1 < nwin) ? S.wl[j + 1] : chunk_end;
                    win[wbase + j] = Window{i, s0, e - s0, c0 + S.wt[j], out.mode == OUT_REDO, -1, 0};
                }
                block_emit_tiles(S.msk, S.base, len, w, NWARP, c0 << 6, ccol + rowbase);
            }
            run_row = chunk_end;
            tiles_row += chunk_tiles;
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            if (out.mode == OUT_SPEC) {
                out.cnnz[i] = run_row;
                out.flag[i] = run_row > nnz ? ROW_OVERFLOW : ROW_COLUMNS;
                if (run_row > nnz) atomicAdd(&ctl->fallback, 1);
            } else if (run_row != nnz) {
                set_err(&ctl->err, DERR_INTERNAL);
            }
        }
    }
    if (threadIdx.x == 0) rows_done(&ctl->rows[ROWS_STRUCT_L]);
}

// ---- large rows from their stored C tile lists (PLAIN mode, tile store present)
// The count pass kept every large row's non-empty C tiles in column order,
// each with its first slot in the row and, for a tile that starts a numeric
// window, the window's ordinal (hsmu_tilelist.cuh).  So the row needs neither
// a second OR walk over B nor any scan: every warp takes 32 consecutive tiles
// at a time, writes the windows they start (slot count left 0: the window
// length pass derives it from the next window's first slot, the row's windows
// being neighbours) and the tiles' columns -- each store of the warp covers
// consecutive entries of the row.  The row's windows were reserved by the
// count pass (ts.wbase); without that (row panels, whose windows restart at 0
// for every panel) one atomic per row reserves them here.
constexpr int SLS_THREADS = 256;

__global__ void __launch_bounds__(SLS_THREADS, 6) k_struct_ls(int M, RowInfo ri, TileStore ts, RowOut out,
                                                           Window *__restrict__ win, long long win_cap, Ctl *ctl) {
    constexpr int NT = SLS_THREADS;
    __shared__ int s_wbase, s_next;
    const int lane = lane_id(), w = threadIdx.x >> 5;
    const int *rows = ri.bins + (size_t)BIN_L * M;
    int b0, b1;
    bin_slice(rows, ctl->bin_count[BIN_L], out, M, b0, b1);
    int *__restrict__ ccol = out.ccol;
    // one row at a time from a counter (RowCounter)
    for (int r = b0 + blockIdx.x; r < b1;) {
        int next = 0;
        if (threadIdx.x == 0) next = draw_row(&ctl->rows[ROWS_STRUCT_LS], b0);
        const int i = rows[r];
        // -1: no list kept (the arena was full), k_struct_l builds this row
        const int n = skip_row(out, i) ? -1 : ts.cnt[i];
        if (n >= 0) {
            const long long sb = ts.off[i];
            const int nwin = ts.nwin[i];
            const long long rowbase = out.crp[i];  // PLAIN or REDO: final row pointers
            const int nnz = out.crp[i + 1] - out.crp[i];
            int wbase;
            if (ts.wbase) {
                wbase = ts.wbase[i];
            } else {
                if (threadIdx.x == 0) s_wbase = atomicAdd(&ctl->win_count, nwin);
                __syncthreads();
                wbase = s_wbase;
            }
            if (wbase >= 0 && (long long)wbase + nwin <= win_cap) {
                for (int q0 = w * WARP; q0 < n; q0 += NT) {
                    const int q = q0 + lane;
                    const bool v = q < n;
                    const int t = v ? __ldg(ts.tcol + sb + q) : 0;
                    // the tile's mask and slot word: one 128-bit load
                    const ulonglong2 e = v ? __ldg(reinterpret_cast<const ulonglong2 *>(ts.tent) + sb + q)
                                           : make_ulonglong2(0ull, 0ull);
                    const unsigned long long m = e.x;
                    const long long info = (long long)e.y;
                    const int slot = (int)(unsigned)info;
                    const int ord1 = (int)(info >> 32);
                    if (ord1) {
                        if (ord1 <= nwin)
                            win[wbase + ord1 - 1] = Window{i, slot, 0, t, out.mode == OUT_REDO, (int)(sb + q), 0};
                        else set_err(&ctl->err, DERR_INTERNAL);
                    }
                    // the 32 tiles' entries: slots s0 .. s0 + (their entries) - 1 of the row
                    const int s0 = __shfl_sync(FULL, slot, 0);
                    const int total = warp_sum(popc64(m));
                    if (s0 + total <= nnz) warp_emit_list(t, m, ccol + rowbase + s0);
                    else if (lane == 0) set_err(&ctl->err, DERR_INTERNAL);
                }
            } else if (threadIdx.x == 0) {
                set_err(&ctl->err, DERR_CAPACITY);
            }
        }
        // s_wbase and s_next are rewritten only after the second barrier
        if (threadIdx.x == 0) s_next = next;
        __syncthreads();
        r = s_next;
        __syncthreads();
    }
    if (threadIdx.x == 0) rows_done(&ctl->rows[ROWS_STRUCT_LS]);
}

constexpr int TINYF_THREADS = 128;

// tiny rows: one thread per row writes its sorted columns and values
template <int AR>
__global__ void __launch_bounds__(TINYF_THREADS) k_fill_tiny(int M, const int *__restrict__ arp,
                                                             const int *__restrict__ acol,
                                                             const double *__restrict__ aval,
                                                             const int *__restrict__ brp,
                                                             const int *__restrict__ bcol,
                                                             const double *__restrict__ bval, RowInfo ri,
                                                             RowOut out, Ctl *ctl) {
    __shared__ int s_cols[TINY_MAX * TINYF_THREADS];
    __shared__ double s_acc[TINY_MAX * TINYF_THREADS];
    const int *rows = ri.bins + (size_t)BIN_TINY * M;
    int b0, b1;
    bin_slice(rows, ctl->bin_count[BIN_TINY], out, M, b0, b1);
    bool bad = false;
    for (int r = b0 + blockIdx.x * TINYF_THREADS + threadIdx.x; r < b1; r += gridDim.x * TINYF_THREADS) {
        const int i = rows[r];
        if (skip_row(out, i)) continue;
        const long long c0 = out_base(out, i);
        const int lim = out_limit(out, i);
        const int got = tiny_row_fill<AR>(arp[i], arp[i + 1], acol, aval, brp, brp + 1, bcol, bval, s_cols + threadIdx.x,
                                          s_acc + threadIdx.x, TINYF_THREADS, lim, out.ccol + c0, out.cval + c0);
        if (out.mode == OUT_SPEC) {
            out.cnnz[i] = got < 0 ? 0 : got;
            out.flag[i] = got < 0 ? ROW_OVERFLOW : ROW_VALUES;
            if (got < 0) bad = true;  // tiny rows get a capacity that always fits
        } else if (got != lim) {
            bad = true;
        }
    }
    if (bad) set_err(&ctl->err, DERR_INTERNAL);
}

void launch_structure(const DevCSR &A, const DevCSR &B, const DevTiles &Bt, RowInfo ri, RowOut out, Window *win,
                      long long win_cap, Ctl *ctl, int arith, int nsm, cudaStream_t st, const int *class_rows,
                      const TileStore *ts) {
    if (!class_rows || class_rows[BIN_TINY] > 0) {
        auto kt = arith == AR_IMUL ? k_fill_tiny<AR_IMUL> : arith == AR_FMA ? k_fill_tiny<AR_FMA> : k_fill_tiny<AR_RN>;
        kt<<<nsm * 4, TINYF_THREADS, 0, st>>>(A.M, A.rp, A.col, A.val, B.rp, B.col, B.val, ri, out, ctl);
    }
    if (!class_rows || class_rows[BIN_DS] > 0) {
        auto kds = arith == AR_IMUL ? k_struct_ds<AR_IMUL> : arith == AR_FMA ? k_struct_ds<AR_FMA> : k_struct_ds<AR_RN>;
        kds<<<nsm * SDS_CTAS_PER_SM, SDS_WARPS * 32, SDS_WARPS * sizeof(SdsSmem), st>>>(
            A.M, A.rp, A.col, A.val, B.rp, B.col, B.val, Bt.ptr, Bt.col, Bt.mask, ri, out, win, win_cap, ctl);
    }
    if (!class_rows || class_rows[BIN_L] > 0) {
        // rows with a stored tile list are streamed by k_struct_ls (PLAIN, REDO; in SPEC
        // mode the count kernel already wrote them), the others take the OR walk
        const bool list = ts && ts->cnt;
        if (list && out.mode != OUT_SPEC) k_struct_ls<<<nsm * 6, SLS_THREADS, 0, st>>>(A.M, ri, *ts, out, win, win_cap, ctl);
        if (!list || !ts->all_stored)
            k_struct_l<<<nsm * 3, SL_THREADS, sizeof(SlSmem), st>>>(A.M, A.rp, A.col, Bt.ptr, Bt.col, Bt.mask, ri, out,
                                                                    win, win_cap, list ? ts->cnt : nullptr, ctl);
    }
}

int configure_structure() {
    for (auto k : {k_struct_ds<AR_RN>, k_struct_ds<AR_FMA>, k_struct_ds<AR_IMUL>}) {
        const int e = (int)cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                SDS_WARPS * (int)sizeof(SdsSmem));
        if (e) return e;
    }
    return (int)cudaFuncSetAttribute(k_struct_l, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SlSmem));
}

}  // namespace hsmu
