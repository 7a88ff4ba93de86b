// Stage 3: exact symbolic count, nnz(C(i,:)) for every row.
//
// GB300 counterpart of the reference's two symbolic passes
// (k_tilePtr_symbolic_* in src/compressed/compressed_tilePtr_symbolic.cuh:174-496,
// which count C tiles with a shared-memory hash, and k_tileOR_* in
// src/compressed/compressed_tileOR.cuh:19-337, which OR the u64 B tile masks
// into those tiles and sum their popcounts).  Both are folded into one pass:
// the row's C tiles are ORed into a dense per-tile table indexed by
// (tile id - first tile of the row), which needs no hashing or probing
// because the bounds kernel already knows the row's exact tile span.
//   BIN_DS rows (span <= SPAN_T): one warp per row, 4 KB table per warp.
//   BIN_L  rows: one CTA per row, the span processed in chunks of DCH_COUNT
//                tiles (64 KB); B tile ranges restricted per chunk by binary
//                search when the span needs more than one chunk.
// Every B tile access is a coalesced 4+8 byte load of the flat (A entry,
// B tile) sequence, 32 lanes busy regardless of row lengths.
// With a tile store, the large-row pass also writes every row's non-empty C
// tiles (id + mask, ascending) to the store, compacted chunk by chunk with one
// block scan, so that the structure pass can stream them (the reference
// likewise keeps C's tiles between its symbolic passes, C->d_tile_col /
// C->d_mask_num, src/compressed/compressed_tileOR.cuh:389-623).
#include "hsmu_block.cuh"
#include "hsmu_kernels.h"
#include "hsmu_rowops.cuh"
#include "hsmu_tilelist.cuh"

namespace hsmu {

constexpr int DS_WARPS = 8;

__global__ void __launch_bounds__(DS_WARPS * 32) k_count_ds(int M, const int *__restrict__ arp,
                                                            const int *__restrict__ acol,
                                                            const int *__restrict__ tptr,
                                                            const int *__restrict__ tcol,
                                                            const unsigned long long *__restrict__ tmask,
                                                            RowInfo ri, Ctl *ctl) {
    __shared__ unsigned long long s_mask[DS_WARPS][SPAN_T];
    const int lane = lane_id(), w = threadIdx.x >> 5;
    unsigned long long *msk = s_mask[w];
    const int n = ctl->bin_count[BIN_DS];
    const int *rows = ri.bins + (size_t)BIN_DS * M;
    for (int r = blockIdx.x * DS_WARPS + w; r < n; r += gridDim.x * DS_WARPS) {
        const int i = rows[r];
        const int t0 = ri.tmin[i];
        const int span = ri.tmax[i] - t0 + 1;
        for (int t = lane; t < span; t += WARP) msk[t] = 0ull;
        __syncwarp();
        bool bad = false;
        warp_or_tiles<false>(arp[i], arp[i + 1], 0, WARP, acol, tptr, tcol, tmask, t0, span, msk, bad);
        if (bad) set_err(&ctl->err, DERR_INTERNAL);
        __syncwarp();
        int cnt = 0;
        for (int t = lane; t < span; t += WARP) cnt += popc64(msk[t]);
        cnt = warp_sum(cnt);
        if (lane == 0) {
            ri.cnnz[i] = cnt;
            if (cnt > FUSE_CAP) {  // goes through numeric windows: count them for the cursor array
                atomicAdd(&ctl->wide_rows, 1);
                const unsigned long long wb = cnt / WIN_CUT + (span - 1) / WIN_TCAP + 1;
                atomicAdd(&ctl->cur_bound, wb * (unsigned long long)(arp[i + 1] - arp[i]));
            }
        }
        __syncwarp();
    }
}

constexpr int L_THREADS = 256;

// Large rows, one CTA per row: the OR of B's tile masks per chunk of the row's
// tile span, then
//   LM_COUNT  the row's nnz;
//   LM_STORE  also the row's tile list in the arena (the plain path: the
//             structure pass streams it once C is allocated);
//   LM_SPEC   the same in the learned path's speculative pass: the row is
//             flagged ROW_OVERFLOW so that the pass after the exact scan
//             writes it, from its list, straight to its place in C.  (Writing
//             the columns into the predicted slot in this pass, so that the
//             list needs no second pass, was measured slower: R-MAT 18 47.3 ms
//             against 44.1 for the plain path -- the emission lengthens this
//             barrier-bound kernel, and the slot still has to be copied to C.)
// A row that finds the arena full keeps no list (ts.cnt = -1) and is left to
// the OR-walk structure kernel.
enum LMode { LM_COUNT = 0, LM_STORE = 1, LM_SPEC = 2 };

template <int MODE>
__global__ void __launch_bounds__(L_THREADS, 6) k_count_l(int M, const int *__restrict__ arp,
                                                       const int *__restrict__ acol,
                                                       const int *__restrict__ tptr,
                                                       const int *__restrict__ tcol,
                                                       const unsigned long long *__restrict__ tmask,
                                                       RowInfo ri, TileStore ts, RowOut out, Ctl *ctl) {
    constexpr bool STORE = MODE != LM_COUNT;
    constexpr bool SPEC = MODE == LM_SPEC;
    extern __shared__ unsigned long long s_dyn[];
    unsigned long long *msk = s_dyn;  // DCH_COUNT entries
    __shared__ int s_red[L_THREADS / 32];
    __shared__ long long s_tsum[L_THREADS / 32];
    __shared__ ListSmem<L_THREADS / 32> s_ls;
    __shared__ long long s_off;
    __shared__ int s_next;
    const int lane = lane_id(), w = threadIdx.x >> 5;
    constexpr int NWARP = L_THREADS / 32;
    const int n = ctl->bin_count[BIN_L];
    const int *rows = ri.bins + (size_t)BIN_L * M;
    // one row at a time from a counter (RowCounter)
    for (int r = blockIdx.x; r < n;) {
        int next = 0;
        if (threadIdx.x == 0) next = draw_row(&ctl->rows[ROWS_COUNT_L], 0);
        const int i = rows[r];
        const int tmin = ri.tmin[i], tmax = ri.tmax[i];
        const int a_lo = arp[i], a_hi = arp[i + 1];
        const bool one_chunk = (tmax - tmin + 1) <= DCH_COUNT;
        int total = 0;
        ListRun run{0, 0, 0, -1ll};
        long long sbase = -1;
        int scap = 0;
        if (ri.store) {
            // the row's list has at most one C tile per tile of its span and per B tile it
            // reads; the sizes add up to the arena the next call wants
            long long ts_sum = 0;
            for (int p = a_lo + (int)threadIdx.x; p < a_hi; p += L_THREADS) {
                const int k = __ldg(acol + p);
                ts_sum += __ldg(tptr + k + 1) - __ldg(tptr + k);
            }
            ts_sum = warp_sum(ts_sum);
            if (lane == 0) s_tsum[w] = ts_sum;
            __syncthreads();
            long long tsum = 0;
            for (int j = 0; j < NWARP; j++) tsum += s_tsum[j];
            scap = (int)min(tsum, (long long)(tmax - tmin + 1));
            if (threadIdx.x == 0) atomicAdd(reinterpret_cast<unsigned long long *>(&ctl->store_tiles), (unsigned long long)scap);
        }
        if (STORE) {
            // reserve the row's list in the arena (none when it is full)
            if (threadIdx.x == 0) {
                long long o = atomicAdd(reinterpret_cast<unsigned long long *>(&ctl->store_used),
                                        (unsigned long long)scap);
                if (o + scap > ts.cap) o = -1;
                s_off = o;
                ts.off[i] = o;
            }
            __syncthreads();
            sbase = s_off;
        }
        for (int c0 = tmin; c0 <= tmax; c0 += DCH_COUNT) {
            const int c1 = min(c0 + DCH_COUNT, tmax + 1);
            for (int t = threadIdx.x; t < c1 - c0; t += L_THREADS) msk[t] = 0ull;
            __syncthreads();
            bool bad = false;
            if (one_chunk)
                warp_or_tiles<false, true>(a_lo, a_hi, w * WARP, NWARP * WARP, acol, tptr, tcol, tmask, c0, c1 - c0, msk, bad);
            else
                warp_or_tiles<true, true>(a_lo, a_hi, w * WARP, NWARP * WARP, acol, tptr, tcol, tmask, c0, c1 - c0, msk, bad);
            if (bad) set_err(&ctl->err, DERR_INTERNAL);
            __syncthreads();
            if (STORE && sbase >= 0) {
                // the chunk's non-empty tiles appended to the row's list, with their slots
                // and window starts (hsmu_tilelist.cuh)
                if (!chunk_to_list<NWARP>(msk, c1 - c0, c0, tmin, run, s_ls, sbase, scap, ts.tcol, ts.tent) &&
                    threadIdx.x == 0)
                    set_err(&ctl->err, DERR_INTERNAL);
                total = run.slots;
            } else {
                int cnt = 0;
                for (int t = threadIdx.x; t < c1 - c0; t += L_THREADS) cnt += popc64(msk[t]);
                cnt = warp_sum(cnt);
                if (lane == 0) s_red[w] = cnt;
                __syncthreads();
                if (threadIdx.x == 0) {
                    int s = 0;
                    for (int j = 0; j < NWARP; j++) s += s_red[j];
                    total += s;
                }
            }
            __syncthreads();
        }
        const bool listed = STORE && sbase >= 0 && run.tiles <= scap;
        if (threadIdx.x == 0) {
            ri.cnnz[i] = total;
            if (STORE) {
                ts.cnt[i] = listed ? run.tiles : -1;  // over the capacity: reported above
                ts.nwin[i] = listed ? run.wins : 0;   // scanned in row order into the rows' first windows
            }
            if (SPEC) out.flag[i] = listed ? ROW_OVERFLOW : ROW_NONE;  // unlisted: the OR-walk kernel
            s_next = next;
        }
        __syncthreads();
        r = s_next;
        __syncthreads();
    }
    if (threadIdx.x == 0) rows_done(&ctl->rows[ROWS_COUNT_L]);
}

constexpr int TINY_THREADS = 256;

// tiny rows: one thread per row, distinct columns counted by sorted insertion
__global__ void __launch_bounds__(TINY_THREADS) k_count_tiny(int M, const int *__restrict__ arp,
                                                             const int *__restrict__ acol,
                                                             const int *__restrict__ brp,
                                                             const int *__restrict__ bcol, RowInfo ri, Ctl *ctl) {
    __shared__ int s_cols[TINY_MAX * TINY_THREADS];
    const int n = ctl->bin_count[BIN_TINY];
    const int *rows = ri.bins + (size_t)BIN_TINY * M;
    bool bad = false;
    for (int r = blockIdx.x * TINY_THREADS + threadIdx.x; r < n; r += gridDim.x * TINY_THREADS) {
        const int i = rows[r];
        const int c = tiny_row_count(arp[i], arp[i + 1], acol, brp, brp + 1, bcol, s_cols + threadIdx.x, TINY_THREADS);
        if (c < 0) bad = true;
        ri.cnnz[i] = c < 0 ? 0 : c;
    }
    if (bad) set_err(&ctl->err, DERR_INTERNAL);
}

void launch_count_small(const DevCSR &A, const DevCSR &B, const DevTiles &Bt, RowInfo ri, Ctl *ctl, int nsm,
                        cudaStream_t st) {
    k_count_tiny<<<nsm * 4, TINY_THREADS, 0, st>>>(A.M, A.rp, A.col, B.rp, B.col, ri, ctl);
    k_count_ds<<<nsm * 6, DS_WARPS * 32, 0, st>>>(A.M, A.rp, A.col, Bt.ptr, Bt.col, Bt.mask, ri, ctl);
}

void launch_count_large(const DevCSR &A, const DevTiles &Bt, RowInfo ri, const TileStore *ts, Ctl *ctl, int nsm,
                        cudaStream_t st) {
    const size_t smem = DCH_COUNT * sizeof(unsigned long long);
    if (ts && ts->tcol && ts->tent && ts->cap > 0 && ri.store)
        k_count_l<LM_STORE><<<nsm * 6, L_THREADS, smem, st>>>(A.M, A.rp, A.col, Bt.ptr, Bt.col, Bt.mask, ri, *ts,
                                                               RowOut{}, ctl);
    else
        k_count_l<LM_COUNT><<<nsm * 6, L_THREADS, smem, st>>>(A.M, A.rp, A.col, Bt.ptr, Bt.col, Bt.mask, ri,
                                                               TileStore{}, RowOut{}, ctl);
}

void launch_spec_large(const DevCSR &A, const DevTiles &Bt, RowInfo ri, const TileStore &ts, RowOut out, Ctl *ctl,
                       int nsm, cudaStream_t st) {
    const size_t smem = DCH_COUNT * sizeof(unsigned long long);
    k_count_l<LM_SPEC><<<nsm * 6, L_THREADS, smem, st>>>(A.M, A.rp, A.col, Bt.ptr, Bt.col, Bt.mask, ri, ts, out, ctl);
}

void launch_count(const DevCSR &A, const DevCSR &B, const DevTiles &Bt, RowInfo ri, Ctl *ctl, int nsm,
                  cudaStream_t st) {
    launch_count_small(A, B, Bt, ri, ctl, nsm, st);
    launch_count_large(A, Bt, ri, nullptr, ctl, nsm, st);
}

int configure_count() {
    for (auto k : {k_count_l<LM_COUNT>, k_count_l<LM_STORE>, k_count_l<LM_SPEC>}) {
        const int e = (int)cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                DCH_COUNT * (int)sizeof(unsigned long long));
        if (e) return e;
    }
    return 0;
}

}  // namespace hsmu
