// Stage 5b: numeric phase, C values, one warp per window.
//
// GB300 counterpart of the HSMU accumulator k_formcval_shared_for_many_rows
// (src/compressed/compressed_Cval.cuh:1-69: binary search of the column in
// the row's sorted column list, then a shared-memory FP64 atomicAdd of
// aval*bval) and of the spECK dense accumulator used for rows with more than
// 4096 nnz (src/external/spECK/dense_acc.cu:2-267).
//
// Work item: a window = consecutive C tiles of one row (< WIN_CAP slots,
// <= WIN_TCAP tiles, <= WIN_SPAN tile span), cut by the structure pass.
// Slot lookup is O(1) through a tile table rebuilt from the window's sorted
// columns.  A window spanning at most WIN_TCAP tiles (the usual case) gets a
// dense table: the column bitmap of its span (one 32-bit shared atomic per
// column) and each tile's first slot as a prefix count,
//   slot(j) = tbase[t] + popc(tmask[t] & ((1 << (j & 63)) - 1)),  t = (j >> 6) - t0;
// a wider window gets a two-level table, where an occupancy bitmap over the
// span with per-word prefix counts gives the tile's rank r, which then
// indexes tmask/tbase:  r = opre[t >> 6] + popc(occ[t >> 6] below bit t & 63).
// Where each B row enters a window is precomputed for every (window, A entry)
// pair by k_win_cursors -- one search per chunk of consecutive windows of a
// row, then a short forward search per window -- so the window kernel reads
// its segment [cursor(w), cursor(w+1)) with two loads instead of searching B
// rows inside its latency-bound loop.
//
// Accumulation order is deterministic and equals the oracle's: the products
// of the window are walked in the flat order (A entry, then B entry), 32 per
// step, one per lane; lanes that hit the same slot within a step add in lane
// order, which is A-entry order, so every C entry is 0.0 + p_1 + p_2 + ...
// in the order of A(i,:) -- the same sum, bit for bit, as the host Gustavson
// oracle.  A step inside one A entry's segment has distinct slots; a step
// spanning several entries finds shared slots by stamping lane ids into a
// byte per slot (tag) and matches only the lanes that share one.  Each product is rounded before
// the add (no FMA contraction), as in the reference (`aval * bval` then
// atomicAdd).  No floating-point atomics are used.
//
// Each product costs a B load, a table lookup and an accumulator
// read-modify-write in shared memory: on power-law rows the kernel is bound by
// instruction issue and shared-memory latency, not by HBM (its traffic is the
// compulsory bytes).  The next step's B loads are issued before the current
// step's lookups and adds.
#include "hsmu_kernels.h"
#include "hsmu_products.cuh"

namespace hsmu {

constexpr int NUM_WARPS = 3;
constexpr int NUM_CTAS_PER_SM = 6;
constexpr int GW = 2;  // consecutive windows per work item, handed out dynamically
constexpr int STAGE_LIMIT = 1 << 20;  // polls of a column copy before the kernel reports a timeout

// per warp; acc first: it also receives the window's columns by bulk copy
// (16-byte aligned) before they are turned into the tile table
struct alignas(16) NumSmem {
    double acc[WIN_CAP];
    unsigned long long tmask[WIN_TCAP];
    unsigned long long occ[WIN_OCCW];
    unsigned long long bar;  // mbarrier of the column copy
    int opre[WIN_OCCW];
    unsigned short tbase[WIN_TCAP];
    unsigned char tag[WIN_CAP];  // slot stamps of the conflict test
};
// the CTAs of one SM fit its 228 KB of shared memory (1 KB reserved per CTA)
static_assert(NUM_CTAS_PER_SM * (NUM_WARPS * sizeof(NumSmem) + 1024) <= 228 * 1024, "CTAs per SM");
static_assert(WIN_CAP * 8 >= (WIN_CAP + 8) * 4, "column stage fits in the accumulator");

// The cursor pass works on chunks: runs of at most CUR_CHUNK consecutive
// windows of one row whose first tiles ascend, aligned to multiples of
// CUR_CHUNK in the window array.  Window w continues the chunk of w - 1 when:
constexpr int CUR_CHUNK = 16;
__device__ __forceinline__ bool cur_continues(const Window *win, int w, int row, int t0) {
    return w % CUR_CHUNK != 0 && win[w - 1].row == row && win[w - 1].t0 < t0;
}

// A entries of each window's row (0 past the emitted windows), scanned into
// the windows' offsets in the cursor array, and the cursor pass's work items
// (CUR_CHUNK).  A window written with a slot
// count of 0 (the large rows built from their stored tiles) gets its count
// here: up to the next window's first slot when that window continues the
// same row, else up to the row's end; and its tile count likewise, up to the
// next window's first tile or the end of the row's list.
__global__ void __launch_bounds__(256) k_win_len(Window *__restrict__ win, int win_cap, int M, const int *__restrict__ arp,
                                                 const int *__restrict__ crp, const long long *__restrict__ ts_off,
                                                 const int *__restrict__ ts_cnt, Ctl *ctl, int *__restrict__ len,
                                                 int *__restrict__ items) {
    const int nwin = min(ctl->win_count, win_cap);
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < win_cap; w += gridDim.x * blockDim.x) {
        int n = 0, it = 0;
        if (w < nwin) {
            const int row = win[w].row;
            if ((unsigned)row >= (unsigned)M) {  // a window left unwritten after a reported error
                set_err(&ctl->err, DERR_INTERNAL);
                len[w] = 0;
                items[w] = 0;
                continue;
            }
            n = arp[row + 1] - arp[row];
            // a chunk of the cursor pass starts here: one work item per 32 A entries
            if (!cur_continues(win, w, row, win[w].t0)) it = (n + WARP - 1) / WARP;
            if (win[w].cnt == 0) {
                const int s0 = win[w].s0, li = win[w].li;
                int e = crp[row + 1] - crp[row];
                long long le = (li >= 0 && ts_off) ? ts_off[row] + ts_cnt[row] : -1;
                if (w + 1 < nwin && win[w + 1].row == row && win[w + 1].s0 > s0) {
                    e = win[w + 1].s0;
                    if (win[w + 1].li > li) le = win[w + 1].li;
                }
                win[w].cnt = e - s0;
                // the tile path of the value pass needs 1..WIN_TCAP tiles; else the columns are used
                win[w].nt = (li >= 0 && le > li && le - li <= WIN_TCAP) ? (int)(le - li) : 0;
            }
        }
        len[w] = n;
        items[w] = it;
    }
}

// largest index w in [0, n] with a[w] <= x, for non-decreasing a with a[0] <= x:
// all 32 lanes probe 32 evenly spaced entries per round (log32(n) rounds)
__device__ __forceinline__ int warp_last_le(const int *__restrict__ a, int n, int x) {
    const int lane = lane_id();
    int lo = 0, hi = n;  // the answer lies in [lo, hi]; a[lo] <= x
    while (hi > lo) {
        const int step = (hi - lo + WARP - 1) / WARP;
        const int p = lo + (lane + 1) * step;
        const bool le = p <= hi && a[p] <= x;
        const int c = __popc(__ballot_sync(FULL, le));  // probes that hold form a prefix
        const int nhi = min(hi, lo + (c + 1) * step - 1);
        lo += c * step;
        hi = nhi;
    }
    return lo;
}

// cursor of (window w, A entry p of its row): index of the first entry of B row
// acol[p] whose column lies in or after the window's first tile -- found in
// B's sorted tile list, whose tile_off gives the tile's first entry.  A work
// item is one chunk of windows (CUR_CHUNK) and 32 A entries of its row, a lane
// per entry: a binary search for the chunk's first window, then, as the
// windows' first tiles ascend, a forward search from the previous position for
// each further window (mostly a probe or two in the same cache lines).  Every
// warp takes an equal share of the items (item_off: the items scanned over the
// windows), finding its first by one warp-wide search.  (A search per pair,
// all pairs in flight, took 4.6 ms of R-MAT 18's 23.8 ms value stage: its
// heavy rows pair thousands of A entries, many of them long B rows, with
// hundreds of windows.  Seeding each window's search from the previous window
// with whole rows per warp was slower still: the chained searches of a heavy
// row formed a tail.)
__global__ void __launch_bounds__(256) k_win_cursors(const Window *__restrict__ win, int win_cap, int M,
                                                     const long long *__restrict__ woff, long long cur_cap,
                                                     const int *__restrict__ arp, const int *__restrict__ acol,
                                                     const int *__restrict__ brp, const int *__restrict__ tptr,
                                                     const int *__restrict__ tcol, const int *__restrict__ toff,
                                                     const int *__restrict__ item_off, int *__restrict__ wcur,
                                                     Ctl *ctl) {
    const int nwin = min(ctl->win_count, win_cap);
    const int lane = lane_id();
    const long long gw = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const long long total = item_off[nwin];
    const int i0 = (int)(total * gw / nw), i1 = (int)(total * (gw + 1) / nw);
    if (i0 >= i1) return;
    int w = warp_last_le(item_off, nwin, i0);
    for (int i = i0; i < i1; i++) {
        while (item_off[w + 1] <= i) w++;  // windows inside the previous chunk have no items
        const Window W = win[w];
        const int row = W.row;
        if ((unsigned)row >= (unsigned)M) continue;  // reported by k_win_len
        const int a_lo = arp[row], a_hi = arp[row + 1];
        const int p = a_lo + (i - item_off[w]) * WARP + lane;
        const bool v = p < a_hi;
        int lo = 0, hi = 0, bend = 0;
        if (v) {
            const int k = __ldg(acol + p);
            lo = __ldg(tptr + k);
            hi = __ldg(tptr + k + 1);
            bend = __ldg(brp + k + 1);
        }
        int idx = v ? lower_bound_i32(tcol, lo, hi, W.t0) : 0;
        for (int ww = w;;) {
            const long long base = woff[ww];
            if (base + (a_hi - a_lo) > cur_cap) {
                if (lane == 0) set_err(&ctl->err, DERR_CAPACITY);
            } else if (v) {
                wcur[base + (p - a_lo)] = idx < hi ? __ldg(toff + idx) : bend;
            }
            if (++ww >= nwin) break;
            const Window W2 = win[ww];
            if (!cur_continues(win, ww, W2.row, W2.t0)) break;  // W2.row == row when it continues
            const int t0 = W2.t0;
            if (v) idx = gallop_gt(tcol, idx, hi, t0 - 1);  // first tile >= t0
        }
    }
}
static_assert(WIN_OCCW == 2 * WARP, "prefix pass assumes two occupancy words per lane");


template <int AR>
__global__ void __launch_bounds__(NUM_WARPS * 32, NUM_CTAS_PER_SM) k_numeric(const int *__restrict__ arp, const int *__restrict__ acol,
                                                            const double *__restrict__ aval,
                                                            const int *__restrict__ brp, const int *__restrict__ bcol,
                                                            const double *__restrict__ bval,
                                                            const int *__restrict__ crp, int *__restrict__ ccol,
                                                            double *__restrict__ cval, const Window *__restrict__ win,
                                                            int win_cap, const unsigned char *__restrict__ flag,
                                                            const int *__restrict__ scol,
                                                            const long long *__restrict__ soff,
                                                            const long long *__restrict__ woff,
                                                            const int *__restrict__ wcur, int wait_polls, int M,
                                                            const int *__restrict__ ts_tcol,
                                                            const TileEnt *__restrict__ ts_tent, Ctl *ctl) {
    extern __shared__ __align__(16) unsigned long long s_dyn[];
    const int lane = lane_id(), w = threadIdx.x >> 5;
    NumSmem &S = reinterpret_cast<NumSmem *>(s_dyn)[w];
    if (lane == 0) mbar_init(&S.bar);
    __syncwarp();
    unsigned phase = 0;
    const int nwin = min(ctl->win_count, win_cap);
    const int ngroups = (nwin + GW - 1) / GW;
    bool bad = false;
    // window costs differ by orders of magnitude (rows with thousands of A entries):
    // warps take the next group of windows from a counter instead of a fixed stride
    while (true) {
        int g = 0;
        if (lane == 0) g = atomicAdd(&ctl->win_next, 1);
        g = __shfl_sync(FULL, g, 0);
        if (g >= ngroups) break;
        const int wend = min(nwin, (g + 1) * GW);
        for (int wi = g * GW; wi < wend; wi++) {
            const Window W = win[wi];
            const int row = W.row, cnt = W.cnt, t0 = W.t0;
            if ((unsigned)row >= (unsigned)M) {  // reported by k_win_len
                bad = true;
                continue;
            }
            if (flag && flag[row] == ROW_OVERFLOW && !W.redo) continue;  // stale: the redo pass emitted fresh windows
            const int row_lo = crp[row], row_hi = crp[row + 1];
            const int s0 = row_lo + W.s0;  // windows carry row-relative offsets
            if (cnt <= 0 || cnt > WIN_CAP || W.s0 < 0 || s0 + cnt > row_hi) {
                bad = true;
                continue;
            }
            // The window's tile table comes from one of two sources.  Rows with a tile
            // list (the count pass kept their C tiles): the window's tiles themselves -- id,
            // mask and first slot -- so the table is filled with one store per tile.  Other
            // rows: the window's sorted columns, in C or (learned path, speculative pass)
            // still in the row's slot -- then they are copied to C here while the table is
            // built.  Either way bulk copies bring them into the accumulator's space.
            const bool from_slot = scol != nullptr && !W.redo;
            const bool tiles_in = ts_tent != nullptr && W.li >= 0 && W.nt > 0 && !from_slot;
            const int nt = W.nt;
            int *stage = reinterpret_cast<int *>(S.acc);
            int lead = 0;
            __syncwarp();
            if (tiles_in) {
                // entries (16 bytes each) at the start of the stage, tile ids 4096 bytes in
                const uintptr_t ga = reinterpret_cast<uintptr_t>(ts_tcol + W.li);
                lead = (int)((ga & 15u) >> 2);
                const unsigned bytes_c = (unsigned)(((lead + nt) * 4 + 15) & ~15);
                if (lane == 0)
                    bulk_g2s2(stage, ts_tent + W.li, (unsigned)nt * 16u, stage + 1024,
                              reinterpret_cast<const void *>(ga & ~(uintptr_t)15), bytes_c, &S.bar);
            } else {
                const int *__restrict__ gsrc = from_slot ? scol + soff[row] + W.s0 : ccol + s0;
                const uintptr_t ga = reinterpret_cast<uintptr_t>(gsrc);
                lead = (int)((ga & 15u) >> 2);
                const unsigned bytes = (unsigned)(((lead + cnt) * 4 + 15) & ~15);
                if (lane == 0) bulk_g2s(stage, reinterpret_cast<const void *>(ga & ~(uintptr_t)15), bytes, &S.bar);
            }
            for (int q = lane; q < WIN_TCAP; q += WARP) S.tmask[q] = 0ull;
            for (int q = lane; q < WIN_OCCW; q += WARP) S.occ[q] = 0ull;
            // wait_polls > 0 (a test hook): that many non-blocking polls, then give up
            const bool arrived = wait_polls > 0 ? mbar_poll(&S.bar, phase, wait_polls)
                                                : mbar_wait(&S.bar, phase, STAGE_LIMIT) ||
                                                      mbar_wait(&S.bar, phase, STAGE_LIMIT);
            if (!__all_sync(FULL, arrived)) {
                if (lane == 0) set_err(&ctl->err, DERR_TIMEOUT);
                // the copy still targets this warp's shared memory: let it land (bounded)
                // before the warp leaves the kernel
                mbar_wait(&S.bar, phase, STAGE_LIMIT) || mbar_wait(&S.bar, phase, STAGE_LIMIT);
                return;
            }
            phase ^= 1u;
            const int *src = stage + lead;  // the columns (column path)
            const TileEnt *ent = reinterpret_cast<const TileEnt *>(stage);  // the tiles (tile path)
            const int *tid = stage + 1024 + lead;
            int c_lo, c_hi;
            if (tiles_in) {
                const unsigned long long m_last = ent[nt - 1].mask;
                c_lo = (tid[0] << 6) + (ent[0].mask ? __ffsll((long long)ent[0].mask) - 1 : 0);
                c_hi = (tid[nt - 1] << 6) + (m_last ? 63 - __clzll((long long)m_last) : 0);
            } else {
                c_lo = src[0];
                c_hi = src[cnt - 1];
            }
            const int span = (c_hi >> 6) - t0 + 1;
            if (span <= 0 || span > WIN_SPAN || (c_lo >> 6) != t0) {
                bad = true;
                continue;
            }
            const int a_lo = arp[row], a_hi = arp[row + 1];
            const bool last = s0 + cnt == row_hi;
            // the next window continues this one: its cursors end this window's segments
            bool cont = false;
            if (!last && wi + 1 < nwin) {
                const Window W1 = win[wi + 1];
                cont = W1.row == row && W1.s0 == W.s0 + cnt && W1.redo == W.redo;
            }
            const int *__restrict__ cur0 = wcur + woff[wi];
            const int *__restrict__ cur1 = cont ? wcur + woff[wi + 1] : nullptr;

            // ---- tile table.  dense: span <= WIN_TCAP, tmask/tbase indexed by tile - t0;
            // otherwise two-level (occupancy + rank).
            const bool dense = span <= WIN_TCAP;
            const int nwords = (span + 63) >> 6;
            __syncwarp();
            if (tiles_in) {
                // one store per tile: its mask and its first slot (row-relative in the list,
                // window-relative here); a two-level table numbers the tiles by rank
                int ent_sum = 0;
                for (int q = lane; q < nt; q += WARP) {
                    const int t = tid[q] - t0;
                    const unsigned long long m = ent[q].mask;
                    const int slot = (int)(unsigned)ent[q].info - W.s0;
                    ent_sum += popc64(m);
                    if ((unsigned)t >= (unsigned)span || (unsigned)slot >= (unsigned)cnt) {
                        bad = true;
                    } else {
                        const int r = dense ? t : q;
                        S.tmask[r] = m;
                        S.tbase[r] = (unsigned short)slot;
                        if (!dense) smem_setbit64(&S.occ[t >> 6], t & 63);
                    }
                }
                if (warp_sum(ent_sum) != cnt) bad = true;
            } else             if (dense) {
                // dense: the window's column bitmap (one 32-bit shared atomic per column),
                // then every tile's first slot as the count of columns in the tiles before it
                for (int sb = 0; sb < cnt; sb += WARP) {
                    const int q = sb + lane;
                    if (q < cnt) {
                        const int c = src[q];
                        if (from_slot) ccol[s0 + q] = c;
                        const int t = (c >> 6) - t0;
                        if ((unsigned)t >= (unsigned)span) bad = true;
                        else smem_setbit64(&S.tmask[t], c & 63);
                    }
                }
                __syncwarp();
                const int per = (span + WARP - 1) / WARP;  // tiles per lane, consecutive
                const int q0 = lane * per, q1 = min(span, q0 + per);
                int sum = 0;
                for (int q = q0; q < q1; q++) sum += popc64(S.tmask[q]);
                const int incl = warp_incl_scan(sum);
                int run = incl - sum;
                for (int q = q0; q < q1; q++) {
                    S.tbase[q] = (unsigned short)run;
                    run += popc64(S.tmask[q]);
                }
                if (__shfl_sync(FULL, incl, WARP - 1) != cnt) bad = true;  // repeated columns
            } else {
                // two-level: tiles are numbered by rank in the window.  Columns are sorted,
                // so the lanes of one tile form a run; the run's first lane (head) stores
                // the tile's first slot and occupancy bit, every lane sets its column's bit
                // with a 32-bit shared atomic (a tile's bits may come from two steps)
                int run = 0, prev_t = -1;
                for (int sb = 0; sb < cnt; sb += WARP) {
                    const int s = sb + lane;
                    const bool v = s < cnt;
                    const int c = v ? src[s] : 0;
                    if (v && from_slot) ccol[s0 + s] = c;
                    const int t = (c >> 6) - t0;
                    const int t_up = __shfl_up_sync(FULL, t, 1);
                    const bool head = v && t != (lane == 0 ? prev_t : t_up);
                    const unsigned heads = __ballot_sync(FULL, head);
                    const int rank = run + __popc(heads & lanemask_le()) - 1;
                    run += __popc(heads);
                    if (v) {
                        if ((unsigned)t >= (unsigned)span || (unsigned)rank >= (unsigned)WIN_TCAP) {
                            bad = true;
                        } else {
                            if (head) {
                                S.tbase[rank] = (unsigned short)s;
                                smem_setbit64(&S.occ[t >> 6], t & 63);
                            }
                            smem_setbit64(&S.tmask[rank], c & 63);
                        }
                    }
                    prev_t = __shfl_sync(FULL, t, min(WARP, cnt - sb) - 1);
                }
            }
            __syncwarp();
            if (!dense) {
                const int q0 = 2 * lane;
                const unsigned long long o0 = q0 < nwords ? S.occ[q0] : 0ull;
                const unsigned long long o1 = q0 + 1 < nwords ? S.occ[q0 + 1] : 0ull;
                const int c0 = popc64(o0);
                const int sum = c0 + popc64(o1);
                const int ex = warp_incl_scan(sum) - sum;
                if (q0 < nwords) S.opre[q0] = ex;
                if (q0 + 1 < nwords) S.opre[q0 + 1] = ex + c0;
            }
            __syncwarp();
            // slot of column j, or -1 when j is not in the window (corrupt input)
            // two-level table (span > WIN_TCAP): occupancy bit and rank of the tile, then its
            // mask; branch-free, an absent tile or column gives -1
            auto lookup = [&](int j) -> int {
                const unsigned t = (unsigned)((j >> 6) - t0);
                const bool in = t < (unsigned)span;
                const int tc = in ? (int)t : 0;
                const unsigned long long sh = S.occ[tc >> 6] << (~tc & 63);
                const bool has = in && (long long)sh < 0;
                const int r = has ? S.opre[tc >> 6] + __popcll(sh) - 1 : 0;
                const int q = tile_slot(S.tmask[r], S.tbase[r], j);
                return has ? q : -1;
            };

            // ---- products in (A entry, B entry) order
            auto seg = [&](int p, int k, int &elo, int &ehi) {
                elo = __ldg(cur0 + (p - a_lo));
                if (cont) ehi = __ldg(cur1 + (p - a_lo));
                else if (last) ehi = __ldg(brp + k + 1);
                else ehi = gallop_gt(bcol, elo, __ldg(brp + k + 1), c_hi);  // next window not adjacent in the list
            };
            // the columns are in the table now: the accumulator takes their place
            for (int q = lane; q < cnt; q += WARP) S.acc[q] = 0.0;
            __syncwarp();
            if (dense) {
                // branch-free: an out-of-span column reads tile 0 and is rejected
                auto lookup_d = [&](int j) -> int {
                    const unsigned t = (unsigned)((j >> 6) - t0);
                    const bool in = t < (unsigned)span;
                    const int tc = in ? (int)t : 0;
                    const int q = tile_slot(S.tmask[tc], S.tbase[tc], j);
                    return in ? q : -1;
                };
                warp_accumulate<AR, true, true, true, false>(a_lo, a_hi, acol, aval, brp, bcol, bval, seg, lookup_d, S.acc,
                                                      bad, S.tag);
            } else {
                warp_accumulate<AR, true, true, true, false>(a_lo, a_hi, acol, aval, brp, bcol, bval, seg, lookup, S.acc,
                                                      bad, S.tag);
            }
            __syncwarp();
            for (int q = lane; q < cnt; q += WARP) cval[s0 + q] = S.acc[q];
            __syncwarp();
        }
    }
    if (__any_sync(FULL, bad) && lane == 0) set_err(&ctl->err, DERR_INTERNAL);
}

void launch_numeric(const DevCSR &A, const DevCSR &B, const DevTiles &Bt, const int *crp, int *ccol, double *cval,
                    const Window *win, long long win_cap, const unsigned char *flag, const int *scol,
                    const long long *soff, const WinCursors &wc, Ctl *ctl, int arith, int nsm, cudaStream_t st,
                    int wait_polls, const TileStore *ts) {
    if (win_cap <= 0) return;
    cudaMemsetAsync(&ctl->win_next, 0, sizeof(int), st);
    k_win_len<<<nsm * 4, 256, 0, st>>>(const_cast<Window *>(win), (int)win_cap, A.M, A.rp, crp, ts ? ts->off : nullptr,
                                       ts ? ts->cnt : nullptr, ctl, wc.len, wc.item_off);
    launch_scan64(wc.len, wc.off, (int)win_cap, wc.total, wc.scan_tmp, st);
    launch_scan(wc.item_off, wc.item_off, (int)win_cap, wc.total + 1, wc.scan_tmp, ctl, st);
    k_win_cursors<<<nsm * 16, 256, 0, st>>>(win, (int)win_cap, A.M, wc.off, wc.cap, A.rp, A.col, B.rp, Bt.ptr, Bt.col,
                                            Bt.off, wc.item_off, wc.cur, ctl);
    auto k = arith == AR_IMUL ? k_numeric<AR_IMUL> : arith == AR_FMA ? k_numeric<AR_FMA> : k_numeric<AR_RN>;
    k<<<nsm * NUM_CTAS_PER_SM, NUM_WARPS * 32, NUM_WARPS * sizeof(NumSmem), st>>>(
        A.rp, A.col, A.val, B.rp, B.col, B.val, crp, ccol, cval, win, (int)win_cap, flag, scol, soff, wc.off, wc.cur,
        wait_polls, A.M, ts ? ts->tcol : nullptr, ts ? ts->tent : nullptr, ctl);
}

int configure_numeric() {
    for (auto k : {k_numeric<AR_RN>, k_numeric<AR_FMA>, k_numeric<AR_IMUL>}) {
        const int e = (int)cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                NUM_WARPS * (int)sizeof(NumSmem));
        if (e) return e;
    }
    return 0;
}

// self-test of the integer-pipe multiply against the FP64 pipe on n operand
// pairs drawn from a xorshift stream (all bit patterns, values in (-1,1),
// short significands); counts mismatching results.
__global__ void k_dmul_selftest(unsigned long long n, unsigned long long seed, unsigned long long *mism) {
    unsigned long long bad = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        unsigned long long s = seed ^ (i * 0x9E3779B97F4A7C15ull);
        auto rnd = [&]() {
            s ^= s << 13;
            s ^= s >> 7;
            s ^= s << 17;
            return s;
        };
        rnd();
        double a, b;
        switch (i % 3) {
        case 0:
            a = bitsd(rnd());
            b = bitsd(rnd());
            break;
        case 1:
            a = (double)(rnd() >> 11) * 0x1p-52 - 1.0;
            b = (double)(rnd() >> 11) * 0x1p-52 - 1.0;
            break;
        default: {
            const int bits = 24 + (int)(rnd() % 8);
            a = scalbn((double)((rnd() >> (64 - bits)) | (1ull << (bits - 1))), (int)(rnd() % 200) - 100);
            b = scalbn((double)((rnd() >> (64 - bits)) | (1ull << (bits - 1))), (int)(rnd() % 200) - 100);
            break;
        }
        }
        const double x = dmul_int(a, b), y = __dmul_rn(a, b);
        const bool nan2 = (x != x) && (y != y);
        if (!nan2 && dbits(x) != dbits(y)) bad++;
    }
    if (bad) atomicAdd(mism, bad);
}

// FP64 pipe throughput probe: 8 multiply chains and 8 add chains per thread,
// independent of each other (no FMA: __dmul_rn / __dadd_rn keep them apart)
__global__ void __launch_bounds__(256) k_fp64_rate(int iters, double seed, double *out) {
    double m[8], a[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
        m[j] = seed + 1e-3 * (threadIdx.x + j);
        a[j] = seed - 1e-3 * (threadIdx.x + j);
    }
    const double f = 1.0 + 1e-12, d = 1e-15;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int j = 0; j < 8; j++) {
            m[j] = __dmul_rn(m[j], f);
            a[j] = __dadd_rn(a[j], d);
        }
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 8; j++) s += m[j] + a[j];
    if (s == 12345.678) out[threadIdx.x] = s;  // keeps the chains alive; never true for these inputs
}

int run_fp64_rate(int iters, int nsm, double *lane_ops_per_s, cudaStream_t st) {
    const int blocks = nsm * 8, threads = 256;
    double *d = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMallocAsync(&d, threads * sizeof(double), st);
    if (!e) e = cudaEventCreate(&e0);
    if (!e) e = cudaEventCreate(&e1);
    if (!e) {
        k_fp64_rate<<<blocks, threads, 0, st>>>(iters / 8 + 1, 1.0, d);  // warm-up
        cudaEventRecord(e0, st);
        k_fp64_rate<<<blocks, threads, 0, st>>>(iters, 1.0, d);
        cudaEventRecord(e1, st);
        e = cudaGetLastError();
    }
    if (!e) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (!e) e = cudaEventElapsedTime(&ms, e0, e1);
    if (!e) *lane_ops_per_s = (double)blocks * threads * (double)iters * 16.0 / (ms * 1e-3);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (d) cudaFreeAsync(d, st);
    cudaStreamSynchronize(st);
    return (int)e;
}

int run_dmul_selftest(unsigned long long n, unsigned long long seed, unsigned long long *out, cudaStream_t st) {
    unsigned long long *d = nullptr;
    cudaError_t e = cudaMallocAsync(&d, sizeof(unsigned long long), st);
    if (e) return (int)e;
    cudaMemsetAsync(d, 0, sizeof(unsigned long long), st);
    k_dmul_selftest<<<1024, 256, 0, st>>>(n, seed, d);
    e = cudaGetLastError();
    if (!e) e = cudaMemcpyAsync(out, d, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    cudaFreeAsync(d, st);
    cudaStreamSynchronize(st);
    return (int)e;
}

}  // namespace hsmu
