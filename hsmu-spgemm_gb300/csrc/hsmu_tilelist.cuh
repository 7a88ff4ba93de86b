// A large row's C tiles as an ordered list: the count pass builds each
// 4096-tile chunk of the row as a dense table in shared memory (OR of B's
// tile masks); chunk_to_list turns that table into the row's list of
// non-empty tiles, in column order, with everything the structure pass needs
// to write the row without any scan of its own:
//   tcol       tile id,
//   tent.mask  column mask,
//   tent.info  (first slot of the tile in the row) | ((window ordinal + 1) << 32)
//              for a tile that starts a numeric window (0 in the high word otherwise).
// Windows are cut where a tile's first slot crosses a multiple of WIN_CUT, its
// rank among the row's tiles crosses a multiple of WIN_TCAP, or its offset
// from the row's first tile crosses a multiple of WIN_SPAN -- the limits of
// the value pass's per-window tables (a window has < WIN_CAP slots, <= WIN_TCAP
// tiles and a span of <= WIN_SPAN tiles).
//
// The chunk is split into one contiguous range per warp; each warp reads its
// range lane-strided (no bank conflicts) and compacts it in order with
// ballots straight into the list; the slot and window walks then run over
// the compacted entries only (a sparse row's table is mostly empty).  Two
// block-wide exchanges of per-warp totals (entries and tiles, then window
// starts) give every warp its place in the row.
#pragma once
#include "hsmu_block.cuh"
#include "hsmu_kernels.h"

namespace hsmu {

// window key of a row's tile: non-decreasing along the row; a window starts
// where it changes
__device__ __forceinline__ long long win_key_row(int slot, int rank, int toff) {
    return ((long long)(slot / WIN_CUT) << 40) | ((long long)(rank / WIN_TCAP) << 20) | (long long)(toff / WIN_SPAN);
}

// what a row's list holds before the current chunk (the same in every thread)
struct ListRun {
    int slots;      // entries
    int tiles;      // non-empty tiles
    int wins;       // windows started
    long long key;  // key of the last tile (-1 at the row's start)
};

template <int NW>
struct ListSmem {
    int pc[NW], ne[NW], st[NW];
};

// Appends the non-empty tiles of the chunk table msk[0..len) (tile ids c0 ..
// c0+len-1 of a row whose first tile is tmin) to the row's list at
// out_*[base + run.tiles ...], and advances `run`.  Every thread of the block
// (NW warps) calls it; it contains three __syncthreads and reads msk only
// (the caller separates chunks with a __syncthreads of its own).
// Steps, each split evenly over the warps: per-warp totals of the dense table;
// the table compacted in order into the list with every tile's slot; window
// starts counted over the compacted entries (every lane holds a tile, so a
// tile's predecessor is the previous lane); window ordinals written.  Returns
// false (nothing written) if the chunk's tiles would go past `cap` entries.
template <int NW>
__device__ bool chunk_to_list(const unsigned long long *msk, int len, int c0, int tmin, ListRun &run, ListSmem<NW> &sm,
                              long long base, int cap, int *__restrict__ out_col, TileEnt *__restrict__ out_ent) {
    const int lane = lane_id(), w = threadIdx.x >> 5;
    const int wspan = (((len + NW - 1) / NW) + WARP - 1) & ~(WARP - 1);
    const int w0 = min(len, w * wspan), w1 = min(len, w0 + wspan);
    // ---- per-warp totals of the dense table: entries and tiles
    {
        int pc = 0, ne = 0;
        for (int t = w0 + lane; t < w1; t += WARP) {
            const unsigned long long m = msk[t];
            pc += popc64(m);
            ne += m != 0ull;
        }
        pc = warp_sum(pc);
        ne = warp_sum(ne);
        if (lane == 0) {
            sm.pc[w] = pc;
            sm.ne[w] = ne;
        }
    }
    __syncthreads();
    int sb = run.slots, rb = run.tiles, tot_pc = 0, tot_ne = 0;
#pragma unroll
    for (int j = 0; j < NW; j++) {
        const int pcj = sm.pc[j], nej = sm.ne[j];
        if (j < w) {
            sb += pcj;
            rb += nej;
        }
        tot_pc += pcj;
        tot_ne += nej;
    }
    const bool fits = run.tiles + tot_ne <= cap;
    // ---- the warp's part compacted in order: tile ids, masks and first slots
    if (fits) {
        long long pos = base + rb;
        int s_run = sb;
        for (int tb = w0; tb < w1; tb += WARP) {
            const int t = tb + lane;
            const unsigned long long m = t < w1 ? msk[t] : 0ull;
            const int pc = popc64(m);
            const int incl = warp_incl_scan(pc);
            const unsigned nz = __ballot_sync(FULL, m != 0ull);
            if (m) {
                const long long at = pos + __popc(nz & lanemask_lt());
                out_col[at] = c0 + t;
                out_ent[at] = TileEnt{m, (long long)(unsigned)(s_run + incl - pc)};
            }
            pos += __popc(nz);
            s_run += __shfl_sync(FULL, incl, WARP - 1);
        }
    }
    __syncthreads();  // the chunk's list entries are visible to the block
    // ---- window starts over the chunk's entries [run.tiles, run.tiles + tot_ne) (row
    // ranks), split evenly over the warps
    const int per = (tot_ne + NW - 1) / NW;
    const int qa = min(tot_ne, w * per), qb = min(tot_ne, qa + per);
    auto key_at = [&](int q) -> long long {  // key of chunk entry q (row rank run.tiles + q)
        const long long at = base + run.tiles + q;
        return win_key_row((int)(unsigned)out_ent[at].info, run.tiles + q, out_col[at] - tmin);
    };
    long long kin = run.key;
    if (fits && qa < qb && qa > 0) kin = key_at(qa - 1);
    auto walk = [&](bool wr, int ob) -> int {
        int starts = 0;
        long long kprev = kin;
        for (int q0 = qa; q0 < qb; q0 += WARP) {
            const int q = q0 + lane;
            const bool v = q < qb;
            const long long key = v ? key_at(q) : LLONG_MAX;
            const long long kup = __shfl_up_sync(FULL, key, 1);
            const bool start = v && key != (lane == 0 ? kprev : kup);
            const unsigned sbits = __ballot_sync(FULL, start);
            if (wr && start) {
                const long long at = base + run.tiles + q;
                const long long ord1 = (long long)(ob + starts + __popc(sbits & lanemask_lt()) + 1);
                out_ent[at].info = (ord1 << 32) | (long long)(unsigned)out_ent[at].info;
            }
            starts += __popc(sbits);
            kprev = __shfl_sync(FULL, key, min(WARP, qb - q0) - 1);
        }
        return starts;
    };
    const int st_w = fits ? walk(false, 0) : 0;
    if (lane == 0) sm.st[w] = st_w;
    __syncthreads();
    int ob = run.wins, tot_st = 0;
#pragma unroll
    for (int j = 0; j < NW; j++) {
        if (j < w) ob += sm.st[j];
        tot_st += sm.st[j];
    }
    if (fits) walk(true, ob);
    // the chunk's last key (its slot half is never rewritten, whatever the ordinal writes do)
    if (fits && tot_ne > 0) run.key = key_at(tot_ne - 1);
    run.slots += tot_pc;
    run.tiles += tot_ne;
    run.wins += tot_st;
    return fits;
}

// Columns of 32 consecutive tiles of a row's list, one per lane (t, m; lanes
// past the list carry m = 0), whose first entry goes to out[0].  The tiles'
// entries are consecutive in the row:
//   dense tiles (at least EMIT_DENSE entries on average): one tile at a time,
//     lane b writes the entries of bits b and b + 32 (every store of the warp
//     lands in one contiguous run);
//   sparse tiles, none with more than EMIT_OWN entries: every lane writes its
//     own tile's entries, lowest set bit first (as many steps as the fullest
//     tile has entries; the stores of a step land a few entries apart);
//   otherwise: lane k of each step writes entry kb + k, found as the
//     (k - first entry of its tile)-th set bit of its tile's mask.
constexpr int EMIT_DENSE = 10;
constexpr int EMIT_OWN = 8;

__device__ __forceinline__ void warp_emit_list(int t, unsigned long long m, int *__restrict__ out) {
    const int lane = lane_id();
    const int pc = popc64(m);
    const int incl = warp_incl_scan(pc);
    const int total = __shfl_sync(FULL, incl, WARP - 1);
    const int excl = incl - pc;
    const int most = (int)__reduce_max_sync(FULL, (unsigned)pc);
    if (most <= EMIT_OWN) {
        unsigned long long mm = m;
        const int cb = t << 6;
        int pos = excl;
        for (int it = 0; it < most; it++) {
            if (mm) {
                out[pos++] = cb + __ffsll((long long)mm) - 1;
                mm &= mm - 1ull;
            }
        }
        return;
    }
    if (total >= WARP * EMIT_DENSE) {
        const unsigned below = lanemask_lt();
        for (int j = 0; j < WARP; j++) {
            const unsigned long long mj = __shfl_sync(FULL, m, j);
            if (!mj) continue;  // the same for every lane
            const int cb = __shfl_sync(FULL, t, j) << 6;
            const int ej = __shfl_sync(FULL, excl, j);
            const unsigned lo = (unsigned)mj, hi = (unsigned)(mj >> 32);
            if ((lo >> lane) & 1u) out[ej + __popc(lo & below)] = cb + lane;
            if ((hi >> lane) & 1u) out[ej + __popc(lo) + __popc(hi & below)] = cb + 32 + lane;
        }
        return;
    }
    for (int kb = 0; kb < total; kb += WARP) {
        const int k = kb + lane;
        const int j = min(seg_of(incl, k), WARP - 1);
        const unsigned long long mj = __shfl_sync(FULL, m, j);
        const int tj = __shfl_sync(FULL, t, j);
        const int r = k - __shfl_sync(FULL, excl, j);
        const unsigned lo = (unsigned)mj, hi = (unsigned)(mj >> 32);
        const int plo = __popc(lo);
        const bool in_lo = r < plo;
        const int bit = nth_set_bit(in_lo ? lo : hi, in_lo ? r : max(0, r - plo)) + (in_lo ? 0 : 32);
        if (k < total) out[k] = (tj << 6) + bit;
    }
}

}  // namespace hsmu
