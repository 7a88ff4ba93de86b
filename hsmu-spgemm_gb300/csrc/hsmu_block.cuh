// Warp- and block-level helpers shared by the symbolic, structure and
// numeric kernels: the flattened walk over the (A entry, B segment) pairs of
// one row, and block scans.
#pragma once
#include "hsmu_common.cuh"

namespace hsmu {

// Index of the segment that owns flat item g, given the inclusive prefix
// `incl` of 32 segment lengths held one per lane (non-decreasing): the number
// of lanes whose incl <= g.  All 32 lanes must call it (5 indexed shuffles).
__device__ __forceinline__ int seg_of(int incl, int g) {
    int s = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
        const int v = __shfl_sync(FULL, incl, s + step - 1);
        if (v <= g) s += step;
    }
    return s;
}

// Visit every B tile of the rows referenced by A entries [a_lo, a_hi) (row k:
// tiles tptr[k] .. tend[k]-1; tend = tptr + 1 for a CSR-style pointer array), with
// the tile range of each B row optionally restricted to tile ids [c0, c1)
// (RESTRICT: lower_bound on the sorted tile ids).  The A entries are taken
// 32 at a time (one per lane: segment = that entry's B tile range); the flat
// sequence of (A entry, B tile) items is then shared out in steps of 32
// consecutive items, starting at flat offset `first` and advancing `stride`
// items, so one warp (first 0, stride 32) or all warps of a CTA
// (first 32*w, stride 32*nwarps) keep every lane busy whatever the B row
// lengths.  fn(tile_index) is called for valid items only.
template <bool RESTRICT, bool NC = true, class Fn>
__device__ __forceinline__ void warp_walk_tiles(int a_lo, int a_hi, int first, int stride,
                                                const int *__restrict__ acol, const int *__restrict__ tptr,
                                                const int *__restrict__ tend, const int *__restrict__ tcol, int c0,
                                                int c1, Fn fn) {
    const int lane = lane_id();
    for (int pb = a_lo; pb < a_hi; pb += WARP) {
        const int p = pb + lane;
        int lo = 0, hi = 0;
        if (p < a_hi) {
            const int k = ldx<NC>(acol + p);
            lo = ldx<NC>(tptr + k);
            hi = ldx<NC>(tend + k);
            if (RESTRICT) {
                lo = lower_bound_x<NC>(tcol, lo, hi, c0);
                hi = lower_bound_x<NC>(tcol, lo, hi, c1);
            }
        }
        const int len = hi - lo;
        const int incl = warp_incl_scan(len);
        const int total = __shfl_sync(FULL, incl, WARP - 1);
        const int excl = incl - len;
        for (int f = first; f < total; f += stride) {
            const int g = f + lane;
            const int s = seg_of(incl, g);
            const int idx = __shfl_sync(FULL, lo, s) + (g - __shfl_sync(FULL, excl, s));
            if (g < total) fn(idx);
        }
    }
}

// OR the column masks of the B tiles of the rows referenced by A entries
// [a_lo, a_hi) into msk[t - t0] for tile ids t0 <= t < t0 + len (tiles
// outside set `bad`); RESTRICT limits each B row to tile ids [t0, t0 + len).
// Items are shared out as in warp_walk_tiles, OR_U steps at a time: the tile
// ids and masks of all OR_U steps are loaded before any of them is ORed in,
// so a warp keeps OR_U L2 round trips in flight instead of one.
constexpr int OR_U = 4;

// PACKED: the non-empty tile ranges of a group of A entries are packed into
// lanes 0..nseg-1 (flat start st, index shift d = lo - st) and every step finds
// the range of each item from the starts that fall inside it (one ballot and
// one OR-reduction) instead of a shuffle search.  It pays off where a group
// holds many short ranges (power-law rows, many steps per group); for groups
// of a few steps (stencil rows) the packing costs more than it saves.
template <bool RESTRICT, bool PACKED = false>
__device__ __forceinline__ void warp_or_tiles(int a_lo, int a_hi, int first, int stride,
                                              const int *__restrict__ acol, const int *__restrict__ tptr,
                                              const int *__restrict__ tcol,
                                              const unsigned long long *__restrict__ tmask, int t0, int len,
                                              unsigned long long *msk, bool &bad) {
    const int lane = lane_id();
    for (int pb = a_lo; pb < a_hi; pb += WARP) {
        const int p = pb + lane;
        int lo = 0, hi = 0;
        if (p < a_hi) {
            const int k = __ldg(acol + p);
            lo = __ldg(tptr + k);
            hi = __ldg(tptr + k + 1);
            if (RESTRICT) {
                lo = lower_bound_i32(tcol, lo, hi, t0);
                hi = lower_bound_i32(tcol, lo, hi, t0 + len);
            }
        }
        const int n = hi - lo;
        const int incl = warp_incl_scan(n);
        const int total = __shfl_sync(FULL, incl, WARP - 1);
        if (total == 0) continue;
        const int excl = incl - n;
        int c_st = 0, c_d = 0;
        if (PACKED) {
            const unsigned ne = __ballot_sync(FULL, n > 0);
            const int nseg = __popc(ne);
            const int src = nth_set_bit(ne, min(lane, nseg - 1));
            const int st_src = __shfl_sync(FULL, excl, src);
            c_d = __shfl_sync(FULL, lo - excl, src);
            c_st = lane < nseg ? st_src : INT_MAX;
        }
        for (int f = first; f < total; f += stride * OR_U) {
            int tt[OR_U];
            unsigned long long mm[OR_U];
#pragma unroll
            for (int u = 0; u < OR_U; u++) {
                const int fu = f + u * stride;
                const int g = fu + lane;
                int idx;
                if (PACKED) {
                    const int before = __popc(__ballot_sync(FULL, c_st < fu));
                    const unsigned rel = (unsigned)(c_st - fu);
                    const unsigned sm = __reduce_or_sync(FULL, rel < 32u ? 1u << rel : 0u);
                    idx = g + __shfl_sync(FULL, c_d, before + __popc(sm & lanemask_le()) - 1);
                } else {
                    const int s = seg_of(incl, g);
                    idx = __shfl_sync(FULL, lo, s) + (g - __shfl_sync(FULL, excl, s));
                }
                tt[u] = INT_MIN;
                mm[u] = 0ull;
                if (g < total) {
                    tt[u] = __ldg(tcol + idx) - t0;
                    mm[u] = __ldg(tmask + idx);
                }
            }
#pragma unroll
            for (int u = 0; u < OR_U; u++) {
                if (tt[u] == INT_MIN) continue;
                if (tt[u] >= 0 && tt[u] < len) smem_or64(msk + tt[u], mm[u]);
                else bad = true;
            }
        }
    }
}

// Block-wide exclusive scans over one value per thread (blockDim.x == NT).
// s_tmp needs NT/32 + 1 entries.  Contains __syncthreads.
template <int NT, class T>
__device__ __forceinline__ T block_excl_sum(T v, T *s_tmp, T &total) {
    const int lane = lane_id(), w = threadIdx.x >> 5;
    T incl = warp_incl_scan(v);
    if (lane == 31) s_tmp[w] = incl;
    __syncthreads();
    if (w == 0) {
        T x = lane < (NT / 32) ? s_tmp[lane] : T(0);
        T xi = warp_incl_scan(x);
        if (lane < (NT / 32)) s_tmp[lane] = xi - x;
        if (lane == 31) s_tmp[NT / 32] = xi;
    }
    __syncthreads();
    total = s_tmp[NT / 32];
    T r = incl - v + s_tmp[w];
    __syncthreads();
    return r;
}

// One-barrier variants: the warp totals go to s_w (NT/32 entries) and every
// thread adds up the ones before its warp itself.  s_w must not be written
// again before the next block-wide barrier (use a separate array per scan).
template <int NT, class T>
__device__ __forceinline__ T block_excl_sum1(T v, T *s_w, T &total) {
    const int lane = lane_id(), w = threadIdx.x >> 5;
    const T incl = warp_incl_scan(v);
    if (lane == 31) s_w[w] = incl;
    __syncthreads();
    T off = T(0), tot = T(0);
#pragma unroll
    for (int j = 0; j < NT / 32; j++) {
        const T x = s_w[j];
        if (j < w) off += x;
        tot += x;
    }
    total = tot;
    return off + incl - v;
}

template <class T>
__device__ __forceinline__ T warp_incl_max(T v);

// exclusive max-scan with one barrier; threads before the first contribute `ident`
template <int NT, class T>
__device__ __forceinline__ T block_excl_max1(T v, T *s_w, T ident) {
    const int lane = lane_id(), w = threadIdx.x >> 5;
    const T incl = warp_incl_max(v);
    T ex = __shfl_up_sync(FULL, incl, 1);
    if (lane == 0) ex = ident;
    if (lane == 31) s_w[w] = incl;
    __syncthreads();
    for (int j = 0; j < w; j++) ex = max(ex, s_w[j]);
    return ex;
}

template <class T>
__device__ __forceinline__ T warp_incl_max(T v) {
    const int lane = lane_id();
#pragma unroll
    for (int d = 1; d < WARP; d <<= 1) {
        T o = __shfl_up_sync(FULL, v, d);
        if (lane >= d) v = max(v, o);
    }
    return v;
}

// exclusive max-scan; threads before the first contribute `ident`
template <int NT, class T>
__device__ __forceinline__ T block_excl_max(T v, T *s_tmp, T ident) {
    const int lane = lane_id(), w = threadIdx.x >> 5;
    T incl = warp_incl_max(v);
    T ex = __shfl_up_sync(FULL, incl, 1);
    if (lane == 0) ex = ident;
    if (lane == 31) s_tmp[w] = incl;
    __syncthreads();
    if (w == 0) {
        T x = lane < (NT / 32) ? s_tmp[lane] : ident;
        T xi = warp_incl_max(x);
        T xe = __shfl_up_sync(FULL, xi, 1);
        if (lane == 0) xe = ident;
        if (lane < (NT / 32)) s_tmp[lane] = xe;
    }
    __syncthreads();
    T r = max(ex, s_tmp[w]);
    __syncthreads();
    return r;
}

}  // namespace hsmu
