// Per-row routines for rows with few intermediate products ("tiny" rows:
// at most TINY_MAX products), one thread per row.
//
// The AMG Galerkin operands (A*P: <= 7 products per row, P^T*(AP): <= 32)
// and the 2-D Laplacian (<= 25) consist of such rows only; a warp per row
// would leave most lanes idle.  A thread walks its row's products in the
// oracle's order (A entry, then B entry), keeping the distinct columns in a
// small sorted list (insertion), so the count pass and the fill pass need no
// B tiles and no sorting afterwards.  In the fill pass every product is added
// to its column's accumulator in that same order: 0.0 + p_1 + p_2 + ...
// (arithmetic per step as in hsmu_products.cuh), bit-identical to the host
// oracle.
//
// The per-thread lists live in shared memory laid out element-major
// ([TINY_MAX][threads]) so that neighbouring threads hit neighbouring banks.
//
// B's row k is given as entries brp[k] .. bre[k]-1 (bre = brp + 1 for a CSR
// row pointer).
#pragma once
#include "hsmu_products.cuh"

namespace hsmu {

constexpr int TINY_MAX = 32;

// A entries of a tiny row handled per batch: their column ids, B row bounds
// and first B entries are fetched in three rounds of independent loads
// before any of them is used (a thread would otherwise wait for ~3 dependent
// memory round trips per A entry)
constexpr int TINY_BATCH = 8;

template <bool NC, bool VALS>
struct TinyFetch {
    int qs[TINY_BATCH], qe[TINY_BATCH], j0[TINY_BATCH];
    double a[TINY_BATCH], b0[TINY_BATCH];

    __device__ __forceinline__ void load(int p0, int a_hi, const int *__restrict__ acol,
                                         const double *__restrict__ aval, const int *__restrict__ brp,
                                         const int *__restrict__ bre, const int *__restrict__ bcol,
                                         const double *__restrict__ bval) {
        int k[TINY_BATCH];
#pragma unroll
        for (int u = 0; u < TINY_BATCH; u++) {
            k[u] = p0 + u < a_hi ? ldx<NC>(acol + p0 + u) : -1;
            if (VALS) a[u] = p0 + u < a_hi ? ldx<NC>(aval + p0 + u) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < TINY_BATCH; u++) {
            qs[u] = qe[u] = 0;
            if (k[u] >= 0) {
                qs[u] = ldx<NC>(brp + k[u]);
                qe[u] = ldx<NC>(bre + k[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < TINY_BATCH; u++) {
            j0[u] = 0;
            b0[u] = 0.0;
            if (qs[u] < qe[u]) {
                j0[u] = ldx<NC>(bcol + qs[u]);
                if (VALS) b0[u] = ldx<NC>(bval + qs[u]);
            }
        }
    }
};

// number of distinct columns of row (a_lo..a_hi) of A*B; -1 if the row has
// more than TINY_MAX products (caller classified it wrongly).
template <bool NC = true>
__device__ __forceinline__ int tiny_row_count(int a_lo, int a_hi, const int *__restrict__ acol,
                                              const int *__restrict__ brp, const int *__restrict__ bre,
                                              const int *__restrict__ bcol, int *cols, int stride) {
    int n = 0, seen = 0;
    for (int p0 = a_lo; p0 < a_hi; p0 += TINY_BATCH) {
        TinyFetch<NC, false> F;
        F.load(p0, a_hi, acol, nullptr, brp, bre, bcol, nullptr);
#pragma unroll
        for (int u = 0; u < TINY_BATCH; u++) {
            for (int q = F.qs[u]; q < F.qe[u]; q++) {
                if (++seen > TINY_MAX) return -1;
                const int j = q == F.qs[u] ? F.j0[u] : ldx<NC>(bcol + q);
                int pos = n;
                while (pos > 0 && cols[(pos - 1) * stride] > j) pos--;
                if (pos > 0 && cols[(pos - 1) * stride] == j) continue;
                for (int t = n; t > pos; t--) cols[t * stride] = cols[(t - 1) * stride];
                cols[pos * stride] = j;
                n++;
            }
        }
    }
    return n;
}

// Builds the row's sorted distinct columns and their accumulated values in
// the thread's list (cols/acc, element stride `stride`, TINY_MAX entries) and
// returns its length; returns -1 (list contents undefined) when the row has
// more than `limit` products (limit <= TINY_MAX).
template <int AR, bool NC = true>
__device__ __forceinline__ int tiny_row_build(int a_lo, int a_hi, const int *__restrict__ acol,
                                              const double *__restrict__ aval, const int *__restrict__ brp,
                                              const int *__restrict__ bre, const int *__restrict__ bcol,
                                              const double *__restrict__ bval, int *cols, double *acc, int stride,
                                              int limit) {
    int n = 0, seen = 0;
    for (int p0 = a_lo; p0 < a_hi; p0 += TINY_BATCH) {
        TinyFetch<NC, true> F;
        F.load(p0, a_hi, acol, aval, brp, bre, bcol, bval);
#pragma unroll
        for (int u = 0; u < TINY_BATCH; u++) {
            const double a = F.a[u];
            for (int q = F.qs[u]; q < F.qe[u]; q++) {
                if (++seen > limit) return -1;
                const bool first = q == F.qs[u];
                const int j = first ? F.j0[u] : ldx<NC>(bcol + q);
                const double pr = term<AR>(a, first ? F.b0[u] : ldx<NC>(bval + q));
                int pos = n;
                while (pos > 0 && cols[(pos - 1) * stride] > j) pos--;
                if (pos > 0 && cols[(pos - 1) * stride] == j) {
                    acc[(pos - 1) * stride] = add_term<AR>(acc[(pos - 1) * stride], a, pr);
                    continue;
                }
                for (int t = n; t > pos; t--) {
                    cols[t * stride] = cols[(t - 1) * stride];
                    acc[t * stride] = acc[(t - 1) * stride];
                }
                cols[pos * stride] = j;
                acc[pos * stride] = add_term<AR>(0.0, a, pr);
                n++;
            }
        }
    }
    return n;
}

// copies a list built by tiny_row_build to out_col/out_val
__device__ __forceinline__ void tiny_row_write(const int *cols, const double *acc, int stride, int n,
                                               int *__restrict__ out_col, double *__restrict__ out_val) {
    for (int t = 0; t < n; t++) {
        out_col[t] = cols[t * stride];
        out_val[t] = acc[t * stride];
    }
}

// Fills the row's sorted columns and values at out_col/out_val and returns
// its nnz; returns -1 on an inconsistency (more than TINY_MAX products, or
// more than `cap` distinct columns).
template <int AR, bool NC = true>
__device__ __forceinline__ int tiny_row_fill(int a_lo, int a_hi, const int *__restrict__ acol,
                                             const double *__restrict__ aval, const int *__restrict__ brp,
                                             const int *__restrict__ bre, const int *__restrict__ bcol,
                                             const double *__restrict__ bval, int *cols, double *acc, int stride,
                                             int cap, int *__restrict__ out_col,
                                             double *__restrict__ out_val) {
    const int n = tiny_row_build<AR, NC>(a_lo, a_hi, acol, aval, brp, bre, bcol, bval, cols, acc, stride, TINY_MAX);
    if (n < 0 || n > cap) return -1;
    tiny_row_write(cols, acc, stride, n, out_col, out_val);
    return n;
}

// ---------------------------------------------------------------------------
// Warp-per-row routines on a dense span table, driven by B's entries (no B
// tiles): used by the batched engine, where B may be produced inside the same
// launch.  msk[] holds SPAN_T u64 masks, base[] SPAN_T ints, acc[] `cap`
// doubles, all private to the warp.

// first and last column of row (a_lo..a_hi) of A*B: min/max over the first /
// last entries of the referenced (sorted) B rows; returns products too.
template <bool NC = true>
__device__ __forceinline__ void warp_row_extent(int a_lo, int a_hi, const int *__restrict__ acol,
                                                const int *__restrict__ brp, const int *__restrict__ bre,
                                                const int *__restrict__ bcol, int &cmin, int &cmax, int &prod) {
    cmin = 0x7fffffff;
    cmax = -1;
    prod = 0;
    for (int p = a_lo + lane_id(); p < a_hi; p += WARP) {
        const int k = ldx<NC>(acol + p);
        const int s = ldx<NC>(brp + k), e = ldx<NC>(bre + k);
        if (e > s) {
            cmin = min(cmin, ldx<NC>(bcol + s));
            cmax = max(cmax, ldx<NC>(bcol + e - 1));
            prod += e - s;
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        cmin = min(cmin, __shfl_xor_sync(FULL, cmin, d));
        cmax = max(cmax, __shfl_xor_sync(FULL, cmax, d));
        prod += __shfl_xor_sync(FULL, prod, d);
    }
}

// OR the row's columns into msk[0..span) (tile t0 + i at msk[i]).  Without
// CLIP a column outside the span is an error (returns false); with CLIP each
// B row is first cut to the span's columns (two binary searches), so a wide
// row can be taken one column window at a time.
template <bool NC = true, bool CLIP = false>
__device__ __forceinline__ bool warp_row_masks(int a_lo, int a_hi, const int *__restrict__ acol,
                                               const int *__restrict__ brp, const int *__restrict__ bre,
                                               const int *__restrict__ bcol, int t0,
                                               int span, unsigned long long *msk) {
    for (int t = lane_id(); t < span; t += WARP) msk[t] = 0ull;
    __syncwarp();
    bool bad = false;
    const int c0 = CLIP ? t0 << 6 : 0;
    const int c1 = CLIP ? (int)min((long long)(t0 + span) << 6, (long long)INT_MAX) : 0;
    warp_walk_tiles<CLIP, NC>(a_lo, a_hi, 0, WARP, acol, brp, bre, bcol, c0, c1, [&](int q) {
        const int j = ldx<NC>(bcol + q);
        const int t = (j >> 6) - t0;
        if (t >= 0 && t < span) smem_setbit64(msk + t, j & 63);
        else bad = true;
    });
    __syncwarp();
    return !__any_sync(FULL, bad);
}

// nnz of the masks
__device__ __forceinline__ int warp_mask_count(const unsigned long long *msk, int span) {
    int c = 0;
    for (int t = lane_id(); t < span; t += WARP) c += popc64(msk[t]);
    return warp_sum(c);
}

// Given the row's masks: write its sorted columns to out_col, accumulate the
// products (oracle order) in acc and write the values to out_val.  nnz must
// equal the masks' popcount and be <= cap.  Returns false on inconsistency.
// CLIP: the masks cover one column window [t0*64, (t0+span)*64) of the row;
// each B row is cut to it, and the output is that window's part of the row.
template <int AR, bool NC = true, bool CLIP = false>
__device__ __forceinline__ bool warp_row_fill(int a_lo, int a_hi, const int *__restrict__ acol,
                                              const double *__restrict__ aval, const int *__restrict__ brp,
                                              const int *__restrict__ bre, const int *__restrict__ bcol,
                                              const double *__restrict__ bval, int t0, int span, const unsigned long long *msk, int *base,
                                              double *acc, int nnz, int *__restrict__ out_col,
                                              double *__restrict__ out_val) {
    const int lane = lane_id();
    const int per = (span + WARP - 1) / WARP;
    const int lo = min(span, lane * per), hi = min(span, lo + per);
    int sum = 0;
    for (int t = lo; t < hi; t++) sum += popc64(msk[t]);
    const int incl = warp_incl_scan(sum);
    if (__shfl_sync(FULL, incl, WARP - 1) != nnz) return false;
    int run = incl - sum;
    for (int t = lo; t < hi; t++) {
        unsigned long long m = msk[t];
        base[t] = run;
        int pos = run;
        const int cb = (t0 + t) << 6;
        run += popc64(m);
        while (m) {
            out_col[pos++] = cb + (__ffsll((long long)m) - 1);
            m &= m - 1ull;
        }
    }
    for (int q = lane; q < nnz; q += WARP) acc[q] = 0.0;
    __syncwarp();
    const int c0 = CLIP ? t0 << 6 : 0;
    const int c1 = CLIP ? (int)min((long long)(t0 + span) << 6, (long long)INT_MAX) : 0;
    auto seg = [&](int, int k, int &elo, int &ehi) {
        elo = ldx<NC>(brp + k);
        ehi = ldx<NC>(bre + k);
        if (CLIP) {
            elo = lower_bound_x<NC>(bcol, elo, ehi, c0);
            ehi = lower_bound_x<NC>(bcol, elo, ehi, c1);
        }
    };
    auto lookup = [&](int j) -> int {
        const int t = (j >> 6) - t0;
        if ((unsigned)t >= (unsigned)span) return -1;
        return tile_slot(msk[t], base[t], j);
    };
    bool bad = false;
    warp_accumulate<AR, NC>(a_lo, a_hi, acol, aval, brp, bcol, bval, seg, lookup, acc, bad);
    __syncwarp();
    for (int q = lane; q < nnz; q += WARP) out_val[q] = acc[q];
    __syncwarp();
    return !__any_sync(FULL, bad);
}

}  // namespace hsmu
