// CSR transpose on the device: B = A^T with the entries of every row of B in
// ascending column order (= ascending row of A), as the A*A^T products need.
//
// The reference transposes on the host before the product (csr2csc,
// src/mmio_highlevel.h:194, called from src/test.cu:40-56 for its AAT mode).
// Here the entries of A, already in (row, column) order, are sorted by
// column with a stable least-significant-digit radix sort (8-bit digits,
// only as many passes as the column count needs); stability keeps the rows
// ascending inside every column, so no per-row sort follows.  One pass:
//   k_tr_hist     one warp per tile of TR_TILE entries: digit histogram
//   scan          over hist[digit][tile] (digit-major), the global offsets
//   k_tr_scatter  one warp per tile: entries taken 32 at a time in order;
//                 lanes with the same digit rank themselves by lane order
//                 (__match_any_sync), a per-digit running count in shared
//                 memory carries the order across steps
// Row pointers of B come from the sorted column ids (first position of every
// column).  Everything is integer and data movement: bit-exact by design.
#include "hsmu_common.cuh"
#include "hsmu_kernels.h"

namespace hsmu {

constexpr int TR_TILE = 1024;   // entries per warp tile
constexpr int TR_WARPS = 8;     // warps per block
constexpr int TR_RADIX = 256;

// row id of every entry of A
__global__ void __launch_bounds__(256) k_tr_rows(int M, const int *__restrict__ rp, int *__restrict__ row) {
    const int lane = lane_id();
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = gw; i < M; i += nw)
        for (int e = rp[i] + lane; e < rp[i + 1]; e += WARP) row[e] = i;
}

__global__ void __launch_bounds__(TR_WARPS * 32) k_tr_hist(const int *__restrict__ key, int n, int shift,
                                                           int ntiles, int *__restrict__ hist) {
    __shared__ int s_h[TR_WARPS][TR_RADIX];
    const int lane = lane_id(), w = threadIdx.x >> 5;
    const int tile = blockIdx.x * TR_WARPS + w;
    for (int d = lane; d < TR_RADIX; d += WARP) s_h[w][d] = 0;
    __syncwarp();
    if (tile < ntiles) {
        const int lo = tile * TR_TILE, hi = min(n, lo + TR_TILE);
        for (int e = lo + lane; e < hi; e += WARP) atomicAdd(&s_h[w][(key[e] >> shift) & (TR_RADIX - 1)], 1);
        __syncwarp();
        for (int d = lane; d < TR_RADIX; d += WARP) hist[d * ntiles + tile] = s_h[w][d];
    }
}

__global__ void __launch_bounds__(TR_WARPS * 32) k_tr_scatter(const int *__restrict__ key, const int *__restrict__ row,
                                                              const double *__restrict__ val, int n, int shift,
                                                              int ntiles, const int *__restrict__ off,
                                                              int *__restrict__ okey, int *__restrict__ orow,
                                                              double *__restrict__ oval) {
    __shared__ int s_run[TR_WARPS][TR_RADIX];
    const int lane = lane_id(), w = threadIdx.x >> 5;
    const int tile = blockIdx.x * TR_WARPS + w;
    if (tile >= ntiles) return;  // whole warp: no warp-wide call follows for it
    for (int d = lane; d < TR_RADIX; d += WARP) s_run[w][d] = off[d * ntiles + tile];
    __syncwarp();
    const int lo = tile * TR_TILE, hi = min(n, lo + TR_TILE);
    for (int b = lo; b < hi; b += WARP) {
        const int e = b + lane;
        const bool v = e < hi;
        const int k = v ? key[e] : 0;
        const int d = v ? (k >> shift) & (TR_RADIX - 1) : TR_RADIX + lane;  // invalid lanes: own group
        const unsigned grp = __match_any_sync(FULL, d);
        if (v) {
            const int pos = s_run[w][d] + __popc(grp & lanemask_lt());
            okey[pos] = k;
            orow[pos] = row[e];
            oval[pos] = val[e];
        }
        __syncwarp();
        if (v && (grp & lanemask_lt()) == 0u) s_run[w][d] += __popc(grp);  // first lane of the group
        __syncwarp();
    }
}

// row pointers of B = A^T from the sorted column ids: rp[c] = first position of column c
__global__ void __launch_bounds__(256) k_tr_rowptr(const int *__restrict__ key, int n, int N, int *__restrict__ rp) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e <= n; e += (long long)gridDim.x * blockDim.x) {
        const int prev = e == 0 ? -1 : min(key[e - 1], N);
        const int cur = e == n ? N : min(key[e], N);
        for (int c = prev + 1; c <= cur; c++) rp[c] = (int)e;  // columns prev+1..cur start here
    }
}

int launch_transpose(const DevCSR &A, int *trp, int *tcol, double *tval, int *scratch_i, double *scratch_d,
                     int *hist, int *scan_tmp, long long *total64, Ctl *ctl, int nsm, cudaStream_t st) {
    const int n = (int)A.nnz;
    if (n == 0) {
        return (int)cudaMemsetAsync(trp, 0, sizeof(int) * ((size_t)A.N + 1), st);
    }
    // buffers: (key, row, val) in ping-pong pairs; pass 0 reads A's columns directly
    int *key0 = scratch_i, *row0 = scratch_i + n, *key1 = scratch_i + 2 * (size_t)n, *row1 = scratch_i + 3 * (size_t)n;
    double *val0 = scratch_d, *val1 = scratch_d + n;
    k_tr_rows<<<nsm * 8, 256, 0, st>>>(A.M, A.rp, row0);
    const int ntiles = (n + TR_TILE - 1) / TR_TILE;
    const int blocks = (ntiles + TR_WARPS - 1) / TR_WARPS;
    const int bits = A.N > 1 ? 32 - __builtin_clz((unsigned)(A.N - 1)) : 1;
    const int passes = (bits + 7) / 8;
    const int *skey = A.col;
    const int *srow = row0;
    const double *sval = A.val;
    for (int p = 0; p < passes; p++) {
        // destination alternates so that the last pass lands in (tcol <- rows, tval <- vals) + a key buffer
        const bool last = p == passes - 1;
        int *dkey = (p % 2 == 0) ? key1 : key0;
        int *drow = last ? tcol : ((p % 2 == 0) ? row1 : row0);
        double *dval = last ? tval : ((p % 2 == 0) ? val1 : val0);
        k_tr_hist<<<blocks, TR_WARPS * 32, 0, st>>>(skey, n, 8 * p, ntiles, hist);
        launch_scan(hist, hist + (size_t)TR_RADIX * ntiles + 1, TR_RADIX * ntiles, total64, scan_tmp, ctl, st);
        // (scan_tmp holds scan_tmp_ints(TR_RADIX * ntiles) ints)
        k_tr_scatter<<<blocks, TR_WARPS * 32, 0, st>>>(skey, srow, sval, n, 8 * p, ntiles,
                                                      hist + (size_t)TR_RADIX * ntiles + 1, dkey, drow, dval);
        skey = dkey;
        srow = drow;
        sval = dval;
    }
    k_tr_rowptr<<<nsm * 8, 256, 0, st>>>(skey, n, A.N, trp);
    return (int)cudaGetLastError();
}

// scratch sizes of launch_transpose for nnz entries
size_t transpose_scratch_ints(long long nnz) { return 4 * (size_t)(nnz > 0 ? nnz : 1); }
size_t transpose_scratch_doubles(long long nnz) { return 2 * (size_t)(nnz > 0 ? nnz : 1); }
size_t transpose_hist_ints(long long nnz) {
    const long long ntiles = (nnz + TR_TILE - 1) / TR_TILE;
    return 2 * (size_t)TR_RADIX * (size_t)(ntiles > 0 ? ntiles : 1) + 2;
}

}  // namespace hsmu
