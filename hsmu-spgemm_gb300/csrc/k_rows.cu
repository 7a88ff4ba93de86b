// Stage 2: per-row bounds + row binning, and the device exclusive scan.
//
// Bounds: for every A row, the number of intermediate products
// sum_{k in A(i,:)} nnz(B(k,:)) (64-bit; the reference counts it on the host,
// src/NHC_spgemm.cuh:37-42, and bounds C tiles per row with k_compute_flop,
// src/small/mask.cuh:14-51) and the exact first/last C tile of the row (the
// min/max over the 64-column tiles of every referenced B row's first and last
// column -- read from B itself, so this pass does not wait for B's tiles and
// runs beside their construction).  The tile span decides the row class
// (one warp with a dense span table, or one CTA with a chunked table), which
// replaces the reference's host-round-trip binning (src/bining.cuh:1-207):
// rows are binned on the device by a stable compaction (count per 32-row
// chunk, scan, emit), so every bin lists its rows in ascending order and the
// rows of a row panel are one contiguous slice of each bin.
//
// Scan: three launches (block sums, scan of block sums, block scans), 64-bit
// running totals, int32 output; replaces cub::DeviceScan::ExclusiveSum plus
// the full-array D2H copies of the reference
// (src/compressed/compressed_tileOR.cuh:620-622).
#include <climits>

#include "hsmu_common.cuh"
#include "hsmu_kernels.h"
#include "hsmu_rowops.cuh"

namespace hsmu {

template <int G>
__global__ void __launch_bounds__(256) k_bounds(int M, const int *__restrict__ arp, const int *__restrict__ acol,
                                                const int *__restrict__ brp, const int *__restrict__ bcol, int N,
                                                RowInfo ri, Ctl *ctl) {
    constexpr int RPB = 256 / G;  // rows per block iteration
    __shared__ int s_cnt[NBIN];
    const int sub = threadIdx.x & (G - 1);
    const int rloc = threadIdx.x / G;
    unsigned long long my_prod = 0, my_wb = 0, my_cb = 0, my_cbd = 0, my_wdp = 0, my_span = 0;
    if (threadIdx.x < NBIN) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    for (int rb = blockIdx.x * RPB; rb < M; rb += gridDim.x * RPB) {
        const int i = rb + rloc;
        long long prod = 0;
        int tmin = INT_MAX, tmax = -1;
        if (i < M) {
            for (int p = arp[i] + sub; p < arp[i + 1]; p += G) {
                const int k = __ldg(acol + p);
                const int bs = __ldg(brp + k), be = __ldg(brp + k + 1);
                prod += be - bs;
                if (be > bs) {
                    tmin = min(tmin, __ldg(bcol + bs) >> 6);
                    tmax = max(tmax, __ldg(bcol + be - 1) >> 6);
                }
            }
        }
#pragma unroll
        for (int d = G / 2; d > 0; d >>= 1) {
            prod += __shfl_xor_sync(FULL, prod, d, G);
            tmin = min(tmin, __shfl_xor_sync(FULL, tmin, d, G));
            tmax = max(tmax, __shfl_xor_sync(FULL, tmax, d, G));
        }
        if (i < M && sub == 0) {
            ri.prod[i] = prod;
            ri.tmin[i] = tmin;
            ri.tmax[i] = tmax;
            int bin = -1;
            if (prod == 0) {
                ri.cnnz[i] = 0;
            } else {
                const int span = tmax - tmin + 1;
                bin = prod <= TINY_MAX ? BIN_TINY : (span <= SPAN_T ? BIN_DS : BIN_L);
                atomicAdd(&s_cnt[bin], 1);
                my_prod += (unsigned long long)prod;
                const long long cap = prod < (long long)N ? prod : (long long)N;
                // windows per row <= slot cuts + tile-rank cuts + span cuts + 1
                const long long tl = cap < (long long)span ? cap : (long long)span;
                const unsigned long long wb = (unsigned long long)(cap / WIN_CUT + tl / WIN_TCAP + (span - 1) / WIN_SPAN + 1);
                my_wb += wb;
                // rows that can reach the window pass: the large class, and warp rows above FUSE_CAP
                if (bin == BIN_L) {
                    my_cb += wb * (unsigned long long)(arp[i + 1] - arp[i]);
                    my_span += (unsigned long long)span;
                }
                if (bin == BIN_DS && prod > FUSE_CAP) {
                    my_cbd += wb * (unsigned long long)(arp[i + 1] - arp[i]);
                    my_wdp += (unsigned long long)prod;
                }
            }
            ri.cls[i] = (signed char)bin;
        }
    }
    __syncthreads();
    if (threadIdx.x < NBIN && s_cnt[threadIdx.x]) atomicAdd(&ctl->bin_count[threadIdx.x], s_cnt[threadIdx.x]);
    my_prod = warp_sum(my_prod);
    my_wb = warp_sum(my_wb);
    my_cb = warp_sum(my_cb);
    my_cbd = warp_sum(my_cbd);
    my_wdp = warp_sum(my_wdp);
    my_span = warp_sum(my_span);
    if (lane_id() == 0) {
        if (my_wdp) atomicAdd(&ctl->wide_ds_prod, my_wdp);
        if (my_span) atomicAdd(reinterpret_cast<unsigned long long *>(&ctl->span_tiles), my_span);
        if (my_prod) atomicAdd(&ctl->products, my_prod);
        if (my_wb) atomicAdd(&ctl->win_bound, my_wb);
        if (my_cb) atomicAdd(&ctl->cur_bound, my_cb);
        if (my_cbd) atomicAdd(&ctl->cur_bound_ds, my_cbd);
    }
}

// stable binning: rows of each class per 32-row chunk (warp per chunk) ...
__global__ void __launch_bounds__(256) k_bin_count(int M, const signed char *__restrict__ cls, int *__restrict__ cnt) {
    const int nch = (M + WARP - 1) / WARP;
    const int lane = lane_id();
    for (int c = (blockIdx.x * blockDim.x + threadIdx.x) / WARP; c < nch; c += gridDim.x * blockDim.x / WARP) {
        const int i = c * WARP + lane;
        const int b = i < M ? cls[i] : -1;
#pragma unroll
        for (int k = 0; k < NBIN; k++) {
            const int n = __popc(__ballot_sync(FULL, b == k));
            if (lane == k) cnt[k * nch + c] = n;
        }
    }
}

// ... then, after the scan of those counts, every row at its place in its bin
__global__ void __launch_bounds__(256) k_bin_emit(int M, const signed char *__restrict__ cls,
                                                  const int *__restrict__ off, int *__restrict__ bins) {
    const int nch = (M + WARP - 1) / WARP;
    const int lane = lane_id();
    for (int c = (blockIdx.x * blockDim.x + threadIdx.x) / WARP; c < nch; c += gridDim.x * blockDim.x / WARP) {
        const int i = c * WARP + lane;
        const int b = i < M ? cls[i] : -1;
#pragma unroll
        for (int k = 0; k < NBIN; k++) {
            const unsigned m = __ballot_sync(FULL, b == k);
            if (b == k) bins[(size_t)k * M + (off[k * nch + c] - off[k * nch]) + __popc(m & lanemask_lt())] = i;
        }
    }
}

size_t bin_scratch_ints(int M) { return (size_t)NBIN * ((M + WARP - 1) / WARP) * 2 + 2; }

void launch_bounds(const DevCSR &A, const DevCSR &B, RowInfo ri, Ctl *ctl, int grid, int *scan_tmp, cudaStream_t st) {
    const double avg = A.M ? (double)A.nnz / A.M : 0.0;
    if (avg <= 6)
        k_bounds<4><<<grid, 256, 0, st>>>(A.M, A.rp, A.col, B.rp, B.col, B.N, ri, ctl);
    else if (avg <= 12)
        k_bounds<8><<<grid, 256, 0, st>>>(A.M, A.rp, A.col, B.rp, B.col, B.N, ri, ctl);
    else if (avg <= 24)
        k_bounds<16><<<grid, 256, 0, st>>>(A.M, A.rp, A.col, B.rp, B.col, B.N, ri, ctl);
    else
        k_bounds<32><<<grid, 256, 0, st>>>(A.M, A.rp, A.col, B.rp, B.col, B.N, ri, ctl);
    const int nch = (A.M + WARP - 1) / WARP;
    int *cnt = ri.bin_cnt, *off = ri.bin_cnt + (size_t)NBIN * nch + 1;
    k_bin_count<<<grid, 256, 0, st>>>(A.M, ri.cls, cnt);
    launch_scan(cnt, off, NBIN * nch, &ctl->binned, scan_tmp, ctl, st);
    k_bin_emit<<<grid, 256, 0, st>>>(A.M, ri.cls, off, ri.bins);
}

// products of every PROD_CHUNK consecutive rows: one warp per chunk (the host
// orders its row panels by them)
__global__ void __launch_bounds__(256) k_chunk_prod(int M, const long long *__restrict__ prod,
                                                    long long *__restrict__ out) {
    static_assert(PROD_CHUNK == 2 * WARP, "two rows per lane");
    const int nch = (M + PROD_CHUNK - 1) / PROD_CHUNK;
    const int lane = lane_id();
    for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < nch; c += (gridDim.x * blockDim.x) >> 5) {
        const int r0 = c * PROD_CHUNK + lane, r1 = r0 + WARP;
        long long v = (r0 < M ? prod[r0] : 0ll) + (r1 < M ? prod[r1] : 0ll);
        v = warp_sum(v);
        if (lane == 0) out[c] = v;
    }
}

void launch_chunk_prod(int M, const long long *prod, long long *out, int grid, cudaStream_t st) {
    if (M > 0) k_chunk_prod<<<grid, 256, 0, st>>>(M, prod, out);
}

// ---------------------------------------------------------------- scan
constexpr int SCAN_T = 256;
constexpr int SCAN_IPT = 8;
constexpr int SCAN_ITEMS = SCAN_T * SCAN_IPT;

// exclusive block scan of one long long per thread; returns block total
__device__ __forceinline__ long long block_excl_scan(long long v, long long *s_warp, long long &total) {
    const int lane = lane_id(), w = threadIdx.x >> 5;
    long long incl = warp_incl_scan(v);
    if (lane == 31) s_warp[w] = incl;
    __syncthreads();
    if (w == 0) {
        long long x = lane < (SCAN_T / 32) ? s_warp[lane] : 0;
        long long xi = warp_incl_scan(x);
        if (lane < (SCAN_T / 32)) s_warp[lane] = xi - x;
        if (lane == 31) s_warp[SCAN_T / 32] = xi;
    }
    __syncthreads();
    total = s_warp[SCAN_T / 32];
    long long r = incl - v + s_warp[w];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(SCAN_T) k_scan_sums(const int *__restrict__ in, int n, long long *bsum) {
    __shared__ long long s_warp[SCAN_T / 32 + 1];
    const long long base = (long long)blockIdx.x * SCAN_ITEMS + threadIdx.x * SCAN_IPT;
    long long v = 0;
#pragma unroll
    for (int j = 0; j < SCAN_IPT; j++)
        if (base + j < n) v += in[base + j];
    long long tot;
    block_excl_scan(v, s_warp, tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(SCAN_T) k_scan_top(long long *bsum, int nb, long long *total64) {
    __shared__ long long s_warp[SCAN_T / 32 + 1];
    long long carry = 0;
    for (int b0 = 0; b0 < nb; b0 += SCAN_T) {
        const int b = b0 + threadIdx.x;
        long long v = b < nb ? bsum[b] : 0;
        long long tot;
        long long ex = block_excl_scan(v, s_warp, tot);
        if (b < nb) bsum[b] = ex + carry;
        carry += tot;
    }
    if (threadIdx.x == 0) *total64 = carry;
}

// in and out may be the same array (in-place scan; the allocation-free tile conversion and the
// AMG generators rely on it), so neither is __restrict__: every thread loads its SCAN_IPT items
// into registers before the block scan's barriers and afterwards stores only those same items,
// blocks cover disjoint ranges, and out[n] lies past every item read.
__global__ void __launch_bounds__(SCAN_T) k_scan_out(const int *in, int *out, int n,
                                                     const long long *__restrict__ boff, const long long *total64,
                                                     Ctl *ctl) {
    __shared__ long long s_warp[SCAN_T / 32 + 1];
    const long long base = (long long)blockIdx.x * SCAN_ITEMS + threadIdx.x * SCAN_IPT;
    int vals[SCAN_IPT];
    long long v = 0;
#pragma unroll
    for (int j = 0; j < SCAN_IPT; j++) {
        vals[j] = base + j < n ? in[base + j] : 0;
        v += vals[j];
    }
    long long tot;
    long long ex = block_excl_scan(v, s_warp, tot) + boff[blockIdx.x];
    const bool ovf = *total64 > (long long)INT_MAX;
#pragma unroll
    for (int j = 0; j < SCAN_IPT; j++) {
        if (base + j < n) out[base + j] = ovf ? 0 : (int)ex;
        ex += vals[j];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        out[n] = ovf ? 0 : (int)*total64;
        if (ovf) set_err(&ctl->err, DERR_OVERFLOW);
    }
}

__global__ void __launch_bounds__(SCAN_T) k_scan_out64(const int *__restrict__ in, long long *__restrict__ out, int n,
                                                       const long long *__restrict__ boff,
                                                       const long long *total64) {
    __shared__ long long s_warp[SCAN_T / 32 + 1];
    const long long base = (long long)blockIdx.x * SCAN_ITEMS + threadIdx.x * SCAN_IPT;
    int vals[SCAN_IPT];
    long long v = 0;
#pragma unroll
    for (int j = 0; j < SCAN_IPT; j++) {
        vals[j] = base + j < n ? in[base + j] : 0;
        v += vals[j];
    }
    long long tot;
    long long ex = block_excl_scan(v, s_warp, tot) + boff[blockIdx.x];
#pragma unroll
    for (int j = 0; j < SCAN_IPT; j++) {
        if (base + j < n) out[base + j] = ex;
        ex += vals[j];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = *total64;
}

void launch_scan64(const int *in, long long *out, int n, long long *total64, int *tmp, cudaStream_t st) {
    const int nb = n > 0 ? (n + SCAN_ITEMS - 1) / SCAN_ITEMS : 1;
    long long *bsum = reinterpret_cast<long long *>(tmp);
    k_scan_sums<<<nb, SCAN_T, 0, st>>>(in, n, bsum);
    k_scan_top<<<1, SCAN_T, 0, st>>>(bsum, nb, total64);
    k_scan_out64<<<nb, SCAN_T, 0, st>>>(in, out, n, bsum, total64);
}

size_t scan_tmp_ints(int n) {
    const int nb = (n + SCAN_ITEMS - 1) / SCAN_ITEMS;
    return (size_t)(nb > 0 ? nb : 1) * 2 + 2;
}

void launch_scan(const int *in, int *out, int n, long long *total64, int *tmp, Ctl *ctl, cudaStream_t st) {
    const int nb = n > 0 ? (n + SCAN_ITEMS - 1) / SCAN_ITEMS : 1;
    long long *bsum = reinterpret_cast<long long *>(tmp);
    k_scan_sums<<<nb, SCAN_T, 0, st>>>(in, n, bsum);
    k_scan_top<<<1, SCAN_T, 0, st>>>(bsum, nb, total64);
    k_scan_out<<<nb, SCAN_T, 0, st>>>(in, out, n, bsum, total64, ctl);
}

}  // namespace hsmu
