// Stage 1: B (CSR, sorted rows) -> 64-column bit tiles.
//
// GB300 counterpart of the reference's Initialize_compressed_mask64_matrix
// (src/compressed/compressed_mask64.cuh:343-424: compute_tile64_nums :61-152,
// k_compute_flop, the CUB scan, compute_tile64_col :153-246 and
// compute_tile64_mask_num :248-342).  The reference builds shared-memory
// bitmaps per row partition, copies tile_ptr to the host and partitions on
// the host; here one warp walks each sorted B row 32 entries at a time: a
// tile starts where (col >> 6) changes (ballot + popc), and the tile's u64
// mask is a segmented OR over the lanes of the tile (5 shuffle steps).  Two
// launches (count, fill) around a device scan; no host round trip; tile
// columns come out sorted, and each tile also records the CSR offset of its
// first entry (tile_off) so the numeric phase can jump straight to it.
#include "hsmu_common.cuh"
#include "hsmu_kernels.h"

namespace hsmu {

template <bool FILL>
__global__ void __launch_bounds__(256) k_tiles(int K, const int *__restrict__ brp, const int *__restrict__ bcol,
                                               int N, int *__restrict__ tcnt_or_ptr, int *__restrict__ tcol,
                                               unsigned long long *__restrict__ tmask, int *__restrict__ toff,
                                               int validate, Ctl *ctl) {
    const int lane = lane_id();
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int k = gw; k < K; k += nw) {
        const int s = brp[k], e = brp[k + 1];
        int run = FILL ? tcnt_or_ptr[k] : 0;  // output position (FILL) / count
        bool have_pend = false;
        int pend_t = -1, pend_off = 0;
        unsigned long long pend_m = 0;
        int prev_col = -1;
        bool bad = false;
        for (int base = s; base < e; base += WARP) {
            const int idx = base + lane;
            const bool valid = idx < e;
            const int c = valid ? __ldg(bcol + idx) : 0;
            if (validate) {
                int cp = __shfl_up_sync(FULL, c, 1);
                if (lane == 0) cp = prev_col;
                if (valid && (c <= cp || c < 0 || c >= N)) bad = true;
                prev_col = __shfl_sync(FULL, c, WARP - 1);
            }
            const int t = c >> 6;
            int tp = __shfl_up_sync(FULL, t, 1);
            if (lane == 0) tp = have_pend ? pend_t : -1;
            const bool head = valid && (t != tp);
            const unsigned heads = __ballot_sync(FULL, head);
            const int nvalid = min(WARP, e - base);
            if (!FILL) {
                run += __popc(heads);
                pend_t = __shfl_sync(FULL, t, nvalid - 1);  // tile open at the end of this chunk
                have_pend = true;
                continue;
            }
            unsigned above = heads & ~((2u << lane) - 1u);
            if (lane == 31) above = 0;
            const int seg_end = above ? (__ffs(above) - 2) : (nvalid - 1);
            unsigned long long v = valid ? (1ull << (c & 63)) : 0ull;
#pragma unroll
            for (int d = 1; d < WARP; d <<= 1) {
                unsigned long long o = __shfl_down_sync(FULL, v, d);
                if (lane + d <= seg_end) v |= o;
            }
            const unsigned long long lane0_or = __shfl_sync(FULL, v, 0);
            if (have_pend) {
                if (!(heads & 1u)) pend_m |= lane0_or;  // lane 0 continues the pending tile
                if (heads) {
                    if (lane == 0) {
                        tcol[run] = pend_t;
                        tmask[run] = pend_m;
                        toff[run] = pend_off;
                    }
                    run++;
                    have_pend = false;
                }
            }
            if (heads) {
                const int last = 31 - __clz(heads);
                if (head && lane != last) {
                    const int pos = run + __popc(heads & lanemask_lt());
                    tcol[pos] = t;
                    tmask[pos] = v;
                    toff[pos] = idx;
                }
                run += __popc(heads) - 1;
                pend_t = __shfl_sync(FULL, t, last);
                pend_m = __shfl_sync(FULL, v, last);
                pend_off = base + last;
                have_pend = true;
            }
        }
        if (FILL) {
            if (have_pend && lane == 0) {
                tcol[run] = pend_t;
                tmask[run] = pend_m;
                toff[run] = pend_off;
            }
        } else {
            if (lane == 0) tcnt_or_ptr[k] = run;
        }
        if (validate && __any_sync(FULL, bad) && lane == 0) set_err(&ctl->err, DERR_UNSORTED);
    }
}

void launch_tiles_count(const DevCSR &B, int *tcnt, int validate, Ctl *ctl, int grid, cudaStream_t st) {
    k_tiles<false><<<grid, 256, 0, st>>>(B.M, B.rp, B.col, B.N, tcnt, nullptr, nullptr, nullptr, validate, ctl);
}

void launch_tiles_fill(const DevCSR &B, const int *tptr, int *tcol, unsigned long long *tmask, int *toff, Ctl *ctl,
                       int grid, cudaStream_t st) {
    k_tiles<true><<<grid, 256, 0, st>>>(B.M, B.rp, B.col, B.N, const_cast<int *>(tptr), tcol, tmask, toff, 0, ctl);
}

// Validation of A: sorted, unique, in-range columns (one warp per row).
__global__ void __launch_bounds__(256) k_validate(int M, const int *__restrict__ rp, const int *__restrict__ col,
                                                  int N, long long nnz, Ctl *ctl) {
    const int lane = lane_id();
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    bool bad = false;
    for (int i = gw; i < M; i += nw) {
        const int s = rp[i], e = rp[i + 1];
        if (s > e || s < 0 || e > nnz) { bad = true; continue; }
        int prev = -1;
        for (int base = s; base < e; base += WARP) {
            const int idx = base + lane;
            const bool valid = idx < e;
            const int c = valid ? col[idx] : 0;
            int cp = __shfl_up_sync(FULL, c, 1);
            if (lane == 0) cp = prev;
            if (valid && (c <= cp || c < 0 || c >= N)) bad = true;
            prev = __shfl_sync(FULL, c, WARP - 1);
        }
    }
    if (bad) set_err(&ctl->err, DERR_UNSORTED);
}

void launch_validate(const DevCSR &A, Ctl *ctl, int grid, cudaStream_t st) {
    k_validate<<<grid, 256, 0, st>>>(A.M, A.rp, A.col, A.N, A.nnz, ctl);
}

}  // namespace hsmu
