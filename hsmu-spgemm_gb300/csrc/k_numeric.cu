// Stage 5b: numeric phase, C values, one warp per window.
//
// GB300 counterpart of the HSMU accumulator k_formcval_shared_for_many_rows
// (src/compressed/compressed_Cval.cuh:1-69: binary search of the column in
// the row's sorted column list, then a shared-memory FP64 atomicAdd of
// aval*bval) and of the spECK dense accumulator used for rows with more than
// 4096 nnz (src/external/spECK/dense_acc.cu:2-267).
//
// Slot lookup is O(1): the window's columns are turned back into a dense
// per-tile table (u64 mask + first slot of the tile), so the slot of column
// j is base[t] + popc(mask[t] & ((1 << (j & 63)) - 1)) with t = (j >> 6) - t0.
//
// Accumulation order is deterministic and equals the oracle's: the products
// of the window are walked in the flat order (A entry, then B entry), 32 per
// step, one per lane; lanes that hit the same slot within a step
// (__match_any_sync) add in lane order, which is A-entry order, so every
// C entry is 0.0 + p_1 + p_2 + ... in the order of A(i,:) -- the same sum,
// bit for bit, as the host Gustavson oracle.  Each product is rounded before
// the add (no FMA contraction), as in the reference (`aval * bval` then
// atomicAdd).  No floating-point atomics are used.
//
// GB300 executes FP64 at ~1.6 lane-ops/clk/SM, two orders of magnitude below
// its int32 rate, so this kernel is bound by the FP64 pipe, not by HBM.
#include "hsmu_block.cuh"
#include "hsmu_kernels.h"

namespace hsmu {

constexpr int NUM_WARPS = 8;

struct NumSmem {
    unsigned long long msk[SPAN_T];
    int base[SPAN_T];
    double acc[WIN_CAP];
};

__global__ void __launch_bounds__(NUM_WARPS * 32) k_numeric(const int *__restrict__ arp, const int *__restrict__ acol,
                                                            const double *__restrict__ aval,
                                                            const int *__restrict__ brp, const int *__restrict__ bcol,
                                                            const double *__restrict__ bval,
                                                            const int *__restrict__ crp, const int *__restrict__ ccol,
                                                            double *__restrict__ cval, const Window *__restrict__ win,
                                                            int win_cap, Ctl *ctl) {
    extern __shared__ unsigned long long s_dyn[];
    const int lane = lane_id(), w = threadIdx.x >> 5;
    NumSmem &S = reinterpret_cast<NumSmem *>(s_dyn)[w];
    const int nwin = min(ctl->win_count, win_cap);
    const int gw = blockIdx.x * NUM_WARPS + w;
    const int nw = gridDim.x * NUM_WARPS;
    bool bad = false;
    for (int wi = gw; wi < nwin; wi += nw) {
        const Window W = win[wi];
        const int row = W.row, s0 = W.s0, cnt = W.cnt, t0 = W.t0;
        const int c_lo = ccol[s0], c_hi = ccol[s0 + cnt - 1];
        const int span = (c_hi >> 6) - t0 + 1;
        if (cnt <= 0 || cnt > WIN_CAP || span <= 0 || span > SPAN_T || (c_lo >> 6) != t0) {
            bad = true;
            continue;
        }
        const bool full = (s0 == crp[row]) && (cnt == crp[row + 1] - s0);
        for (int t = lane; t < span; t += WARP) S.msk[t] = 0ull;
        for (int s = lane; s < cnt; s += WARP) S.acc[s] = 0.0;
        __syncwarp();
        for (int s = lane; s < cnt; s += WARP) {
            const int c = ccol[s0 + s];
            const int t = (c >> 6) - t0;
            if (c >= 0 && t >= 0 && t < span) atomicOr(&S.msk[t], 1ull << (c & 63));
            else bad = true;
        }
        __syncwarp();
        {
            const int per = (span + WARP - 1) / WARP;
            const int lo = min(span, lane * per), hi = min(span, lo + per);
            int sum = 0;
            for (int t = lo; t < hi; t++) sum += popc64(S.msk[t]);
            int run = warp_incl_scan(sum) - sum;
            for (int t = lo; t < hi; t++) {
                S.base[t] = run;
                run += popc64(S.msk[t]);
            }
        }
        __syncwarp();
        const int a_lo = arp[row], a_hi = arp[row + 1];
        for (int pb = a_lo; pb < a_hi; pb += WARP) {
            const int p = pb + lane;
            int elo = 0, ehi = 0;
            double a = 0.0;
            if (p < a_hi) {
                const int k = __ldg(acol + p);
                a = __ldg(aval + p);
                elo = __ldg(brp + k);
                ehi = __ldg(brp + k + 1);
                if (!full) {
                    elo = lower_bound_i32(bcol, elo, ehi, c_lo);
                    ehi = lower_bound_i32(bcol, elo, ehi, c_hi + 1);
                }
            }
            const int len = ehi - elo;
            const int incl = warp_incl_scan(len);
            const int total = __shfl_sync(FULL, incl, WARP - 1);
            const int excl = incl - len;
            for (int f = 0; f < total; f += WARP) {
                const int g = f + lane;
                const bool gv = g < total;
                const int sg = seg_of(incl, g);
                const int e = __shfl_sync(FULL, elo, sg) + (g - __shfl_sync(FULL, excl, sg));
                const double as = __shfl_sync(FULL, a, sg);
                int slot = -1 - lane;
                double prod = 0.0;
                if (gv) {
                    const int j = __ldg(bcol + e);
                    const double b = __ldg(bval + e);
                    prod = __dmul_rn(as, b);
                    const int tt = (j >> 6) - t0;
                    if (tt >= 0 && tt < span) {
                        const unsigned long long m = S.msk[tt];
                        const int bit = j & 63;
                        if ((m >> bit) & 1ull) slot = S.base[tt] + rank64(m, bit);
                        else bad = true;
                    } else {
                        bad = true;
                    }
                }
                const bool act = slot >= 0;
                const unsigned grp = __match_any_sync(FULL, slot);
                const int rank = __popc(grp & lanemask_lt());
                const int maxr = (int)__reduce_max_sync(FULL, act ? (unsigned)rank : 0u);
                for (int rr = 0; rr <= maxr; rr++) {
                    if (act && rank == rr) S.acc[slot] = __dadd_rn(S.acc[slot], prod);
                    __syncwarp();
                }
            }
        }
        __syncwarp();
        for (int s = lane; s < cnt; s += WARP) cval[s0 + s] = S.acc[s];
        __syncwarp();
    }
    if (__any_sync(FULL, bad) && lane == 0) set_err(&ctl->err, DERR_INTERNAL);
}

void launch_numeric(const DevCSR &A, const DevCSR &B, const int *crp, const int *ccol, double *cval,
                    const Window *win, long long win_cap, Ctl *ctl, int arith, int nsm, cudaStream_t st) {
    (void)arith;
    k_numeric<<<nsm * 2, NUM_WARPS * 32, NUM_WARPS * sizeof(NumSmem), st>>>(A.rp, A.col, A.val, B.rp, B.col, B.val,
                                                                            crp, ccol, cval, win, (int)win_cap, ctl);
}

int configure_numeric() {
    return (int)cudaFuncSetAttribute(k_numeric, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     NUM_WARPS * (int)sizeof(NumSmem));
}

}  // namespace hsmu
