// The product loop shared by the fused row kernel (k_struct_ds) and the
// window kernel (k_numeric): accumulate a_ik * b_kj into a shared-memory
// accumulator for one C row (or one window of it), in the oracle's order.
//
// Order: for each C entry the products are added as 0.0 + p_1 + p_2 + ...
// in A(i,:)'s storage order, exactly like the host Gustavson oracle, so
// results are bit-identical to it in each arithmetic mode (AR_RN: every
// p = a*b rounded before the add, as the reference does; AR_FMA: each step
// one fused multiply-add).
//
// The A entries are taken 32 at a time (one per lane); seg(p) gives the B
// entry range [elo, ehi) that A entry p contributes to this accumulator.
//   * long B segments (average >= LONG_SEG_MIN entries; callers may turn this
//     path off): one segment at a time, in chunks of up to LU steps of 32
//     entries.  Entries of one B row have distinct columns, so a chunk has no
//     slot conflicts and only a change of segment needs a warp sync.  The
//     next chunk's B loads are issued before the current chunk's
//     multiply/lookup/add (software pipeline).
//   * otherwise: the flat sequence of (A entry, B entry) items, 32 per step.
//     The non-empty segments are packed into lanes; one OR-reduction per step
//     marks the segment starts inside it, so every lane gets its segment from
//     a popcount.  A step inside one segment has distinct slots; lanes of a
//     step spanning several segments that hit the same slot add in lane order
//     = A-entry order (found by __match_any_sync, or with TAG by stamping lane
//     ids into a byte per slot and matching only the lanes that collide).
#pragma once
#include "hsmu_block.cuh"
#include "hsmu_dmul.cuh"

namespace hsmu {

// Arithmetic of one accumulation step c <- c + a*b (hsmu_opts.arith):
//   AR_RN   (0) product rounded, then added: RN(c + RN(a*b));
//   AR_FMA  (1) fused, one rounding per product: RN(c + a*b) -- one FP64
//               pipe operation per product instead of two;
//   AR_IMUL (2) as AR_RN, with the product formed exactly on the integer pipe.
// term() is what can be computed before the accumulator slot is known;
// add_term() folds it into the accumulator.
enum Arith { AR_RN = 0, AR_FMA = 1, AR_IMUL = 2 };

template <int AR>
__device__ __forceinline__ double term(double a, double b) {
    if (AR == AR_FMA) return b;
    if (AR == AR_IMUL) return dmul_int(a, b);
    return __dmul_rn(a, b);
}

template <int AR>
__device__ __forceinline__ double add_term(double c, double a, double t) {
    if (AR == AR_FMA) return __fma_rn(a, t, c);
    return __dadd_rn(c, t);
}

// steps of 32 B entries per chunk of the long-segment path
constexpr int LU = 3;
// a group of A entries takes the long-segment path when its non-empty
// segments average at least this many B entries (measured: the flat path
// is as fast below it, e.g. on power-law rows)
constexpr int LONG_SEG_MIN = 64;

// SegFn:    void(int p, int k, int &elo, int &ehi)  -- called for valid lanes
// LookupFn: int(int j) -> slot in acc, or -1 if j is not in the accumulator
// PG: load the next group of 32 A entries before processing the current one
// (for rows with many A entries; costs registers in the short-row kernels)
// TAG: `tag` is a byte per accumulator slot (any contents), used to find the
// lanes of a step that share a slot; without it every multi-entry step runs
// a full-warp match.
// LONG: groups with long segments take the long-segment path (else every group
// runs flat, where a step inside one segment needs no conflict test either).
template <int AR, bool NC = true, bool PG = false, bool TAG = false, bool LONG = true, class SegFn,
          class LookupFn>
__device__ __forceinline__ void warp_accumulate(int a_lo, int a_hi, const int *__restrict__ acol,
                                                const double *__restrict__ aval, const int *__restrict__ brp,
                                                const int *__restrict__ bcol, const double *__restrict__ bval,
                                                SegFn seg, LookupFn lookup, double *acc, bool &bad,
                                                unsigned char *tag = nullptr) {
    const int lane = lane_id();
    // A entries 32 at a time (PG: the next group's entries and segments are
    // loaded before the current group is processed)
    int n_elo = 0, n_ehi = 0;
    double n_a = 0.0;
    if (PG && a_lo + lane < a_hi) {
        n_a = ldx<NC>(aval + a_lo + lane);
        seg(a_lo + lane, ldx<NC>(acol + a_lo + lane), n_elo, n_ehi);
    }
    for (int pb = a_lo; pb < a_hi; pb += WARP) {
        int elo = 0, ehi = 0;
        double a = 0.0;
        if (PG) {
            elo = n_elo;
            ehi = n_ehi;
            a = n_a;
            n_elo = n_ehi = 0;
            n_a = 0.0;
            if (pb + WARP + lane < a_hi) {
                const int pn = pb + WARP + lane;
                n_a = ldx<NC>(aval + pn);
                seg(pn, ldx<NC>(acol + pn), n_elo, n_ehi);
            }
        } else if (pb + lane < a_hi) {
            a = ldx<NC>(aval + pb + lane);
            seg(pb + lane, ldx<NC>(acol + pb + lane), elo, ehi);
        }
        const int len = ehi - elo;
        const int incl = warp_incl_scan(len);
        const int total = __shfl_sync(FULL, incl, WARP - 1);
        if (total == 0) continue;
        const unsigned ne = __ballot_sync(FULL, len > 0);
        unsigned todo = ne;
        if (LONG && total >= LONG_SEG_MIN * __popc(todo)) {
            // ---- long segments: one A entry at a time, its B entries in chunks of up
            // to LU*32 (LU steps of 32); the next chunk's loads are issued before the
            // current chunk is used.  Entries of one B row have distinct columns, so a
            // chunk has no slot conflicts; a change of A entry needs a warp sync.
            int sgi = __ffs(todo) - 1;
            todo &= todo - 1;
            int es = __shfl_sync(FULL, elo, sgi), ls = __shfl_sync(FULL, len, sgi);
            double as = __shfl_sync(FULL, a, sgi);
            int off = 0;
            int jc[LU];
            double bc[LU];
#pragma unroll
            for (int u = 0; u < LU; u++) {
                const int e = u * WARP + lane;
                jc[u] = 0;
                bc[u] = 0.0;
                if (e < ls) {
                    jc[u] = ldx<NC>(bcol + es + e);
                    bc[u] = ldx<NC>(bval + es + e);
                }
            }
            while (true) {
                int n_off = off + LU * WARP, n_es = es, n_ls = ls;
                double n_as = as;
                bool more = true, seg_change = false;
                if (n_off >= ls) {
                    if (!todo) {
                        more = false;
                    } else {
                        const int n_sgi = __ffs(todo) - 1;
                        todo &= todo - 1;
                        n_es = __shfl_sync(FULL, elo, n_sgi);
                        n_ls = __shfl_sync(FULL, len, n_sgi);
                        n_as = __shfl_sync(FULL, a, n_sgi);
                        n_off = 0;
                        seg_change = true;
                    }
                }
                int jn[LU];
                double bn[LU];
#pragma unroll
                for (int u = 0; u < LU; u++) {
                    const int e = n_off + u * WARP + lane;
                    jn[u] = 0;
                    bn[u] = 0.0;
                    if (more && e < n_ls) {
                        jn[u] = ldx<NC>(bcol + n_es + e);
                        bn[u] = ldx<NC>(bval + n_es + e);
                    }
                }
#pragma unroll
                for (int u = 0; u < LU; u++) {
                    if (off + u * WARP >= ls) break;  // warp-uniform: the chunk is shorter
                    if (off + u * WARP + lane < ls) {
                        const double pr = term<AR>(as, bc[u]);
                        const int q = lookup(jc[u]);
                        if (q >= 0) acc[q] = add_term<AR>(acc[q], as, pr);
                        else bad = true;
                    }
                }
                if (!more) break;
                if (seg_change) __syncwarp();
                es = n_es;
                ls = n_ls;
                as = n_as;
                off = n_off;
#pragma unroll
                for (int u = 0; u < LU; u++) {
                    jc[u] = jn[u];
                    bc[u] = bn[u];
                }
            }
            __syncwarp();
            continue;
        }
        // ---- short segments: flat (A entry, B entry) order, 32 items per step.
        // The non-empty segments are packed into lanes 0..nseg-1 (flat start
        // st, B-entry shift d = elo - st, a).  Each step ORs the starts that
        // fall inside it into one 32-bit mask; the segment of a lane's item is
        // then the number of starts up to it (one popc), and a step with no
        // start after its first item holds one A entry (no slot conflicts).
        const int nseg = __popc(ne);
        const int excl = incl - len;
        const int src = nth_set_bit(ne, min(lane, nseg - 1));
        const int st_src = __shfl_sync(FULL, excl, src);
        const int c_d = __shfl_sync(FULL, elo - excl, src);
        const double c_a = __shfl_sync(FULL, a, src);
        const int c_st = lane < nseg ? st_src : INT_MAX;
        const unsigned le = lanemask_le();
        auto starts = [&](int f) -> unsigned {
            const unsigned rel = (unsigned)(c_st - f);
            return __reduce_or_sync(FULL, rel < 32u ? 1u << rel : 0u);
        };
        unsigned sm = starts(0);
        int cb = 0;  // packed segments that start before the current step
        int j = 0;
        double b = 0.0, as;
        {
            const int sg = __popc(sm & le) - 1;
            const int e = lane + __shfl_sync(FULL, c_d, sg);
            as = __shfl_sync(FULL, c_a, sg);
            if (lane < total) {
                j = ldx<NC>(bcol + e);
                b = ldx<NC>(bval + e);
            }
        }
        for (int f = 0; f < total; f += WARP) {
            const bool gv = f + lane < total;
            const bool multi = (sm >> 1) != 0u;  // a segment starts after the step's first item
            cb += __popc(sm);
            int j_n = 0;
            double b_n = 0.0, as_n = 0.0;
            if (f + WARP < total) {
                sm = starts(f + WARP);
                const int sg_n = cb + __popc(sm & le) - 1;
                const int gn = f + WARP + lane;
                const int e = gn + __shfl_sync(FULL, c_d, sg_n);
                as_n = __shfl_sync(FULL, c_a, sg_n);
                if (gn < total) {
                    j_n = ldx<NC>(bcol + e);
                    b_n = ldx<NC>(bval + e);
                }
            }
            // every lane multiplies and looks up (invalid lanes: b = 0, result unused)
            const double pr = term<AR>(as, b);
            const int q = lookup(j);
            bad |= gv && q < 0;
            const bool act = gv && q >= 0;
            const int slot = act ? q : -1 - lane;
            if (!multi) {
                // one A entry in this step: all slots distinct
                if (act) acc[slot] = add_term<AR>(acc[slot], as, pr);
            } else if (TAG) {
                // each lane stamps its id on its slot; a lane that reads back another
                // id shares the slot with that lane.  Only such lanes are matched.
                if (act) tag[slot] = (unsigned char)lane;
                __syncwarp();
                const int seen = act ? (int)tag[slot] : lane;
                const bool lost = seen != lane;
                const unsigned lm = __ballot_sync(FULL, lost);
                if (lm == 0u) {
                    if (act) acc[slot] = add_term<AR>(acc[slot], as, pr);
                } else {
                    const unsigned cm = lm | __reduce_or_sync(FULL, lost ? 1u << seen : 0u);
                    const bool inc = (cm >> lane) & 1u;
                    int rank = 0;
                    if (inc) rank = __popc(__match_any_sync(cm, slot) & lanemask_lt());
                    const int maxr = (int)__reduce_max_sync(FULL, (unsigned)rank);
                    // round 0: the lanes that share no slot together with the first lane
                    // of each shared slot (all their slots are distinct), then one round
                    // per further lane of a shared slot
                    if (act && rank == 0) acc[slot] = add_term<AR>(acc[slot], as, pr);
                    __syncwarp();
                    for (int rr = 1; rr <= maxr; rr++) {
                        if (inc && rank == rr) acc[slot] = add_term<AR>(acc[slot], as, pr);
                        __syncwarp();
                    }
                }
            } else {
                const unsigned grp = __match_any_sync(FULL, slot);
                const int rank = __popc(grp & lanemask_lt());
                const int maxr = (int)__reduce_max_sync(FULL, act ? (unsigned)rank : 0u);
                for (int rr = 0; rr < maxr; rr++) {
                    if (act && rank == rr) acc[slot] = add_term<AR>(acc[slot], as, pr);
                    __syncwarp();
                }
                if (act && rank == maxr) acc[slot] = add_term<AR>(acc[slot], as, pr);
            }
            __syncwarp();
            j = j_n;
            b = b_n;
            as = as_n;
        }
    }
}

}  // namespace hsmu
