// Batched persistent engine: many independent SpGEMMs (C_p = A_p * B_p) or
// AMG Galerkin triple products (C_p = Pt_p * (A_p * P_p)) in ONE launch.
//
// The reference runs each product separately, with ~10 blocking host round
// trips and several cudaMalloc calls per product
// (src/compressed/compressed_NHC_spgemm.cu:22-248); for hundreds of small
// products that overhead, not the arithmetic, sets the time.  Here all rows of
// all products form one flattened row space and a single cooperative,
// persistent kernel walks it in phases separated by grid-wide barriers:
//   COUNT  exact nnz of every C row (thread per row for rows with <= `tiny`
//          products, warp per row with a dense tile-span table otherwise)
//   SCAN   one device-wide exclusive scan of the row counts; the scan is also
//          the output allocator: product p's entries start at the scan value
//          of its first row inside one preallocated pool (no cudaMalloc)
//   FILL   sorted columns and values of every row (same classes)
// and, for Galerkin products, the same three phases again with A = Pt and B =
// the A*P just produced.  No host synchronisation happens inside; the launch
// can be captured once in a CUDA graph and replayed.
//
// Grid barriers spin on a generation counter with an iteration limit: a
// barrier that gives up sets an error bit (HSMU_ERR_TIMEOUT) and every block
// returns, so a fault in one block can never hang the GPU.
//
// Rows that need the large-row (CTA) path of the plain engine (tile span >
// SPAN_T or more than B_FUSE_CAP entries) are not handled in a batch: the
// kernel flags them, hsmu_batch_status reports HSMU_ERR_UNSUPPORTED, and the
// caller runs such products with hsmu_spgemm.
//
// Tuning: the thread-per-row threshold (`tiny`) and the grid size are
// parameters of the launch; hsmu_batch_autotune times the candidates on the
// actual batch and keeps the fastest.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <new>
#include <vector>

#include "hsmu_gb.h"
#include "hsmu_kernels.h"
#include "hsmu_rowops.cuh"

namespace hsmu {

constexpr int B_FUSE_CAP = 512;  // nnz of a warp-path row in a batch
constexpr unsigned long long SPIN_LIMIT = 1ull << 25;
enum BatchErr : int { BERR_TIMEOUT = 16, BERR_UNSUPPORTED = 32, BERR_CAPACITY = 64, BERR_INTERNAL = 128 };

struct BOp {  // one CSR operand on the device; row k is rp[k] .. re[k]-1 (re = rp + 1 for CSR)
    int M, N;
    const int *rp;
    const int *re;
    const int *col;
    const double *val;
};

struct BRound {
    int nprod;
    const BOp *A;          // left operand per product
    const BOp *B;          // right operand per product (unused when b_from_prev)
    int b_from_prev;       // B_p = C_p of the previous round
    const long long *row0; // [nprod+1] flattened row offsets
    const long long *rpo;  // [nprod+1] offsets of each product's row_ptr in rp_pool (sum of M+1)
    long long R;           // total rows
    int *cnnz;             // [R]
    long long *excl;       // [R+1]
    int *rp_pool;          // [rpo[nprod]]
    int *col_pool;         // [cap]
    double *val_pool;      // [cap]
    long long cap;
    // padded round (the A*P of Galerkin products, read only by the next round): every
    // row has a slot of its product bound, excl holds the slots' offsets (set once at
    // creation), rp_pool their starts within the product; one fill pass writes the row,
    // its count (cnnz) and its end (re_pool).  No count pass, no scan.
    int padded;
    int *re_pool;          // [rpo[nprod]] (padded rounds)
};

struct GridBar {
    unsigned count;
    unsigned gen;
};

struct BParams {
    BRound rnd[2];
    int nrounds;
    int tiny;              // products threshold of the thread-per-row class
    long long *bsum;       // [gridDim.x + 1]
    GridBar *bar;
    int *err;
    int arith;             // hsmu_opts.arith of the batch
    unsigned long long spin_limit;  // polls of a grid barrier before it gives up
};

__device__ bool grid_sync(GridBar *gb, int *err, unsigned long long spin_limit) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        volatile unsigned *vgen = &gb->gen;
        const unsigned g = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(&gb->count, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(&gb->count, 0u);
            __threadfence();
            atomicAdd(&gb->gen, 1u);
        } else {
            unsigned long long it = 0;
            while (*vgen == g) {
                if (++it > spin_limit) {
                    atomicOr(err, BERR_TIMEOUT);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        if (*(volatile int *)err & BERR_TIMEOUT) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// product owning flattened row i (row0 ascending)
__device__ __forceinline__ int find_prod(const long long *row0, int n, long long i) {
    int lo = 0, hi = n;  // row0[lo] <= i < row0[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(row0 + mid) <= i) lo = mid; else hi = mid;
    }
    return lo;
}

// the B operand of product p in round r (C of the previous round for Galerkin)
__device__ __forceinline__ BOp b_operand(const BParams &P, int r, int p) {
    const BRound &R = P.rnd[r];
    if (!R.b_from_prev) return R.B[p];
    const BRound &Q = P.rnd[r - 1];
    const long long r0 = Q.row0[p];
    const long long base = Q.excl[r0];
    BOp b;
    b.M = (int)(Q.row0[p + 1] - r0);
    b.N = -1;  // not needed by the row routines
    b.rp = Q.rp_pool + Q.rpo[p];
    b.re = Q.padded ? Q.re_pool + Q.rpo[p] : b.rp + 1;
    b.col = Q.col_pool + base;
    b.val = Q.val_pool + base;
    return b;
}

constexpr int BW = 8;  // warps per block (launch uses BW*32 threads)

struct BWarpSmem {
    union {
        struct {
            unsigned long long msk[SPAN_T];
            int base[SPAN_T];
            double acc[B_FUSE_CAP];
        } w;
        struct {
            int cols[TINY_MAX * WARP];
            double acc[TINY_MAX * WARP];
        } t;
    };
};

enum RowMode { RM_COUNT = 0, RM_FILL = 1, RM_PADDED = 2 };

// one pass over the rows of round r: COUNT (exact nnz), FILL (columns and
// values at the scanned offsets) or PADDED (fill at the row's bound slot,
// recording its nnz and end)
template <int AR, int MODE, bool NC>
__device__ void phase_rows(const BParams &P, int r, BWarpSmem &S) {
    constexpr bool FILL = MODE != RM_COUNT;
    const BRound &R = P.rnd[r];
    const int lane = lane_id(), w = threadIdx.x >> 5;
    const long long step = (long long)gridDim.x * BW * WARP;
    for (long long g0 = ((long long)blockIdx.x * BW + w) * WARP; g0 < R.R; g0 += step) {
        const long long i = g0 + lane;
        bool big = false;
        if (i < R.R) {
            const int p = find_prod(R.row0, R.nprod, i);
            const BOp A = R.A[p];
            const BOp B = b_operand(P, r, p);
            const int li = (int)(i - R.row0[p]);
            const int a_lo = ldx<NC>(A.rp + li), a_hi = ldx<NC>(A.rp + li + 1);
            // with the class threshold at the list capacity, the thread path is tried
            // directly and gives up (returns -1, nothing written) on a row with more
            // products: no separate pass over the row to classify it
            const bool direct = P.tiny >= TINY_MAX;
            const int prod = direct ? 0 : tiny_products<NC>(a_lo, a_hi, A.col, B.rp, B.re, P.tiny);
            if (prod > P.tiny) {
                big = true;
            } else if (!FILL) {
                const int c = tiny_row_count<NC>(a_lo, a_hi, A.col, B.rp, B.re, B.col, S.t.cols + lane, WARP);
                if (c < 0 && direct) {
                    big = true;
                } else {
                    R.cnnz[i] = c < 0 ? 0 : c;
                    if (c < 0) atomicOr(P.err, BERR_INTERNAL);
                }
            } else if (MODE == RM_PADDED) {
                const long long o = R.excl[i];
                const int cap = (int)(R.excl[i + 1] - o);
                const int got = tiny_row_fill<AR, NC>(a_lo, a_hi, A.col, A.val, B.rp, B.re, B.col, B.val,
                                                      S.t.cols + lane, S.t.acc + lane, WARP, cap, R.col_pool + o,
                                                      R.val_pool + o);
                if (got < 0) {
                    big = true;  // more than TINY_MAX products (a slot always holds the row)
                } else {
                    const long long at = R.rpo[p] + li;
                    R.cnnz[i] = got;
                    R.re_pool[at] = R.rp_pool[at] + got;
                }
            } else {
                const long long o = R.excl[i];
                const int nnz = R.cnnz[i];
                if (o + nnz <= R.cap) {
                    const int got = tiny_row_fill<AR, NC>(a_lo, a_hi, A.col, A.val, B.rp, B.re, B.col, B.val,
                                                          S.t.cols + lane, S.t.acc + lane, WARP, nnz, R.col_pool + o,
                                                          R.val_pool + o);
                    if (got < 0 && direct) big = true;
                    else if (got != nnz) atomicOr(P.err, BERR_INTERNAL);
                }
            }
        }
        __syncwarp();
        unsigned bigs = __ballot_sync(FULL, big);
        while (bigs) {
            const int src = __ffs(bigs) - 1;
            bigs &= bigs - 1;
            const long long ib = g0 + src;
            const int p = find_prod(R.row0, R.nprod, ib);
            const BOp A = R.A[p];
            const BOp B = b_operand(P, r, p);
            const int li = (int)(ib - R.row0[p]);
            const int a_lo = ldx<NC>(A.rp + li), a_hi = ldx<NC>(A.rp + li + 1);
            int cmin, cmax, prod;
            warp_row_extent<NC>(a_lo, a_hi, A.col, B.rp, B.re, B.col, cmin, cmax, prod);
            const int t0 = cmin >> 6;
            const int span = (cmax >> 6) - t0 + 1;
            if (span > SPAN_T) {
                if (lane == 0) atomicOr(P.err, BERR_UNSUPPORTED);
                if (!FILL && lane == 0) R.cnnz[ib] = 0;
                continue;
            }
            if (!warp_row_masks<NC>(a_lo, a_hi, A.col, B.rp, B.re, B.col, t0, span, S.w.msk)) {
                if (lane == 0) atomicOr(P.err, BERR_INTERNAL);
                continue;
            }
            if (!FILL) {
                const int c = warp_mask_count(S.w.msk, span);
                if (lane == 0) R.cnnz[ib] = c;
                if (c > B_FUSE_CAP && lane == 0) atomicOr(P.err, BERR_UNSUPPORTED);
            } else {
                const long long o = R.excl[ib];
                int nnz;
                if (MODE == RM_PADDED) {
                    nnz = warp_mask_count(S.w.msk, span);
                    if (nnz > B_FUSE_CAP || o + nnz > R.excl[ib + 1]) {
                        if (lane == 0) atomicOr(P.err, nnz > B_FUSE_CAP ? BERR_UNSUPPORTED : BERR_INTERNAL);
                        continue;
                    }
                    if (lane == 0) {
                        const long long at = R.rpo[p] + li;
                        R.cnnz[ib] = nnz;
                        R.re_pool[at] = R.rp_pool[at] + nnz;
                    }
                } else {
                    nnz = R.cnnz[ib];
                }
                if (nnz <= B_FUSE_CAP && o + nnz <= R.cap) {
                    if (!warp_row_fill<AR, NC>(a_lo, a_hi, A.col, A.val, B.rp, B.re, B.col, B.val, t0, span,
                                                S.w.msk, S.w.base, S.w.acc, nnz, R.col_pool + o, R.val_pool + o) &&
                        lane == 0)
                        atomicOr(P.err, BERR_INTERNAL);
                }
            }
            __syncwarp();
        }
    }
}

// device-wide exclusive scan of cnnz into excl (3 steps, 2 barriers inside)
__device__ bool phase_scan(const BParams &P, int r) {
    const BRound &R = P.rnd[r];
    __shared__ long long s_tmp[BW + 1];
    const long long per = (R.R + gridDim.x - 1) / gridDim.x;
    const long long lo = min((long long)blockIdx.x * per, R.R), hi = min(lo + per, R.R);
    long long v = 0;
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) v += R.cnnz[i];
    long long tot;
    block_excl_sum<BW * 32>(v, s_tmp, tot);
    if (threadIdx.x == 0) P.bsum[blockIdx.x] = tot;
    if (!grid_sync(P.bar, P.err, P.spin_limit)) return false;
    if (blockIdx.x == 0) {
        long long carry = 0;
        for (int b0 = 0; b0 < (int)gridDim.x; b0 += blockDim.x) {
            const int b = b0 + threadIdx.x;
            const long long x = b < (int)gridDim.x ? P.bsum[b] : 0;
            long long t2;
            const long long ex = block_excl_sum<BW * 32>(x, s_tmp, t2);
            if (b < (int)gridDim.x) P.bsum[b] = ex + carry;
            carry += t2;
        }
        if (threadIdx.x == 0) {
            P.bsum[gridDim.x] = carry;
            R.excl[R.R] = carry;
            if (carry > R.cap) atomicOr(P.err, BERR_CAPACITY);
        }
    }
    if (!grid_sync(P.bar, P.err, P.spin_limit)) return false;
    // block scan of the chunk, in tiles of SCAN_RUN rows per thread (one block scan,
    // three barriers, per tile of blockDim * SCAN_RUN rows)
    constexpr int SCAN_RUN = 16;
    long long run = P.bsum[blockIdx.x];
    for (long long b = lo; b < hi; b += (long long)blockDim.x * SCAN_RUN) {
        const long long i0 = b + (long long)threadIdx.x * SCAN_RUN;
        int x[SCAN_RUN];
        long long s = 0;
#pragma unroll
        for (int u = 0; u < SCAN_RUN; u++) {
            x[u] = i0 + u < hi ? R.cnnz[i0 + u] : 0;
            s += x[u];
        }
        long long t2;
        long long e = run + block_excl_sum<BW * 32>(s, s_tmp, t2);
#pragma unroll
        for (int u = 0; u < SCAN_RUN; u++) {
            if (i0 + u < hi) R.excl[i0 + u] = e;
            e += x[u];
        }
        run += t2;
    }
    return true;
}

// per-product row pointers (0-based within the product) from the global scan
__device__ void phase_rowptr(const BParams &P, int r) {
    const BRound &R = P.rnd[r];
    const long long nthr = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < R.R; i += nthr) {
        const int p = find_prod(R.row0, R.nprod, i);
        const long long r0 = R.row0[p];
        R.rp_pool[R.rpo[p] + (i - r0)] = (int)(R.excl[i] - R.excl[r0]);
        if (i == R.row0[p + 1] - 1) R.rp_pool[R.rpo[p] + (i - r0) + 1] = (int)(R.excl[i + 1] - R.excl[r0]);
    }
    // products without rows
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < R.nprod; p += (int)nthr)
        if (R.row0[p + 1] == R.row0[p]) R.rp_pool[R.rpo[p]] = 0;
}

template <int AR>
__global__ void __launch_bounds__(BW * 32) k_batch(BParams P) {
    extern __shared__ unsigned long long s_dyn[];
    BWarpSmem &S = reinterpret_cast<BWarpSmem *>(s_dyn)[threadIdx.x >> 5];
    for (int r = 0; r < P.nrounds; r++) {
        if (r > 0 && !grid_sync(P.bar, P.err, P.spin_limit)) return;
        if (P.rnd[r].padded) {  // only round 0 (operands from the caller) is ever padded
            phase_rows<AR, RM_PADDED, true>(P, r, S);
            continue;
        }
        if (r == 0) phase_rows<AR, RM_COUNT, true>(P, r, S);
        else phase_rows<AR, RM_COUNT, false>(P, r, S);
        if (!grid_sync(P.bar, P.err, P.spin_limit)) return;
        if (!phase_scan(P, r)) return;
        if (!grid_sync(P.bar, P.err, P.spin_limit)) return;
        if (*(volatile int *)P.err & BERR_CAPACITY) return;
        phase_rowptr(P, r);
        if (r == 0) phase_rows<AR, RM_FILL, true>(P, r, S);
        else phase_rows<AR, RM_FILL, false>(P, r, S);
    }
}

// ---------------------------------------------------------------- sizing
// per row of round 1: products and the bound min(products, N) on its nnz;
// for Galerkin also the bound of round 2 (sum over the Pt row of the round-1
// row bounds, capped by N)
__global__ void k_batch_bound(const BOp *A, const BOp *B, const long long *row0, int nprod, long long R,
                              int *rowbound, unsigned long long *total) {
    unsigned long long my = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < R; i += (long long)gridDim.x * blockDim.x) {
        const int p = find_prod(row0, nprod, i);
        const BOp a = A[p], b = B[p];
        const int li = (int)(i - row0[p]);
        long long prod = 0;
        for (int q = a.rp[li]; q < a.rp[li + 1]; q++) {
            const int k = a.col[q];
            prod += b.rp[k + 1] - b.rp[k];
        }
        const long long bnd = prod < b.N ? prod : b.N;
        if (rowbound) rowbound[i] = (int)bnd;
        my += (unsigned long long)bnd;
    }
    my = warp_sum(my);
    if (lane_id() == 0 && my) atomicAdd(total, my);
}

// starts of the padded rows of a round within their product (from the scanned bounds)
__global__ void k_pad_starts(const long long *row0, int nprod, long long R, const long long *excl,
                             const long long *rpo, int *rp) {
    const long long nthr = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < R; i += nthr) {
        const int p = find_prod(row0, nprod, i);
        const long long r0 = row0[p];
        rp[rpo[p] + (i - r0)] = (int)(excl[i] - excl[r0]);
        if (i == row0[p + 1] - 1) rp[rpo[p] + (i - r0) + 1] = (int)(excl[i + 1] - excl[r0]);
    }
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nprod; p += (int)nthr)
        if (row0[p + 1] == row0[p]) rp[rpo[p]] = 0;
}

__global__ void k_batch_bound2(const BOp *Pt, const long long *row0_2, const long long *row0_1, int nprod, long long R,
                               const int *rowbound1, const int *ncols, unsigned long long *total) {
    unsigned long long my = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < R; i += (long long)gridDim.x * blockDim.x) {
        const int p = find_prod(row0_2, nprod, i);
        const BOp a = Pt[p];
        const int li = (int)(i - row0_2[p]);
        long long prod = 0;
        for (int q = a.rp[li]; q < a.rp[li + 1]; q++) prod += rowbound1[row0_1[p] + a.col[q]];
        my += (unsigned long long)(prod < ncols[p] ? prod : ncols[p]);
    }
    my = warp_sum(my);
    if (lane_id() == 0 && my) atomicAdd(total, my);
}

}  // namespace hsmu

using namespace hsmu;

struct hsmu_batch_s {
    int kind, nprod;
    int nsm, grid, threads, tiny, arith;
    size_t smem;
    BParams P;
    // device allocations
    void *dev_ops;            // BOp tables
    std::vector<void *> allocs;
    std::vector<long long> row0[2], rpo[2];
    std::vector<int> ncol[2];
    cudaGraph_t graph;
    cudaGraphExec_t gexec;
};

namespace {

template <class T>
cudaError_t balloc(hsmu_batch_s *b, T **p, size_t n) {
    *p = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess) b->allocs.push_back(*p);
    return e;
}

int launch_batch(hsmu_batch_s *b, cudaStream_t st) {
    if (cudaMemsetAsync(b->P.bar, 0, sizeof(GridBar), st) != cudaSuccess) return HSMU_ERR_CUDA;
    if (cudaMemsetAsync(b->P.err, 0, sizeof(int), st) != cudaSuccess) return HSMU_ERR_CUDA;
    b->P.tiny = b->tiny;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(b->grid);
    cfg.blockDim = dim3(b->threads);
    cfg.dynamicSmemBytes = b->smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = b->arith == AR_IMUL  ? cudaLaunchKernelEx(&cfg, k_batch<AR_IMUL>, b->P)
                    : b->arith == AR_FMA ? cudaLaunchKernelEx(&cfg, k_batch<AR_FMA>, b->P)
                                         : cudaLaunchKernelEx(&cfg, k_batch<AR_RN>, b->P);
    return e == cudaSuccess ? HSMU_OK : HSMU_ERR_CUDA;
}

int configure_batch(hsmu_batch_s *b, int dev) {
    b->threads = BW * 32;
    b->smem = BW * sizeof(BWarpSmem);
    for (auto k : {k_batch<AR_RN>, k_batch<AR_FMA>, k_batch<AR_IMUL>})
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem) != cudaSuccess)
            return HSMU_ERR_CUDA;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<AR_RN>, b->threads, b->smem) != cudaSuccess ||
        per_sm < 1)
        return HSMU_ERR_CUDA;
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop) return HSMU_ERR_NO_DEVICE;
    b->grid = b->nsm * per_sm;
    return HSMU_OK;
}

}  // namespace

extern "C" {

int hsmu_batch_create(hsmu_handle h, int kind, int n, const hsmu_csr *A, const hsmu_csr *B, const hsmu_csr *Pt,
                      const hsmu_opts *opts, hsmu_batch *out, void *stream) {
    if (!h || !out || n <= 0 || !A || !B) return HSMU_ERR_INVALID;
    if (kind != HSMU_BATCH_PRODUCT && kind != HSMU_BATCH_GALERKIN) return HSMU_ERR_INVALID;
    if (kind == HSMU_BATCH_GALERKIN && !Pt) return HSMU_ERR_INVALID;
    if (opts && (opts->arith < HSMU_ARITH_RN || opts->arith > HSMU_ARITH_IMUL)) return HSMU_ERR_INVALID;
    *out = nullptr;
    for (int p = 0; p < n; p++) {
        if (A[p].N != B[p].M || !A[p].row_ptr || !B[p].row_ptr) return HSMU_ERR_INVALID;
        if (kind == HSMU_BATCH_GALERKIN && (Pt[p].N != A[p].M || !Pt[p].row_ptr)) return HSMU_ERR_INVALID;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    hsmu_batch_s *b = new (std::nothrow) hsmu_batch_s();
    if (!b) return HSMU_ERR_ALLOC;
    b->kind = kind;
    b->nprod = n;
    b->arith = opts ? opts->arith : AR_RN;
    // test hook: barriers that give up after opts->wait_polls spins
    b->P.spin_limit = (opts && opts->wait_polls > 0) ? (unsigned long long)opts->wait_polls : SPIN_LIMIT;
    b->tiny = TINY_MAX;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, dev);
    int rc = configure_batch(b, dev);
    const int nr = kind == HSMU_BATCH_GALERKIN ? 2 : 1;
    BOp *dA = nullptr, *dB = nullptr;
    int *rowbound = nullptr, *dncol = nullptr;
    unsigned long long *dtot = nullptr, htot[2] = {0, 0};
    long long *drow0[2] = {nullptr, nullptr}, *drpo[2] = {nullptr, nullptr};
    std::vector<BOp> hA(n), hB(n);
    if (rc) goto fail;
    b->P.nrounds = nr;
    // operand tables and row offsets
    for (int r = 0; r < nr; r++) {
        const hsmu_csr *L = (r == 0) ? A : Pt;
        b->row0[r].assign(n + 1, 0);
        b->rpo[r].assign(n + 1, 0);
        b->ncol[r].assign(n, 0);
        for (int p = 0; p < n; p++) {
            b->row0[r][p + 1] = b->row0[r][p] + L[p].M;
            b->rpo[r][p + 1] = b->rpo[r][p] + L[p].M + 1;
            b->ncol[r][p] = B[p].N;
        }
        for (int p = 0; p < n; p++) {
            hA[p] = BOp{L[p].M, L[p].N, L[p].row_ptr, L[p].row_ptr + 1, L[p].col, L[p].val};
            hB[p] = BOp{B[p].M, B[p].N, B[p].row_ptr, B[p].row_ptr + 1, B[p].col, B[p].val};
        }
        if (balloc(b, &dA, n) || balloc(b, &dB, n) || balloc(b, &drow0[r], n + 1) || balloc(b, &drpo[r], n + 1)) {
            rc = HSMU_ERR_ALLOC;
            goto fail;
        }
        cudaMemcpy(dA, hA.data(), sizeof(BOp) * n, cudaMemcpyHostToDevice);
        cudaMemcpy(dB, hB.data(), sizeof(BOp) * n, cudaMemcpyHostToDevice);
        cudaMemcpy(drow0[r], b->row0[r].data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice);
        cudaMemcpy(drpo[r], b->rpo[r].data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice);
        BRound &R = b->P.rnd[r];
        R.nprod = n;
        R.A = dA;
        R.B = (r == 0) ? dB : nullptr;
        R.b_from_prev = r > 0;
        R.row0 = drow0[r];
        R.rpo = drpo[r];
        R.R = b->row0[r][n];
    }
    // capacity bounds (one sizing pass and one host read)
    if (balloc(b, &dtot, 2)) {
        rc = HSMU_ERR_ALLOC;
        goto fail;
    }
    cudaMemsetAsync(dtot, 0, 2 * sizeof(unsigned long long), st);
    if (nr == 2 && balloc(b, &rowbound, (size_t)b->P.rnd[0].R)) {
        rc = HSMU_ERR_ALLOC;
        goto fail;
    }
    k_batch_bound<<<b->nsm * 8, 256, 0, st>>>(b->P.rnd[0].A, b->P.rnd[0].B, b->P.rnd[0].row0, n, b->P.rnd[0].R,
                                              rowbound, dtot);
    if (nr == 2) {
        std::vector<int> nc(n);
        for (int p = 0; p < n; p++) nc[p] = B[p].N;
        if (balloc(b, &dncol, n)) {
            rc = HSMU_ERR_ALLOC;
            goto fail;
        }
        cudaMemcpy(dncol, nc.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
        k_batch_bound2<<<b->nsm * 8, 256, 0, st>>>(b->P.rnd[1].A, b->P.rnd[1].row0, b->P.rnd[0].row0, n,
                                                   b->P.rnd[1].R, rowbound, dncol, dtot + 1);
    }
    if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(htot, dtot, sizeof(htot), cudaMemcpyDeviceToHost, st) ||
        cudaStreamSynchronize(st)) {
        rc = HSMU_ERR_CUDA;
        goto fail;
    }
    for (int r = 0; r < nr; r++) {
        BRound &R = b->P.rnd[r];
        R.cap = (long long)htot[r];
        if (balloc(b, &R.cnnz, (size_t)R.R) || balloc(b, &R.excl, (size_t)R.R + 1) ||
            balloc(b, &R.rp_pool, (size_t)b->rpo[r][n]) || balloc(b, &R.col_pool, (size_t)R.cap) ||
            balloc(b, &R.val_pool, (size_t)R.cap)) {
            rc = HSMU_ERR_ALLOC;
            goto fail;
        }
    }
    if (balloc(b, &b->P.bsum, (size_t)b->grid + 1) || balloc(b, &b->P.bar, 1) || balloc(b, &b->P.err, 1)) {
        rc = HSMU_ERR_ALLOC;
        goto fail;
    }
    // Galerkin: A*P is read only by the second round, so its rows go straight into slots of
    // their product bound (offsets = scan of the bounds, fixed for the batch's lifetime)
    if (nr == 2 && b->P.rnd[0].R <= INT_MAX && htot[0] <= (unsigned long long)INT_MAX) {
        BRound &R0 = b->P.rnd[0];
        int *scan_tmp = nullptr;
        long long *tot64 = nullptr;
        if (balloc(b, &R0.re_pool, (size_t)b->rpo[0][n]) || balloc(b, &scan_tmp, scan_tmp_ints((int)R0.R)) ||
            balloc(b, &tot64, 1)) {
            rc = HSMU_ERR_ALLOC;
            goto fail;
        }
        launch_scan64(rowbound, R0.excl, (int)R0.R, tot64, scan_tmp, st);
        k_pad_starts<<<b->nsm * 8, 256, 0, st>>>(R0.row0, n, R0.R, R0.excl, R0.rpo, R0.rp_pool);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
            rc = HSMU_ERR_CUDA;
            goto fail;
        }
        for (void *q : {(void *)scan_tmp, (void *)tot64}) {
            cudaFree(q);
            b->allocs.erase(std::find(b->allocs.begin(), b->allocs.end(), q));
        }
        R0.padded = 1;
    }
    if (rowbound) {  // only needed for sizing
        cudaFree(rowbound);
        b->allocs.erase(std::find(b->allocs.begin(), b->allocs.end(), (void *)rowbound));
    }
    b->P.arith = b->arith;
    *out = b;
    return HSMU_OK;
fail:
    hsmu_batch_destroy(b);
    return rc;
}

int hsmu_batch_execute(hsmu_batch b, void *stream) {
    if (!b) return HSMU_ERR_INVALID;
    return launch_batch(b, static_cast<cudaStream_t>(stream));
}

int hsmu_batch_graph_launch(hsmu_batch b, void *stream) {
    if (!b) return HSMU_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (!b->gexec) {
        cudaStream_t cap;
        if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return HSMU_ERR_CUDA;
        int rc = HSMU_OK;
        if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = HSMU_ERR_CUDA;
        if (!rc) rc = launch_batch(b, cap);
        cudaGraph_t g = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(cap, &g);
        if (!rc && ee != cudaSuccess) rc = HSMU_ERR_CUDA;
        if (!rc && cudaGraphInstantiate(&b->gexec, g, 0) != cudaSuccess) rc = HSMU_ERR_CUDA;
        if (g) b->graph = g;
        cudaStreamDestroy(cap);
        if (rc) {
            cudaGetLastError();
            return rc;
        }
    }
    return cudaGraphLaunch(b->gexec, st) == cudaSuccess ? HSMU_OK : HSMU_ERR_CUDA;
}

int hsmu_batch_status(hsmu_batch b, void *stream) {
    if (!b) return HSMU_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int err = 0;
    if (cudaMemcpyAsync(&err, b->P.err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return HSMU_ERR_CUDA;
    if (err & BERR_TIMEOUT) return HSMU_ERR_TIMEOUT;
    if (err & BERR_UNSUPPORTED) return HSMU_ERR_UNSUPPORTED;
    if (err & BERR_CAPACITY) return HSMU_ERR_OVERFLOW;
    if (err) return HSMU_ERR_INTERNAL;
    return HSMU_OK;
}

int hsmu_batch_result(hsmu_batch b, int p, hsmu_csr *C) {
    if (!b || !C || p < 0 || p >= b->nprod) return HSMU_ERR_INVALID;
    const int r = b->P.nrounds - 1;
    const BRound &R = b->P.rnd[r];
    long long ex[2] = {0, 0};
    const long long r0 = b->row0[r][p], r1 = b->row0[r][p + 1];
    if (cudaMemcpy(&ex[0], R.excl + r0, sizeof(long long), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&ex[1], R.excl + r1, sizeof(long long), cudaMemcpyDeviceToHost) != cudaSuccess)
        return HSMU_ERR_CUDA;
    C->M = (int)(r1 - r0);
    C->N = b->ncol[r][p];
    C->nnz = (int)(ex[1] - ex[0]);
    C->owned = 0;
    C->row_ptr = R.rp_pool + b->rpo[r][p];
    C->col = R.col_pool + ex[0];
    C->val = R.val_pool + ex[0];
    return HSMU_OK;
}

int hsmu_batch_set_params(hsmu_batch b, int tiny, int grid) {
    if (!b || tiny < 0 || tiny > TINY_MAX || grid < 0) return HSMU_ERR_INVALID;
    b->tiny = tiny;
    if (grid > 0) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<AR_RN>, b->threads, b->smem);
        if (grid > b->nsm * per_sm) return HSMU_ERR_INVALID;  // cooperative launch needs all blocks resident
        b->grid = grid;
    }
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    return HSMU_OK;
}

int hsmu_batch_autotune(hsmu_batch b, void *stream, int *best_tiny, int *best_grid, float *best_ms) {
    if (!b) return HSMU_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<AR_RN>, b->threads, b->smem);
    const int tinies[] = {8, 16, 32};
    std::vector<int> grids = {b->nsm * per_sm};
    if (per_sm > 1) grids.push_back(b->nsm);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int bt = b->tiny, bg = b->grid, rc = HSMU_OK;
    for (int t : tinies)
        for (int g : grids) {
            if ((rc = hsmu_batch_set_params(b, t, g))) break;
            if ((rc = launch_batch(b, st))) break;  // warm-up
            cudaEventRecord(e0, st);
            for (int k = 0; k < 2 && !rc; k++) rc = launch_batch(b, st);
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) != cudaSuccess) rc = HSMU_ERR_CUDA;
            if (rc) break;
            if ((rc = hsmu_batch_status(b, st))) break;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            ms *= 0.5f;
            if (ms < best) {
                best = ms;
                bt = t;
                bg = g;
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    rc = hsmu_batch_set_params(b, bt, bg);
    if (best_tiny) *best_tiny = bt;
    if (best_grid) *best_grid = bg;
    if (best_ms) *best_ms = best;
    return rc;
}

int hsmu_batch_destroy(hsmu_batch b) {
    if (!b) return HSMU_OK;
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (void *p : b->allocs) cudaFree(p);
    delete b;
    return HSMU_OK;
}

}  // extern "C"
