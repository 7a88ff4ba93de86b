// Host orchestration and C ABI of the GB300 HSMU SpGEMM engine.
//
// Pipeline for C = A * B (reference: compressed_NHC_spgemm,
// src/compressed/compressed_NHC_spgemm.cu:22-248):
//   1. B -> 64-column bit tiles (k_tiles count, scan, fill)      [skipped with hsmu_spgemm_tiled]
//   2. per-row bounds + row binning (k_bounds)
//   3. exact symbolic count (k_count_ds / k_count_l)
//   4. exclusive scan -> C row_ptr, nnz(C); ONE host read (8 bytes + flags)
//      and the output allocation
//   5a. sorted C columns + numeric windows (k_struct_ds / k_struct_l)
//   5b. values (k_numeric)
// The reference makes ~10 blocking host round trips and several cudaMalloc
// calls inside its timed region; this engine makes one read of a small
// control block and allocates from a stream-ordered pool that keeps freed
// memory cached across calls.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <initializer_list>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "hsmu_gb.h"
#include "hsmu_common.cuh"
#include "hsmu_kernels.h"

namespace hsmu {
int configure_count();

int status_from_dev_err(int err) {
    if (!err) return HSMU_OK;
    if (err & DERR_UNSORTED) return HSMU_ERR_UNSORTED;
    if (err & DERR_OVERFLOW) return HSMU_ERR_OVERFLOW;
    if (err & DERR_TIMEOUT) return HSMU_ERR_TIMEOUT;
    return HSMU_ERR_INTERNAL;
}
int configure_structure();
int configure_numeric();
}  // namespace hsmu

using namespace hsmu;

struct hsmu_handle_s {
    int device;
    int nsm;
    Ctl *h_ctl;  // pinned host mirror of the control block
    cudaEvent_t ev[8];
    // tile store arena (C tiles of the large rows, kept by the count pass): grown, up to
    // STORE_MAX_TILES, to the largest need a call has reported, before the next call
    int *arena_col;
    TileEnt *arena_ent;
    long long arena_cap, arena_want;
    // host-buffer entry: copy streams and their ordering events, and a page-locked
    // array of the products per PROD_CHUNK rows (grown on demand) that orders the row panels
    cudaStream_t cs_in, cs_out;
    cudaEvent_t ev_in, ev_panel, ev_out;
    long long *h_prod;
    size_t h_prod_cap;
    // B's tile conversion runs on its own stream beside the bounds pass
    cudaStream_t cs_tiles;
    cudaEvent_t ev_tiles_start, ev_tiles_done;
};

namespace {

const char *kErr[] = {"ok",
                      "invalid argument",
                      "allocation failed",
                      "CUDA error",
                      "overflow: nnz(C) or a scratch size does not fit int32",
                      "input CSR not canonical (columns must be strictly increasing and in range)",
                      "internal consistency check failed on the device",
                      "bounded device wait timed out",
                      "no usable sm_103 device",
                      "unsupported (no call returns this status)",
                      "output buffers too small: C->nnz holds the required number of entries"};

// hsmu_spgemm_host: output bytes (columns + values) per row panel, the most
// panels, and how panel sizes follow each other.  Nothing hides the first
// panel's compute (the copy back starts after it) or the last panel's copy.
// A product whose output outruns the host link (more than HOST_LINK_BOUND
// output bytes per intermediate product: the copy takes longer than the
// compute) is cut into panels that grow by HOST_PANEL_GROWTH to the middle,
// then shrink as much; one whose compute is the longer part only needs a small
// last panel, and its sizes shrink by HOST_PANEL_RATIO from the first (small
// panels leave the GPU partly idle, so only one end is made small).
// The panels then run in the order that keeps the link busy soonest and
// longest (panel_order): products per output entry differ by orders of
// magnitude between rows (R-MAT's hub rows), so in row order the first panel
// can hold many times its share of the compute.
constexpr long long HOST_PANEL_BYTES = 32ll << 20;

// entries of B from which its tile conversion runs on a second stream beside the bounds pass
constexpr int TILES_ASIDE_MIN_NNZ = 1 << 19;
constexpr long long HOST_MAX_PANELS = 8;
constexpr double HOST_PANEL_GROWTH = 2.0;
constexpr double HOST_PANEL_RATIO = 0.7;
constexpr double HOST_LINK_BOUND = 1.5;

// learned path: the least share of the products in warp-class rows that may need (bounds
// pass) or are predicted to need (after the prediction) numeric windows for the prediction
// to be used
constexpr double LEARNED_MIN_SHARE = 0.25;

int from_cuda(cudaError_t e) {
    if (e == cudaSuccess) return HSMU_OK;
    if (e == cudaErrorMemoryAllocation) return HSMU_ERR_ALLOC;
    return HSMU_ERR_CUDA;
}

#define CK(x)                                \
    do {                                     \
        cudaError_t _e = (x);                \
        if (_e != cudaSuccess) {             \
            rc = from_cuda(_e);              \
            goto done;                       \
        }                                    \
    } while (0)

int err_from_dev(int err) { return status_from_dev_err(err); }

// C's column array: 4 ints of slack past nnz, so that the value pass can fetch a
// window's columns in 16-byte units with bulk copies
constexpr size_t COL_PAD = 4;
// largest tile store arena (20 bytes per tile: 16 GB); rows beyond it are built
// by the structure pass's own OR walk instead
constexpr long long STORE_MAX_TILES = (16ll << 30) / 20;

bool csr_ok(const hsmu_csr *X) {
    if (!X || X->M < 0 || X->N < 0 || X->nnz < 0) return false;
    if (!X->row_ptr) return false;
    if (X->nnz > 0 && (!X->col || !X->val)) return false;
    return true;
}

DevCSR dev(const hsmu_csr *X) { return DevCSR{X->M, X->N, (long long)X->nnz, X->row_ptr, X->col, X->val}; }

// allocation-failure injection (hsmu_debug_fail_alloc): the countdown reaches 0
// at the allocation that is made to fail; 0 = disarmed
std::atomic<long long> g_fail_alloc_countdown{0};

template <class T>
cudaError_t palloc(T **p, size_t n, cudaStream_t st) {
    *p = nullptr;
    if (n == 0) n = 1;
    if (g_fail_alloc_countdown.load(std::memory_order_relaxed) > 0 &&
        g_fail_alloc_countdown.fetch_sub(1, std::memory_order_relaxed) == 1)
        return cudaErrorMemoryAllocation;
    return cudaMallocAsync(reinterpret_cast<void **>(p), n * sizeof(T), st);
}

template <class T>
void pfree(T *&p, cudaStream_t st) {
    if (p) cudaFreeAsync(p, st);
    p = nullptr;
}

int grid_rows(const hsmu_handle_s *h) { return h->nsm * 8; }

// arrays the library allocated from the stream-ordered pool and handed to the caller:
// returned to the pool once every stream of the device is done with them (the free
// functions take no stream; a plain cudaFree measured not to give the bytes back to
// the pool's in-use count)
void free_owned(std::initializer_list<const void *> ptrs) {
    bool any = false;
    for (const void *p : ptrs) any |= p != nullptr;
    if (!any) return;
    cudaDeviceSynchronize();
    for (const void *p : ptrs)
        if (p) cudaFreeAsync(const_cast<void *>(p), 0);
    cudaStreamSynchronize(0);
}

// B -> tiles into caller-visible arrays (tile arrays sized by nnz(B) >= tiles)
// B -> 64-column tiles.  Allocations on `st`; with `run` the kernels run on that
// stream instead (after everything already queued on `st`), the scratch is
// released there too, and ev_done marks the end: the caller makes `st` wait on
// it before anything reads the tiles.
int build_tiles(hsmu_handle_s *h, const hsmu_csr *B, hsmu_btiles *out, Ctl *ctl, int validate, cudaStream_t st,
                bool read_count, cudaStream_t run = nullptr, cudaEvent_t ev_start = nullptr,
                cudaEvent_t ev_done = nullptr) {
    int rc = HSMU_OK;
    cudaStream_t ks = st;
    int *tcnt = nullptr, *scan_tmp = nullptr;
    long long *tot = nullptr;
    DevCSR Bd = dev(B);
    out->M = B->M;
    out->N = B->N;
    out->ntiles = 0;
    out->tile_ptr = nullptr;
    out->tile_col = nullptr;
    out->mask = nullptr;
    out->tile_off = nullptr;
    CK(palloc(&out->tile_ptr, (size_t)B->M + 1, st));
    CK(palloc(&out->tile_col, (size_t)B->nnz, st));
    CK(palloc(&out->mask, (size_t)B->nnz, st));
    CK(palloc(&out->tile_off, (size_t)B->nnz, st));
    CK(palloc(&tcnt, (size_t)B->M + 1, st));
    CK(palloc(&scan_tmp, scan_tmp_ints(B->M), st));
    CK(palloc(&tot, 1, st));
    if (run && ev_start && ev_done) {
        CK(cudaEventRecord(ev_start, st));
        CK(cudaStreamWaitEvent(run, ev_start, 0));
        ks = run;
    }
    launch_tiles_count(Bd, tcnt, validate, ctl, grid_rows(h), ks);
    launch_scan(tcnt, out->tile_ptr, B->M, tot, scan_tmp, ctl, ks);
    launch_tiles_fill(Bd, out->tile_ptr, out->tile_col, reinterpret_cast<unsigned long long *>(out->mask), out->tile_off, ctl, grid_rows(h), ks);
    CK(cudaGetLastError());
    if (read_count) {
        CK(cudaMemcpyAsync(&ctl->ntiles, out->tile_ptr + B->M, sizeof(int), cudaMemcpyDeviceToDevice, ks));
    }
done:
    pfree(tcnt, ks);
    pfree(scan_tmp, ks);
    pfree(tot, ks);
    if (ks != st && ev_done) cudaEventRecord(ev_done, ks);
    if (rc != HSMU_OK) {
        // stream-ordered allocations go back the same way
        pfree(out->tile_ptr, st);
        pfree(out->tile_col, st);
        pfree(out->mask, st);
        pfree(out->tile_off, st);
    }
    return rc;
}

#define CKR(x)                              \
    do {                                    \
        const cudaError_t _e = (x);         \
        if (_e != cudaSuccess) return from_cuda(_e); \
    } while (0)

bool arith_ok(const hsmu_opts &o) { return o.arith >= HSMU_ARITH_RN && o.arith <= HSMU_ARITH_IMUL; }

// One plain product on the device, in stages: begin (control block,
// validation), symbolic (tiles, bounds, exact count, scan -> row pointers and
// nnz(C), one host read), alloc_output, then structure(lo, hi) + values()
// for one or more row panels, and finish (completion read, device checks).
// hsmu_spgemm runs one panel of all rows; hsmu_spgemm_host runs several so
// that copies of finished panels overlap the next panel's kernels.
struct PlainRun {
    hsmu_handle_s *h;
    cudaStream_t st;
    hsmu_opts o;
    int M = 0;
    DevCSR Ad{}, Bd{};
    hsmu_btiles bt{};
    bool own_tiles = false;
    bool tiles_aside = false;  // B's tiles are being built on the handle's conversion stream
    DevTiles Btd{};
    RowInfo ri{};
    long long *chunk_prod = nullptr;  // products per PROD_CHUNK rows (host-buffer entry)
    int *scan_tmp = nullptr;
    Window *win = nullptr;
    long long win_cap = 0;
    WinCursors wc{};
    int *crp = nullptr, *ccol = nullptr;
    double *cval = nullptr;
    // caller-owned column/value arrays (int64 path: the panel's place in C); not freed here
    int *ext_col = nullptr;
    double *ext_val = nullptr;
    Ctl *ctl = nullptr;
    Ctl hc{};
    int launches = 0;
    // C tiles of the large rows, kept by the count pass for the structure pass (in the
    // handle's arena; per-row offsets and counts here)
    long long *ts_off = nullptr;
    int *ts_cnt = nullptr, *ts_nwin = nullptr, *ts_wbase = nullptr;
    bool have_store = false;
    // the count pass reserves the large rows' windows (one product, one panel of
    // structure + values); the row panels of the host-buffer path restart the window
    // buffer at 0 for every panel and reserve them in the structure pass instead
    bool reserve_windows = true;

    PlainRun(hsmu_handle_s *h_, cudaStream_t st_, const hsmu_opts &o_) : h(h_), st(st_), o(o_) {}
    ~PlainRun() { release(); }

    int begin(const hsmu_csr *A, const hsmu_csr *B) {
        M = A->M;
        Ad = dev(A);
        Bd = dev(B);
        CKR(palloc(&ctl, 1, st));
        CKR(cudaMemsetAsync(ctl, 0, sizeof(Ctl), st));
        if (o.validate) {
            // check both operands before any kernel indexes through them
            launch_validate(Ad, ctl, grid_rows(h), st);
            launch_validate(Bd, ctl, grid_rows(h), st);
            launches += 2;
            CKR(cudaGetLastError());
            CKR(cudaMemcpyAsync(h->h_ctl, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
            CKR(cudaStreamSynchronize(st));
            if (h->h_ctl->err) return err_from_dev(h->h_ctl->err);
        }
        return HSMU_OK;
    }

    // host_rp != NULL: the row pointers of C are copied there in the same host read
    // host_prod != NULL: also the products of every PROD_CHUNK rows (ceil(M / PROD_CHUNK) entries)
    int symbolic(const hsmu_csr *B, const hsmu_btiles *Bt_in, bool count_tiles, int32_t *host_rp,
                 cudaEvent_t ev_tiles, long long *host_prod = nullptr) {
        int rc = tiles_bounds(B, Bt_in, count_tiles, ev_tiles, o.no_tile_store == 0);
        if (!rc) rc = count_scan(host_rp, host_prod);
        return rc;
    }

    // B's tiles (built, or the caller's) and the bounds pass: products, tile span and class
    // of every row of A, the class bins; with `store`, also every large row's tile bound
    // and the per-row arrays of the tile store (the arena is grown here when the previous
    // call needed more than it had)
    int tiles_bounds(const hsmu_csr *B, const hsmu_btiles *Bt_in, bool count_tiles, cudaEvent_t ev_tiles,
                     bool store) {
        if (Bt_in) {
            bt = *Bt_in;
        } else {
            // B's tiles on their own stream, beside the bounds pass (which reads B's columns);
            // a small B is converted in line (the hand-over would cost more than it overlaps)
            tiles_aside = B->nnz >= TILES_ASIDE_MIN_NNZ;
            const int rc = tiles_aside ? build_tiles(h, B, &bt, ctl, 0, st, count_tiles, h->cs_tiles,
                                                     h->ev_tiles_start, h->ev_tiles_done)
                                       : build_tiles(h, B, &bt, ctl, 0, st, count_tiles);
            if (rc) {
                if (tiles_aside) cudaStreamWaitEvent(st, h->ev_tiles_done, 0);
                return rc;
            }
            own_tiles = true;
            launches += 5;
        }
        Btd = DevTiles{bt.tile_ptr, bt.tile_col, reinterpret_cast<const unsigned long long *>(bt.mask), bt.tile_off};
        if (ev_tiles) cudaEventRecord(ev_tiles, tiles_aside ? h->cs_tiles : st);
        CKR(palloc(&ri.prod, (size_t)M, st));
        CKR(palloc(&ri.tmin, (size_t)M, st));
        CKR(palloc(&ri.tmax, (size_t)M, st));
        CKR(palloc(&ri.bins, (size_t)M * NBIN, st));
        CKR(palloc(&ri.cls, (size_t)M, st));
        CKR(palloc(&ri.bin_cnt, bin_scratch_ints(M), st));
        CKR(palloc(&ri.cnnz, (size_t)M + 1, st));
        CKR(palloc(&scan_tmp, scan_tmp_ints(M), st));
        if (store) {
            CKR(grow_arena());
            ri.store = 1;
            if (h->arena_cap > 0) {
                CKR(palloc(&ts_off, (size_t)M, st));
                CKR(palloc(&ts_cnt, (size_t)M, st));
                CKR(palloc(&ts_nwin, (size_t)M, st));
                CKR(cudaMemsetAsync(ts_nwin, 0, sizeof(int) * (size_t)M, st));
                if (reserve_windows) CKR(palloc(&ts_wbase, (size_t)M + 1, st));
                have_store = true;
            }
        }
        launch_bounds(Ad, Bd, ri, ctl, grid_rows(h), scan_tmp, st);
        launches += 6;  // bounds + binning
        // everything after this reads B's tiles
        if (tiles_aside) CKR(cudaStreamWaitEvent(st, h->ev_tiles_done, 0));
        CKR(cudaGetLastError());
        return HSMU_OK;
    }

    cudaError_t grow_arena() {
        if (h->arena_want <= h->arena_cap) return cudaSuccess;
        const long long want = std::min(h->arena_want, STORE_MAX_TILES);
        pfree(h->arena_col, st);
        pfree(h->arena_ent, st);
        h->arena_cap = 0;
        // 4 ints of slack: the value pass fetches a window's tile ids in 16-byte units
        cudaError_t e = palloc(&h->arena_col, (size_t)want + 4, st);
        if (e == cudaSuccess) e = palloc(&h->arena_ent, (size_t)want, st);
        if (e != cudaSuccess) {
            pfree(h->arena_col, st);
            pfree(h->arena_ent, st);
            h->arena_want = 0;
            return e;
        }
        h->arena_cap = want;
        return cudaSuccess;
    }

    // exact count of every row (the large rows' tiles kept in the arena while it lasts),
    // scan into C's row pointers and nnz(C), one host read
    int count_scan(int32_t *host_rp, long long *host_prod = nullptr) {
        CKR(palloc(&crp, (size_t)M + 1, st));
        launch_count_small(Ad, Bd, Btd, ri, ctl, h->nsm, st);
        const TileStore tsd = store_view();
        launch_count_large(Ad, Btd, ri, have_store ? &tsd : nullptr, ctl, h->nsm, st);
        if (have_store && ts_wbase) {
            // the listed rows' windows in row order, ahead of every other window: the value
            // pass hands windows out in array order, and R-MAT's heaviest rows come first
            launch_scan(ts_nwin, ts_wbase, M, &ctl->win_listed, scan_tmp, ctl, st);
            CKR(cudaMemcpyAsync(&ctl->win_count, ts_wbase + M, sizeof(int), cudaMemcpyDeviceToDevice, st));
            launches += 3;
        }
        launch_scan(ri.cnnz, crp, M, &ctl->nnz, scan_tmp, ctl, st);
        launches += 6;  // count 3, scan 3
        CKR(cudaGetLastError());
        CKR(cudaMemcpyAsync(h->h_ctl, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
        if (host_rp) CKR(cudaMemcpyAsync(host_rp, crp, sizeof(int32_t) * ((size_t)M + 1), cudaMemcpyDeviceToHost, st));
        if (host_prod && M > 0) {
            const size_t nch = ((size_t)M + PROD_CHUNK - 1) / PROD_CHUNK;
            CKR(palloc(&chunk_prod, nch, st));
            launch_chunk_prod(M, ri.prod, chunk_prod, grid_rows(h), st);
            launches++;
            CKR(cudaMemcpyAsync(host_prod, chunk_prod, sizeof(long long) * nch, cudaMemcpyDeviceToHost, st));
        }
        CKR(cudaStreamSynchronize(st));
        hc = *h->h_ctl;
        if (ri.store && hc.store_tiles > h->arena_want) h->arena_want = hc.store_tiles;  // for the next call
        if (hc.err) return err_from_dev(hc.err);
        if (hc.nnz > INT_MAX) return HSMU_ERR_OVERFLOW;
        win_cap = (long long)hc.win_bound;
        if (win_cap > INT_MAX) return HSMU_ERR_OVERFLOW;
        return HSMU_OK;
    }

    int alloc_output() {
        if (ext_col) {
            ccol = ext_col;
            cval = ext_val;
        } else {
            CKR(palloc(&ccol, (size_t)hc.nnz + COL_PAD, st));
            CKR(palloc(&cval, (size_t)hc.nnz, st));
        }
        CKR(palloc(&win, (size_t)win_cap, st));
        if (hc.bin_count[BIN_L] == 0 && hc.wide_rows == 0) return HSMU_OK;  // no windows
        return alloc_cursors(win_cap, (long long)hc.cur_bound);
    }

    int alloc_cursors(long long nwin, long long cap) {
        if (nwin == 0) return HSMU_OK;
        wc.cap = cap;
        CKR(palloc(&wc.len, (size_t)nwin, st));
        CKR(palloc(&wc.off, (size_t)nwin + 1, st));
        CKR(palloc(&wc.total, 2, st));
        CKR(palloc(&wc.scan_tmp, scan_tmp_ints((int)nwin), st));
        CKR(palloc(&wc.item_off, (size_t)nwin + 1, st));
        CKR(palloc(&wc.cur, (size_t)cap, st));
        return HSMU_OK;
    }

    TileStore store_view() const {
        return TileStore{ts_off,        ts_cnt,       ts_nwin,       reserve_windows ? ts_wbase : nullptr,
                         h->arena_col, h->arena_ent, h->arena_cap,
                         (int)(hc.store_used <= h->arena_cap)};
    }

    // sorted columns of rows lo..hi-1, values of warp-sized rows, numeric windows of the others
    void structure(int lo, int hi) {
        if (hc.nnz == 0) return;
        const TileStore tsd = store_view();
        launch_structure(Ad, Bd, Btd, ri, RowOut{OUT_PLAIN, crp, nullptr, ccol, cval, nullptr, nullptr, lo, hi}, win,
                         win_cap, ctl, o.arith, h->nsm, st, hc.bin_count, have_store ? &tsd : nullptr);
        for (int b = 0; b < NBIN; b++) launches += hc.bin_count[b] > 0;
    }

    // values of the windows made by the preceding structure() call (none unless a row
    // of the large class or a warp row above FUSE_CAP exists)
    void values() {
        if (hc.nnz == 0 || win_cap == 0 || (hc.bin_count[BIN_L] == 0 && hc.wide_rows == 0)) return;
        const TileStore tsd = store_view();
        launch_numeric(Ad, Bd, Btd, crp, ccol, cval, win, win_cap, nullptr, nullptr, nullptr, wc, ctl, o.arith, h->nsm,
                       st, o.wait_polls, have_store ? &tsd : nullptr);
        launches += 9;  // window lengths, two scans of 3, cursors, values
    }

    // start a new panel: its windows reuse the window buffer from slot 0
    int next_panel() {
        CKR(cudaMemsetAsync(&ctl->win_count, 0, sizeof(int), st));
        return HSMU_OK;
    }

    // completion + device-side checks
    int finish() {
        CKR(cudaGetLastError());
        CKR(cudaMemcpyAsync(h->h_ctl, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
        CKR(cudaStreamSynchronize(st));
        hc = *h->h_ctl;
        return hc.err ? err_from_dev(hc.err) : HSMU_OK;
    }

    void release() {
        pfree(ctl, st);
        if (own_tiles) {
            pfree(bt.tile_ptr, st);
            pfree(bt.tile_col, st);
            pfree(bt.mask, st);
            pfree(bt.tile_off, st);
            own_tiles = false;
        }
        pfree(ri.prod, st);
        pfree(chunk_prod, st);
        pfree(ri.tmin, st);
        pfree(ri.tmax, st);
        pfree(ri.bins, st);
        pfree(ri.cls, st);
        pfree(ri.bin_cnt, st);
        pfree(ri.cnnz, st);
        pfree(ts_off, st);
        pfree(ts_cnt, st);
        pfree(ts_nwin, st);
        pfree(ts_wbase, st);
        have_store = false;
        pfree(scan_tmp, st);
        pfree(win, st);
        pfree(wc.len, st);
        pfree(wc.off, st);
        pfree(wc.total, st);
        pfree(wc.scan_tmp, st);
        pfree(wc.item_off, st);
        pfree(wc.cur, st);
        pfree(crp, st);
        if (ext_col) {
            ccol = nullptr;
            cval = nullptr;
        }
        pfree(ccol, st);
        pfree(cval, st);
    }
};

void fill_stats(hsmu_handle_s *h, const PlainRun &r, const hsmu_btiles *Bt_in, hsmu_stats *stats) {
    float t;
    stats->products = r.hc.products;
    stats->nnz_c = r.hc.nnz;
    stats->ntiles_b = Bt_in ? Bt_in->ntiles : r.hc.ntiles;
    stats->windows = r.hc.win_count;
    cudaEventElapsedTime(&t, h->ev[0], h->ev[1]);
    stats->ms_convert = t;
    cudaEventElapsedTime(&t, h->ev[1], h->ev[2]);
    stats->ms_symbolic = t;
    cudaEventElapsedTime(&t, h->ev[2], h->ev[3]);
    stats->ms_alloc = t;
    cudaEventElapsedTime(&t, h->ev[3], h->ev[4]);
    stats->ms_structure = t;
    cudaEventElapsedTime(&t, h->ev[4], h->ev[5]);
    stats->ms_numeric = t;
    cudaEventElapsedTime(&t, h->ev[0], h->ev[5]);
    stats->ms_total = t;
    stats->launches = r.launches;
}

int spgemm_impl(hsmu_handle_s *h, const hsmu_csr *A, const hsmu_csr *B, const hsmu_btiles *Bt_in, hsmu_csr *C,
                const hsmu_opts *opts, cudaStream_t st, hsmu_stats *stats) {
    if (!h || !csr_ok(A) || !csr_ok(B) || !C) return HSMU_ERR_INVALID;
    if (A->N != B->M) return HSMU_ERR_INVALID;
    if (Bt_in && (Bt_in->M != B->M || Bt_in->N != B->N || !Bt_in->tile_ptr)) return HSMU_ERR_INVALID;
    hsmu_opts o{};
    if (opts) o = *opts;
    if (!arith_ok(o)) return HSMU_ERR_INVALID;
    std::memset(C, 0, sizeof(*C));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        cudaEventRecord(h->ev[0], st);
    }
    PlainRun r(h, st, o);
    int rc = r.begin(A, B);
    if (!rc) rc = r.symbolic(B, Bt_in, stats != nullptr, nullptr, stats ? h->ev[1] : nullptr);
    if (!rc && stats) cudaEventRecord(h->ev[2], st);
    if (!rc) rc = r.alloc_output();
    if (!rc) {
        if (stats) cudaEventRecord(h->ev[3], st);
        r.structure(0, A->M);
        if (stats) cudaEventRecord(h->ev[4], st);
        r.values();
        if (stats) cudaEventRecord(h->ev[5], st);
        rc = r.finish();
    }
    if (rc != HSMU_OK) {
        r.release();
        cudaStreamSynchronize(st);
        return rc;
    }
    C->M = A->M;
    C->N = B->N;
    C->nnz = (int32_t)r.hc.nnz;
    C->owned = 1;
    C->row_ptr = r.crp;
    C->col = r.ccol;
    C->val = r.cval;
    r.crp = nullptr;
    r.ccol = nullptr;
    r.cval = nullptr;
    if (stats) fill_stats(h, r, Bt_in, stats);
    return HSMU_OK;
}

// Host-buffer product with the output copy pipelined behind the compute.
//   copy stream in:  values of B (and A), while tiles/bounds/count run on `st`
//   st:              symbolic pass, one host read (nnz and the row pointers,
//                    straight into C->row_ptr), then row panels of about
//                    equal nnz: structure + values of panel q
//   copy stream out: columns and values of panel q while panel q+1 computes
// (Stores from the kernels straight into page-locked host memory measured
// 2.8x slower than this on GB300: the fused kernel's row-sized writes go out
// over the CPU link at a fraction of its copy bandwidth.)
// The result is the same as hsmu_spgemm followed by a download.
// Order of the row panels (cut: np + 1 row bounds; rp: C's row pointers on the host):
// the order of a two-stage flow shop (compute, then the copy back) that ends first,
// by S. M. Johnson's rule (1954) -- panels whose copy is the longer part first, by
// increasing compute, then the others by decreasing copy.  A panel's compute is
// counted in intermediate products (chunk: the products of every PROD_CHUNK rows,
// a chunk cut by a panel bound shared by row count; nullable: row order), its copy
// in output bytes / HOST_LINK_BOUND.
std::vector<int> panel_order(const std::vector<int> &cut, const int32_t *rp, const long long *chunk, int M) {
    const int np = (int)cut.size() - 1;
    std::vector<int> order((size_t)np);
    for (int q = 0; q < np; q++) order[(size_t)q] = q;
    if (!chunk || np < 2) return order;
    // products of rows [0, r): whole chunks, then the share of the chunk that r cuts
    auto before = [&](int r, long long &c_at, double &acc_at) -> double {
        const long long c = r / PROD_CHUNK;
        for (; c_at < c; c_at++) acc_at += (double)chunk[c_at];
        const int rows = (int)std::min<long long>(PROD_CHUNK, (long long)M - c * PROD_CHUNK);
        return acc_at + (r % PROD_CHUNK && rows > 0 ? (double)chunk[c] * (r % PROD_CHUNK) / rows : 0.0);
    };
    std::vector<double> comp((size_t)np), copy((size_t)np);
    long long c_at = 0;
    double acc_at = 0.0, prev = 0.0;
    for (int q = 0; q < np; q++) {
        const double upto = before(cut[(size_t)q + 1], c_at, acc_at);
        comp[(size_t)q] = upto - prev;
        prev = upto;
        copy[(size_t)q] = 12.0 * (double)(rp[cut[(size_t)q + 1]] - rp[cut[(size_t)q]]) / HOST_LINK_BOUND;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const bool la = comp[(size_t)a] < copy[(size_t)a], lb = comp[(size_t)b] < copy[(size_t)b];
        if (la != lb) return la;
        return la ? comp[(size_t)a] < comp[(size_t)b] : copy[(size_t)a] > copy[(size_t)b];
    });
    return order;
}

// The host-buffer call's row panels: cut (np + 1 row bounds, panel q = rows
// [cut[q], cut[q+1]), each ending at the first row whose entries start at or
// after the panel's share of nnz) and the order they run in (panel_order).
// rp: C's row pointers (M + 1); products: the product's intermediate products;
// chunk: products per PROD_CHUNK rows (nullable); panels: hsmu_opts.panels.
void plan_panels(int M, const int32_t *rp, long long products, const long long *chunk, int panels,
                 std::vector<int> &cut, std::vector<int> &order) {
    const long long nnz = rp[M];
    long long np = panels > 0 ? panels : (nnz * 12 + HOST_PANEL_BYTES - 1) / HOST_PANEL_BYTES;
    np = np < 1 ? 1 : (np > HOST_MAX_PANELS ? HOST_MAX_PANELS : np);
    if (np > M) np = M > 0 ? M : 1;
    cut.assign(1, 0);
    const bool link_bound = 12.0 * (double)nnz > HOST_LINK_BOUND * (double)products;
    std::vector<double> share((size_t)np);
    double wsum = 0.0;
    for (long long q = 0; q < np; q++)
        wsum += (share[q] = link_bound ? std::pow(HOST_PANEL_GROWTH, (double)std::min(q, np - 1 - q))
                                       : std::pow(HOST_PANEL_RATIO, (double)q));
    double acc = 0.0;
    for (long long q = 1; q < np; q++) {
        acc += share[q - 1];
        const long long target = (long long)((double)nnz * (acc / wsum));
        const int row = (int)(std::lower_bound(rp, rp + M + 1, (int32_t)target) - rp);
        cut.push_back(row < cut.back() ? cut.back() : (row > M ? M : row));
    }
    cut.push_back(M);
    order = panel_order(cut, rp, chunk, M);
}

int spgemm_host_impl(hsmu_handle_s *h, const hsmu_csr *A, const hsmu_csr *B, hsmu_csr *C, const hsmu_opts *opts,
                     cudaStream_t st, hsmu_stats *stats) {
    if (!h || !csr_ok(A) || !csr_ok(B) || !C || !C->row_ptr) return HSMU_ERR_INVALID;
    if (A->N != B->M || C->nnz < 0 || (C->nnz > 0 && (!C->col || !C->val))) return HSMU_ERR_INVALID;
    hsmu_opts o{};
    if (opts) o = *opts;
    if (!arith_ok(o) || o.panels < 0) return HSMU_ERR_INVALID;
    const long long capacity = C->nnz;
    const bool same = A->row_ptr == B->row_ptr && A->col == B->col && A->val == B->val && A->M == B->M &&
                      A->N == B->N && A->nnz == B->nnz;
    const int M = A->M;
    int rc = HSMU_OK;
    hsmu_csr dA{}, dB{};
    PlainRun r(h, st, o);
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        cudaEventRecord(h->ev[0], st);
    }
    auto upload = [&](const hsmu_csr *X, hsmu_csr *D) -> int {
        *D = *X;
        D->owned = 0;
        D->row_ptr = nullptr;
        D->col = nullptr;
        D->val = nullptr;
        CKR(palloc(&D->row_ptr, (size_t)X->M + 1, st));
        CKR(palloc(&D->col, (size_t)X->nnz, st));
        CKR(palloc(&D->val, (size_t)X->nnz, st));
        // index arrays on st (the symbolic pass needs them first) ...
        CKR(cudaMemcpyAsync(D->row_ptr, X->row_ptr, sizeof(int32_t) * ((size_t)X->M + 1), cudaMemcpyHostToDevice, st));
        if (X->nnz) CKR(cudaMemcpyAsync(D->col, X->col, sizeof(int32_t) * (size_t)X->nnz, cudaMemcpyHostToDevice, st));
        // ... values on the input copy stream, behind the symbolic pass
        CKR(cudaEventRecord(h->ev_in, st));
        CKR(cudaStreamWaitEvent(h->cs_in, h->ev_in, 0));
        if (X->nnz)
            CKR(cudaMemcpyAsync(D->val, X->val, sizeof(double) * (size_t)X->nnz, cudaMemcpyHostToDevice, h->cs_in));
        return HSMU_OK;
    };
    // products per PROD_CHUNK rows, read with the row pointers, order the panels
    // (page-locked, kept by the handle; without it the panels run in row order)
    const size_t nchunk = ((size_t)M + PROD_CHUNK - 1) / PROD_CHUNK;
    if (nchunk > 0 && h->h_prod_cap < nchunk) {
        if (h->h_prod) cudaFreeHost(h->h_prod);
        h->h_prod = nullptr;
        h->h_prod_cap = 0;
        if (cudaMallocHost(reinterpret_cast<void **>(&h->h_prod), sizeof(long long) * nchunk) == cudaSuccess)
            h->h_prod_cap = nchunk;
        else
            h->h_prod = nullptr, (void)cudaGetLastError();
    }
    long long *host_prod = nchunk > 0 && h->h_prod_cap >= nchunk ? h->h_prod : nullptr;
    std::vector<int> cut;
    r.reserve_windows = false;  // the output is written in row panels
    rc = upload(B, &dB);
    if (!rc) {
        if (same) dA = dB;
        else rc = upload(A, &dA);
    }
    if (!rc) CK(cudaEventRecord(h->ev_in, h->cs_in));
    if (!rc) rc = r.begin(&dA, &dB);
    if (!rc) rc = r.symbolic(&dB, nullptr, stats != nullptr, C->row_ptr, stats ? h->ev[1] : nullptr, host_prod);
    if (!rc && stats) cudaEventRecord(h->ev[2], st);
    if (!rc && r.hc.nnz > capacity) {
        // report the size; the row pointers are already in C->row_ptr
        C->M = M;
        C->N = B->N;
        C->nnz = (int32_t)r.hc.nnz;
        rc = HSMU_ERR_CAPACITY;
    }
    if (!rc) rc = r.alloc_output();
    if (!rc) {
        if (stats) cudaEventRecord(h->ev[3], st);
        CK(cudaStreamWaitEvent(st, h->ev_in, 0));  // values of A and B are on the device
        std::vector<int> order;
        plan_panels(M, C->row_ptr, (long long)r.hc.products, host_prod, o.panels, cut, order);
        bool first = true;
        for (const int q : order) {
            const int lo = cut[q], hi = cut[q + 1];
            if (lo == hi) continue;
            if (!first) {
                rc = r.next_panel();
                if (rc) break;
            }
            first = false;
            const long long e0 = C->row_ptr[lo], e1 = C->row_ptr[hi];
            // the columns are final after the structure pass: their copy starts while the
            // value pass runs
            r.structure(lo, hi);
            if (e1 > e0) {
                CK(cudaEventRecord(h->ev_panel, st));
                CK(cudaStreamWaitEvent(h->cs_out, h->ev_panel, 0));
                CK(cudaMemcpyAsync(C->col + e0, r.ccol + e0, sizeof(int32_t) * (size_t)(e1 - e0),
                                   cudaMemcpyDeviceToHost, h->cs_out));
            }
            r.values();
            if (e1 == e0) continue;
            CK(cudaEventRecord(h->ev_panel, st));
            CK(cudaStreamWaitEvent(h->cs_out, h->ev_panel, 0));
            CK(cudaMemcpyAsync(C->val + e0, r.cval + e0, sizeof(double) * (size_t)(e1 - e0), cudaMemcpyDeviceToHost,
                               h->cs_out));
        }
        if (stats) cudaEventRecord(h->ev[4], st);
        if (!rc) CK(cudaEventRecord(h->ev_out, h->cs_out));
        if (!rc) CK(cudaStreamWaitEvent(st, h->ev_out, 0));
        if (stats) cudaEventRecord(h->ev[5], st);
        if (!rc) rc = r.finish();
    }
done:
    // copies still in flight on the copy streams finish before their buffers go
    cudaStreamSynchronize(h->cs_in);
    cudaStreamSynchronize(h->cs_out);
    r.release();
    if (dA.row_ptr && dA.row_ptr != dB.row_ptr) {
        pfree(dA.row_ptr, st);
        pfree(dA.col, st);
        pfree(dA.val, st);
    }
    pfree(dB.row_ptr, st);
    pfree(dB.col, st);
    pfree(dB.val, st);
    if (rc != HSMU_OK) {
        cudaStreamSynchronize(st);
        return rc;
    }
    C->M = M;
    C->N = B->N;
    C->nnz = (int32_t)r.hc.nnz;
    C->owned = 0;
    if (stats) {
        fill_stats(h, r, nullptr, stats);
        stats->launches = r.launches;
    }
    return HSMU_OK;
}

// Learned path (see learned.cu): predicted slots instead of the exact count pass.
// B's tiles and the bounds pass are shared with the plain path (a PlainRun holds
// them).  What the prediction saves is the count pass of the warp-class rows
// that take numeric windows (more than FUSE_CAP entries): their count is an OR
// walk of its own.  Large rows are counted exactly either way (their count
// builds the tile lists the structure pass streams); for every other row the
// exact count is about as cheap as the prediction, and filling speculative
// slots costs a compaction copy.  So the plain path finishes the product on
// the same tiles and bounds unless warp-class rows of more than FUSE_CAP
// products hold LEARNED_MIN_SHARE of the products (known after the bounds
// pass) and the rows predicted above FUSE_CAP entries hold as much (known
// after the prediction).  Either way the output is the plain path's, bit for
// bit.
int spgemm_learned_impl(hsmu_handle_s *h, const hsmu_csr *A, const hsmu_csr *B, hsmu_csr *C, const hsmu_mlp *model,
                        const hsmu_opts *opts, cudaStream_t st, hsmu_stats *stats) {
    if (!h || !csr_ok(A) || !csr_ok(B) || !C || !model || !model->params) return HSMU_ERR_INVALID;
    if (A->N != B->M) return HSMU_ERR_INVALID;
    hsmu_opts o{};
    if (opts) o = *opts;
    if (o.arith < HSMU_ARITH_RN || o.arith > HSMU_ARITH_IMUL) return HSMU_ERR_INVALID;
    const int M = A->M;
    int rc = HSMU_OK;
    int *cap = nullptr, *crp = nullptr, *ccol = nullptr, *scol = nullptr;
    long long *soff = nullptr;
    float4 *feat = nullptr;
    unsigned char *flag = nullptr;
    double *cval = nullptr, *sval = nullptr;
    Window *win = nullptr;
    long long win_cap = 0, spec_total = 0, cur_cap = 0;
    WinCursors wc{};
    Ctl hc{};
    std::memset(C, 0, sizeof(*C));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        cudaEventRecord(h->ev[0], st);
    }
    PlainRun r(h, st, o);
    rc = r.begin(A, B);
    if (!rc) rc = r.tiles_bounds(B, nullptr, stats != nullptr, stats ? h->ev[1] : nullptr, o.no_tile_store == 0);
    if (rc) goto done;
    CK(cudaMemcpyAsync(h->h_ctl, r.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    hc = *h->h_ctl;
    if (hc.err) {
        rc = err_from_dev(hc.err);
        goto done;
    }
    // what the prediction can save is the count pass of warp-class rows that need numeric
    // windows: with few products in warp-class rows of more than FUSE_CAP products, the plain
    // path finishes on the same tiles and bounds (large rows are counted exactly either way:
    // their count builds their tile lists)
    if (!o.learned_always &&
        (hc.products == 0 || (double)hc.wide_ds_prod < LEARNED_MIN_SHARE * (double)hc.products))
        goto plain;
    {
        // the large rows' tile lists: the arena is sized now, from what earlier calls needed
        // or else from the bounds pass's bound (the sum of the large rows' tile spans)
        if (r.ri.store && hc.bin_count[BIN_L] > 0) {
            if (h->arena_want == 0) h->arena_want = hc.span_tiles;
            CK(r.grow_arena());
            if (h->arena_cap > 0 && !r.ts_off) {
                CK(palloc(&r.ts_off, (size_t)M, st));
                CK(palloc(&r.ts_cnt, (size_t)M, st));
                CK(palloc(&r.ts_nwin, (size_t)M, st));
                CK(cudaMemsetAsync(r.ts_nwin, 0, sizeof(int) * (size_t)M, st));
                CK(palloc(&r.ts_wbase, (size_t)M + 1, st));
            }
            r.have_store = h->arena_cap > 0;
        }
        CK(palloc(&feat, (size_t)M, st));
        CK(palloc(&cap, (size_t)M + 1, st));
        CK(palloc(&soff, (size_t)M + 1, st));
        launch_features(r.Ad, r.Bd, feat, nullptr, h->nsm, st);
        // large rows with a tile list need no slot (they are written at their place in C)
        launch_capacity(model->params, feat, r.ri.prod, r.ri.cls, M, B->N, model->margin, cap, h->nsm, st,
                        &r.ctl->pred_wide_prod, r.have_store);
        launch_scan64(cap, soff, M, &r.ctl->nnz, r.scan_tmp, st);  // nnz field holds the slot total for now
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(h->h_ctl, r.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        hc = *h->h_ctl;
        if (hc.err) {
            rc = err_from_dev(hc.err);
            goto done;
        }
        if (!o.learned_always && (double)hc.pred_wide_prod < LEARNED_MIN_SHARE * (double)hc.products) goto plain;
        goto learned;
    }
plain:
    {
        // the plain path on the same tiles and bounds
        CK(cudaMemsetAsync(&r.ctl->nnz, 0, sizeof(long long), st));
        rc = r.count_scan(nullptr);
        if (!rc && stats) cudaEventRecord(h->ev[2], st);
        if (!rc) rc = r.alloc_output();
        if (!rc) {
            if (stats) cudaEventRecord(h->ev[3], st);
            r.structure(0, M);
            if (stats) cudaEventRecord(h->ev[4], st);
            r.values();
            if (stats) cudaEventRecord(h->ev[5], st);
            rc = r.finish();
        }
        if (rc) goto done;
        C->M = M;
        C->N = B->N;
        C->nnz = (int32_t)r.hc.nnz;
        C->owned = 1;
        C->row_ptr = r.crp;
        C->col = r.ccol;
        C->val = r.cval;
        r.crp = nullptr;
        r.ccol = nullptr;
        r.cval = nullptr;
        if (stats) {
            fill_stats(h, r, nullptr, stats);
            stats->routed = 1;
        }
        goto done;
    }
learned:
    {
        Ctl *ctl = r.ctl;
        const DevCSR &Ad = r.Ad, &Bd = r.Bd;
        const DevTiles &Btd = r.Btd;
        RowInfo &ri = r.ri;
        CK(palloc(&flag, (size_t)M, st));
        CK(cudaMemsetAsync(flag, 0, (size_t)M, st));
        if (stats) cudaEventRecord(h->ev[2], st);
        spec_total = hc.nnz;
        win_cap = 2 * (long long)hc.win_bound;  // speculative pass + redo of overflowing rows
        if (win_cap > INT_MAX) {
            rc = HSMU_ERR_OVERFLOW;
            goto done;
        }
        CK(palloc(&scol, (size_t)spec_total + COL_PAD, st));
        CK(palloc(&sval, (size_t)spec_total, st));
        CK(palloc(&win, (size_t)win_cap, st));
        CK(palloc(&crp, (size_t)M + 1, st));
        // cursors of the windows of both passes (no exact count pass: every warp row above FUSE_CAP products)
        cur_cap = 2 * (long long)(hc.cur_bound + hc.cur_bound_ds);
        if (win_cap > 0) {
            wc.cap = cur_cap;
            CK(palloc(&wc.len, (size_t)win_cap, st));
            CK(palloc(&wc.off, (size_t)win_cap + 1, st));
            CK(palloc(&wc.total, 2, st));
            CK(palloc(&wc.scan_tmp, scan_tmp_ints((int)win_cap), st));
            CK(palloc(&wc.item_off, (size_t)win_cap + 1, st));
            CK(palloc(&wc.cur, (size_t)cur_cap, st));
        }
        if (stats) cudaEventRecord(h->ev[3], st);
        // structure (+ values of warp-sized rows) into the slots; exact counts found here.
        // Large rows with a tile list: exact count and list now, written at their place in
        // C by the redo pass (the prediction has nothing to skip for them: their count pass
        // builds the list the structure pass streams).
        const RowOut spec{OUT_SPEC, nullptr, soff, scol, sval, ri.cnnz, flag, 0, M};
        // The listed large rows' windows are placed first, in row order (scan of their
        // counts), before any warp row's window: the value pass hands windows out in array
        // order, and R-MAT's heaviest rows come first.  The redo pass then streams those rows
        // without barriers.
        TileStore tsd{r.ts_off, r.ts_cnt, r.ts_nwin, r.ts_wbase, h->arena_col, h->arena_ent,
                      h->arena_cap, 0};
        const int small_rows[NBIN] = {hc.bin_count[BIN_DS], 0, hc.bin_count[BIN_TINY]};
        const int large_rows[NBIN] = {0, hc.bin_count[BIN_L], 0};
        if (hc.bin_count[BIN_L] > 0 && r.have_store) {
            launch_spec_large(Ad, Btd, ri, tsd, spec, ctl, h->nsm, st);
            launch_scan(r.ts_nwin, r.ts_wbase, M, &ctl->win_listed, r.scan_tmp, ctl, st);
            CK(cudaMemcpyAsync(&ctl->win_count, r.ts_wbase + M, sizeof(int), cudaMemcpyDeviceToDevice, st));
        }
        launch_structure(Ad, Bd, Btd, ri, spec, win, win_cap, ctl, o.arith, h->nsm, st, small_rows);
        if (hc.bin_count[BIN_L] > 0)
            launch_structure(Ad, Bd, Btd, ri, spec, win, win_cap, ctl, o.arith, h->nsm, st, large_rows,
                             r.have_store ? &tsd : nullptr);
        launch_scan(ri.cnnz, crp, M, &ctl->nnz, r.scan_tmp, ctl, st);
        // exact nnz(C): rows that overflowed their slot can make it larger than the slot total
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(h->h_ctl, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        hc = *h->h_ctl;
        if (hc.err) {
            rc = err_from_dev(hc.err);
            goto done;
        }
        if (r.ri.store && hc.store_tiles > h->arena_want) h->arena_want = hc.store_tiles;  // for the next call
        if (hc.nnz > INT_MAX) {
            rc = HSMU_ERR_OVERFLOW;
            goto done;
        }
        CK(palloc(&ccol, (size_t)hc.nnz + COL_PAD, st));
        CK(palloc(&cval, (size_t)hc.nnz, st));
        launch_compact(M, soff, crp, flag, scol, sval, ccol, cval, h->nsm, st);
        launch_structure(Ad, Bd, Btd, ri, RowOut{OUT_REDO, crp, nullptr, ccol, cval, nullptr, flag, 0, M}, win,
                         win_cap, ctl, o.arith, h->nsm, st, nullptr, r.have_store ? &tsd : nullptr);
        if (stats) cudaEventRecord(h->ev[4], st);
        launch_numeric(Ad, Bd, Btd, crp, ccol, cval, win, win_cap, flag, scol, soff, wc, ctl, o.arith, h->nsm, st,
                       o.wait_polls, r.have_store ? &tsd : nullptr);
        CK(cudaGetLastError());
        if (stats) cudaEventRecord(h->ev[5], st);
        CK(cudaMemcpyAsync(h->h_ctl, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        hc = *h->h_ctl;
        if (hc.err) {
            rc = err_from_dev(hc.err);
            goto done;
        }
        if (hc.nnz > INT_MAX) {
            rc = HSMU_ERR_OVERFLOW;
            goto done;
        }
    }
    C->M = M;
    C->N = B->N;
    C->nnz = (int32_t)hc.nnz;
    C->owned = 1;
    C->row_ptr = crp;
    C->col = ccol;
    C->val = cval;
    crp = nullptr;
    ccol = nullptr;
    cval = nullptr;
    if (stats) {
        float t;
        stats->products = hc.products;
        stats->nnz_c = hc.nnz;
        stats->ntiles_b = hc.ntiles;
        stats->windows = hc.win_count;
        stats->spec_capacity = spec_total;
        stats->fallback_rows = hc.fallback;
        cudaEventElapsedTime(&t, h->ev[0], h->ev[1]);
        stats->ms_convert = t;
        cudaEventElapsedTime(&t, h->ev[1], h->ev[2]);
        stats->ms_symbolic = t;
        cudaEventElapsedTime(&t, h->ev[2], h->ev[3]);
        stats->ms_alloc = t;
        cudaEventElapsedTime(&t, h->ev[3], h->ev[4]);
        stats->ms_structure = t;
        cudaEventElapsedTime(&t, h->ev[4], h->ev[5]);
        stats->ms_numeric = t;
        cudaEventElapsedTime(&t, h->ev[0], h->ev[5]);
        stats->ms_total = t;
        // tiles 5, bounds + binning 6, features 1, capacity 1, scan 3, structure 3, scan 3, compact 1, redo 3,
        // window lengths 1, their two scans 6, cursors 1, numeric 1
        stats->launches = (o.validate ? 2 : 0) + (win_cap > 0 ? 35 : 27);
    }
done:
    pfree(feat, st);
    pfree(cap, st);
    pfree(soff, st);
    pfree(flag, st);
    pfree(scol, st);
    pfree(sval, st);
    pfree(win, st);
    pfree(wc.len, st);
    pfree(wc.off, st);
    pfree(wc.total, st);
    pfree(wc.scan_tmp, st);
    pfree(wc.item_off, st);
    pfree(wc.cur, st);
    pfree(crp, st);
    pfree(ccol, st);
    pfree(cval, st);
    r.release();
    if (rc != HSMU_OK) cudaStreamSynchronize(st);
    return rc;
}

// exact nnz of every row of A*B through the symbolic pass (training labels)
int row_nnz_impl(hsmu_handle_s *h, const hsmu_csr *A, const hsmu_csr *B, int32_t *nnz_out, cudaStream_t st) {
    if (!h || !csr_ok(A) || !csr_ok(B) || !nnz_out || A->N != B->M) return HSMU_ERR_INVALID;
    const int M = A->M;
    int rc = HSMU_OK;
    Ctl *ctl = nullptr;
    hsmu_btiles bt{};
    RowInfo ri{};
    int *scan_tmp = nullptr;
    DevCSR Ad = dev(A), Bd = dev(B);
    DevTiles Btd{};
    CK(palloc(&ctl, 1, st));
    CK(cudaMemsetAsync(ctl, 0, sizeof(Ctl), st));
    rc = build_tiles(h, B, &bt, ctl, 0, st, false);
    if (rc) goto done;
    Btd = DevTiles{bt.tile_ptr, bt.tile_col, reinterpret_cast<const unsigned long long *>(bt.mask), bt.tile_off};
    CK(palloc(&ri.prod, (size_t)M, st));
    CK(palloc(&ri.tmin, (size_t)M, st));
    CK(palloc(&ri.tmax, (size_t)M, st));
    CK(palloc(&ri.bins, (size_t)M * NBIN, st));
    CK(palloc(&ri.cls, (size_t)M, st));
    CK(palloc(&ri.bin_cnt, bin_scratch_ints(M), st));
    CK(palloc(&scan_tmp, scan_tmp_ints(M), st));
    ri.cnnz = nnz_out;
    launch_bounds(Ad, Bd, ri, ctl, grid_rows(h), scan_tmp, st);
    launch_count(Ad, Bd, Btd, ri, ctl, h->nsm, st);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h->h_ctl, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (h->h_ctl->err) rc = err_from_dev(h->h_ctl->err);
done:
    pfree(ctl, st);
    pfree(bt.tile_ptr, st);
    pfree(bt.tile_col, st);
    pfree(bt.mask, st);
    pfree(bt.tile_off, st);
    pfree(ri.prod, st);
    pfree(ri.tmin, st);
    pfree(ri.tmax, st);
    pfree(ri.bins, st);
    pfree(ri.cls, st);
    pfree(ri.bin_cnt, st);
    pfree(scan_tmp, st);
    if (rc != HSMU_OK) cudaStreamSynchronize(st);
    return rc;
}

// hsmu_spgemm64: exact nnz of every row, int64 row pointers (device scan, one host read of
// them), then panels of consecutive rows whose entries fit int32, each run by the plain
// engine straight into its place in C; B's tiles are built once for all panels
int spgemm64_impl(hsmu_handle_s *h, const hsmu_csr *A, const hsmu_csr *B, hsmu_csr64 *C, long long max_panel,
                  const hsmu_opts *opts, cudaStream_t st) {
    if (!h || !csr_ok(A) || !csr_ok(B) || !C || A->N != B->M || max_panel < 0) return HSMU_ERR_INVALID;
    hsmu_opts o{};
    if (opts) o = *opts;
    if (!arith_ok(o)) return HSMU_ERR_INVALID;
    std::memset(C, 0, sizeof(*C));
    const long long cap = (max_panel == 0 || max_panel > INT_MAX) ? INT_MAX : max_panel;
    const int M = A->M;
    int rc = HSMU_OK;
    int *cnt = nullptr, *scan_tmp = nullptr, *col = nullptr;
    long long *rp = nullptr, *tot = nullptr;
    double *val = nullptr;
    Ctl *ctl = nullptr;
    hsmu_btiles bt{};
    std::vector<long long> hrp;
    hsmu_opts po = o;
    po.validate = 0;  // the panels are views into A: the operands are checked once, here
    if (o.validate) {
        PlainRun v(h, st, o);
        rc = v.begin(A, B);
        v.release();
        if (rc) goto done;
    }
    CK(palloc(&cnt, (size_t)M + 1, st));
    rc = row_nnz_impl(h, A, B, cnt, st);
    if (rc) goto done;
    CK(palloc(&rp, (size_t)M + 1, st));
    CK(palloc(&tot, 1, st));
    CK(palloc(&scan_tmp, scan_tmp_ints(M), st));
    launch_scan64(cnt, rp, M, tot, scan_tmp, st);
    CK(cudaGetLastError());
    hrp.resize((size_t)M + 1);
    CK(cudaMemcpyAsync(hrp.data(), rp, sizeof(long long) * ((size_t)M + 1), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    CK(palloc(&col, (size_t)hrp[M] + COL_PAD, st));
    CK(palloc(&val, (size_t)hrp[M], st));
    CK(palloc(&ctl, 1, st));
    CK(cudaMemsetAsync(ctl, 0, sizeof(Ctl), st));
    rc = build_tiles(h, B, &bt, ctl, 0, st, true);
    if (rc) goto done;
    for (int r0 = 0; r0 < M;) {
        // rows r0 .. r1-1: as many as keep the panel within the cap, at least one
        int r1 = (int)(std::upper_bound(hrp.begin() + r0 + 1, hrp.end(), hrp[r0] + cap) - hrp.begin()) - 1;
        if (r1 <= r0) r1 = r0 + 1;
        hsmu_csr Ap = *A;
        Ap.M = r1 - r0;
        Ap.row_ptr = A->row_ptr + r0;
        PlainRun r(h, st, po);
        r.ext_col = col + hrp[r0];
        r.ext_val = val + hrp[r0];
        rc = r.begin(&Ap, B);
        if (!rc) rc = r.symbolic(B, &bt, false, nullptr, nullptr);
        if (!rc && r.hc.nnz != hrp[r1] - hrp[r0]) rc = HSMU_ERR_INTERNAL;
        if (!rc) rc = r.alloc_output();
        if (!rc) {
            r.structure(0, Ap.M);
            r.values();
            rc = r.finish();
        }
        r.release();
        if (rc) goto done;
        r0 = r1;
    }
    C->M = M;
    C->N = B->N;
    C->nnz = hrp[M];
    C->owned = 1;
    C->row_ptr = reinterpret_cast<int64_t *>(rp);
    C->col = col;
    C->val = val;
    rp = nullptr;
    col = nullptr;
    val = nullptr;
done:
    pfree(cnt, st);
    pfree(scan_tmp, st);
    pfree(tot, st);
    pfree(ctl, st);
    pfree(bt.tile_ptr, st);
    pfree(bt.tile_col, st);
    pfree(bt.mask, st);
    pfree(bt.tile_off, st);
    pfree(rp, st);
    pfree(col, st);
    pfree(val, st);
    cudaStreamSynchronize(st);
    return rc;
}

}  // namespace

extern "C" {

const char *hsmu_strerror(int status) {
    if (status < 0 || status >= (int)(sizeof(kErr) / sizeof(kErr[0]))) return "unknown status";
    return kErr[status];
}

int hsmu_abi_version(void) { return HSMU_ABI_VERSION; }

int hsmu_handle_create(hsmu_handle *out) {
    if (!out) return HSMU_ERR_INVALID;
    *out = nullptr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return HSMU_ERR_NO_DEVICE;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return HSMU_ERR_NO_DEVICE;
    if (prop.major < 10) return HSMU_ERR_NO_DEVICE;
    hsmu_handle_s *h = new (std::nothrow) hsmu_handle_s();
    if (!h) return HSMU_ERR_ALLOC;
    h->device = dev;
    h->nsm = prop.multiProcessorCount;
    if (cudaMallocHost(reinterpret_cast<void **>(&h->h_ctl), sizeof(Ctl)) != cudaSuccess) {
        delete h;
        return HSMU_ERR_ALLOC;
    }

    for (auto &e : h->ev) cudaEventCreate(&e);
    if (cudaStreamCreateWithFlags(&h->cs_in, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->cs_out, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_in, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_panel, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_out, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->cs_tiles, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_tiles_start, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_tiles_done, cudaEventDisableTiming) != cudaSuccess) {
        hsmu_handle_destroy(h);
        return HSMU_ERR_CUDA;
    }
    // keep freed pool memory cached between calls (no re-mapping of large outputs)
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        unsigned long long thr = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    int e = configure_count();
    if (!e) e = configure_structure();
    if (!e) e = configure_numeric();
    if (e) {
        hsmu_handle_destroy(h);
        return HSMU_ERR_CUDA;
    }
    *out = h;
    return HSMU_OK;
}

int hsmu_handle_destroy(hsmu_handle h) {
    if (!h) return HSMU_OK;
    for (auto &e : h->ev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : {h->ev_in, h->ev_panel, h->ev_out, h->ev_tiles_start, h->ev_tiles_done})
        if (e) cudaEventDestroy(e);
    if (h->arena_col || h->arena_ent) {
        cudaDeviceSynchronize();  // no call of this handle still reads the arena
        for (void *p : {(void *)h->arena_col, (void *)h->arena_ent})
            if (p) cudaFreeAsync(p, 0);
        cudaStreamSynchronize(0);
    }
    for (cudaStream_t s : {h->cs_in, h->cs_out, h->cs_tiles})
        if (s) cudaStreamDestroy(s);
    if (h->h_ctl) cudaFreeHost(h->h_ctl);
    if (h->h_prod) cudaFreeHost(h->h_prod);
    delete h;
    return HSMU_OK;
}

int hsmu_spgemm(hsmu_handle h, const hsmu_csr *A, const hsmu_csr *B, hsmu_csr *C, const hsmu_opts *opts,
                void *stream, hsmu_stats *stats) {
    return spgemm_impl(h, A, B, nullptr, C, opts, static_cast<cudaStream_t>(stream), stats);
}

int hsmu_spgemm_host(hsmu_handle h, const hsmu_csr *A, const hsmu_csr *B, hsmu_csr *C, const hsmu_opts *opts,
                     void *stream, hsmu_stats *stats) {
    return spgemm_host_impl(h, A, B, C, opts, static_cast<cudaStream_t>(stream), stats);
}

int hsmu_spgemm_tiled(hsmu_handle h, const hsmu_csr *A, const hsmu_csr *B, const hsmu_btiles *Bt, hsmu_csr *C,
                      const hsmu_opts *opts, void *stream, hsmu_stats *stats) {
    if (!Bt) return HSMU_ERR_INVALID;
    return spgemm_impl(h, A, B, Bt, C, opts, static_cast<cudaStream_t>(stream), stats);
}

int hsmu_spgemm_learned(hsmu_handle h, const hsmu_csr *A, const hsmu_csr *B, hsmu_csr *C, const hsmu_mlp *model,
                        const hsmu_opts *opts, void *stream, hsmu_stats *stats) {
    return spgemm_learned_impl(h, A, B, C, model, opts, static_cast<cudaStream_t>(stream), stats);
}

int hsmu_spgemm64(hsmu_handle h, const hsmu_csr *A, const hsmu_csr *B, hsmu_csr64 *C, int64_t max_panel_nnz,
                  const hsmu_opts *opts, void *stream) {
    return spgemm64_impl(h, A, B, C, (long long)max_panel_nnz, opts, static_cast<cudaStream_t>(stream));
}

int hsmu_csr64_free(hsmu_csr64 *C) {
    if (!C) return HSMU_ERR_INVALID;
    if (C->owned) free_owned({C->row_ptr, C->col, C->val});
    std::memset(C, 0, sizeof(*C));
    return HSMU_OK;
}

int hsmu_row_nnz(hsmu_handle h, const hsmu_csr *A, const hsmu_csr *B, int32_t *nnz, void *stream) {
    return row_nnz_impl(h, A, B, nnz, static_cast<cudaStream_t>(stream));
}

int hsmu_btiles_build(hsmu_handle h, const hsmu_csr *B, hsmu_btiles *out, void *stream) {
    if (!h || !csr_ok(B) || !out) return HSMU_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = HSMU_OK;
    Ctl *ctl = nullptr;
    Ctl hc{};
    std::memset(out, 0, sizeof(*out));
    CK(palloc(&ctl, 1, st));
    CK(cudaMemsetAsync(ctl, 0, sizeof(Ctl), st));
    launch_validate(dev(B), ctl, grid_rows(h), st);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h->h_ctl, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (h->h_ctl->err) {
        rc = err_from_dev(h->h_ctl->err);
        goto done;
    }
    rc = build_tiles(h, B, out, ctl, 0, st, true);
    if (rc) goto done;
    CK(cudaMemcpyAsync(h->h_ctl, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    hc = *h->h_ctl;
    if (hc.err) {
        rc = err_from_dev(hc.err);
        hsmu_btiles_free(out);
        goto done;
    }
    out->ntiles = hc.ntiles;
done:
    pfree(ctl, st);
    return rc;
}

int hsmu_btiles_free(hsmu_btiles *t) {
    if (!t) return HSMU_ERR_INVALID;
    free_owned({t->tile_ptr, t->tile_col, t->mask, t->tile_off});
    std::memset(t, 0, sizeof(*t));
    return HSMU_OK;
}

int hsmu_csr_transpose(hsmu_handle h, const hsmu_csr *A, hsmu_csr *At, void *stream) {
    if (!h || !csr_ok(A) || !At) return HSMU_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    std::memset(At, 0, sizeof(*At));
    int rc = HSMU_OK;
    const long long n = A->nnz;
    int *trp = nullptr, *tcol = nullptr, *si = nullptr, *hist = nullptr, *scan_tmp = nullptr;
    double *tval = nullptr, *sd = nullptr;
    long long *tot = nullptr;
    Ctl *ctl = nullptr;
    const long long ntiles_scan = (long long)transpose_hist_ints(n) / 2;
    CK(palloc(&trp, (size_t)A->N + 1, st));
    CK(palloc(&tcol, (size_t)n, st));
    CK(palloc(&tval, (size_t)n, st));
    CK(palloc(&si, transpose_scratch_ints(n), st));
    CK(palloc(&sd, transpose_scratch_doubles(n), st));
    CK(palloc(&hist, transpose_hist_ints(n), st));
    CK(palloc(&scan_tmp, scan_tmp_ints((int)ntiles_scan), st));
    CK(palloc(&tot, 1, st));
    CK(palloc(&ctl, 1, st));
    CK(cudaMemsetAsync(ctl, 0, sizeof(Ctl), st));
    CK((cudaError_t)launch_transpose(dev(A), trp, tcol, tval, si, sd, hist, scan_tmp, tot, ctl, h->nsm, st));
    CK(cudaMemcpyAsync(h->h_ctl, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (h->h_ctl->err) {
        rc = err_from_dev(h->h_ctl->err);
        goto done;
    }
    At->M = A->N;
    At->N = A->M;
    At->nnz = A->nnz;
    At->owned = 1;
    At->row_ptr = trp;
    At->col = tcol;
    At->val = tval;
    trp = tcol = nullptr;
    tval = nullptr;
done:
    pfree(trp, st);
    pfree(tcol, st);
    pfree(tval, st);
    pfree(si, st);
    pfree(sd, st);
    pfree(hist, st);
    pfree(scan_tmp, st);
    pfree(tot, st);
    pfree(ctl, st);
    if (rc != HSMU_OK) cudaStreamSynchronize(st);
    return rc;
}

int hsmu_csr_free(hsmu_csr *C) {
    if (!C) return HSMU_ERR_INVALID;
    if (C->owned) free_owned({C->row_ptr, C->col, C->val});
    std::memset(C, 0, sizeof(*C));
    return HSMU_OK;
}

int hsmu_selftest_dmul(uint64_t n, uint64_t seed, uint64_t *mismatches, void *stream) {
    if (!mismatches) return HSMU_ERR_INVALID;
    unsigned long long m = 0;
    int e = run_dmul_selftest(n, seed, &m, static_cast<cudaStream_t>(stream));
    *mismatches = m;
    return e ? HSMU_ERR_CUDA : HSMU_OK;
}

int hsmu_debug_fail_alloc(int64_t nth) {
    if (nth < 0) return HSMU_ERR_INVALID;
    g_fail_alloc_countdown.store((long long)nth, std::memory_order_relaxed);
    return HSMU_OK;
}

int hsmu_debug_plan_panels(int32_t M, const int32_t *row_ptr, int64_t products, const int64_t *chunk_products,
                           int32_t panels, int32_t *n_panels, int32_t *cut, int32_t *order) {
    if (M < 0 || !row_ptr || panels < 0 || !n_panels || !cut || !order) return HSMU_ERR_INVALID;
    static_assert(sizeof(long long) == sizeof(int64_t), "chunk products");
    std::vector<int> c, ord;
    plan_panels(M, row_ptr, (long long)products, reinterpret_cast<const long long *>(chunk_products), panels, c, ord);
    *n_panels = (int32_t)ord.size();
    for (size_t q = 0; q < c.size(); q++) cut[q] = c[q];
    for (size_t q = 0; q < ord.size(); q++) order[q] = ord[q];
    return HSMU_OK;
}

int hsmu_probe_fp64_rate(int iters, double *lane_ops_per_s, void *stream) {
    if (!lane_ops_per_s || iters <= 0) return HSMU_ERR_INVALID;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return HSMU_ERR_NO_DEVICE;
    return run_fp64_rate(iters, nsm, lane_ops_per_s, static_cast<cudaStream_t>(stream)) ? HSMU_ERR_CUDA : HSMU_OK;
}

int hsmu_csr_download(const hsmu_csr *C, int32_t *row_ptr, int32_t *col, double *val, void *stream) {
    if (!csr_ok(C) || !row_ptr || (C->nnz > 0 && (!col || !val))) return HSMU_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = HSMU_OK;
    CK(cudaMemcpyAsync(row_ptr, C->row_ptr, sizeof(int32_t) * ((size_t)C->M + 1), cudaMemcpyDeviceToHost, st));
    if (C->nnz > 0) {
        CK(cudaMemcpyAsync(col, C->col, sizeof(int32_t) * (size_t)C->nnz, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(val, C->val, sizeof(double) * (size_t)C->nnz, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
done:
    return rc;
}

int hsmu_csr64_download(const hsmu_csr64 *C, int64_t *row_ptr, int32_t *col, double *val, void *stream) {
    if (!C || C->M < 0 || C->nnz < 0 || !C->row_ptr || !row_ptr || (C->nnz > 0 && (!C->col || !C->val || !col || !val)))
        return HSMU_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = HSMU_OK;
    CK(cudaMemcpyAsync(row_ptr, C->row_ptr, sizeof(int64_t) * ((size_t)C->M + 1), cudaMemcpyDeviceToHost, st));
    if (C->nnz > 0) {
        CK(cudaMemcpyAsync(col, C->col, sizeof(int32_t) * (size_t)C->nnz, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(val, C->val, sizeof(double) * (size_t)C->nnz, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
done:
    return rc;
}

}  // extern "C"
