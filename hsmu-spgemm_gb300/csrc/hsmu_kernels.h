// Host-side launch wrappers of the engine's kernels (one translation unit
// per stage; the orchestration in engine.cu only sees these declarations).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace hsmu {

struct Ctl;
struct Window;

struct DevCSR {
    int M, N;
    long long nnz;
    const int *rp;
    const int *col;
    const double *val;
};

struct DevTiles {
    const int *ptr;                  // [K+1]
    const int *col;                  // [T]
    const unsigned long long *mask;  // [T]
    const int *off;                  // [T]
};

// where the structure pass puts each row (see k_structure.cu)
enum OutMode : int { OUT_PLAIN = 0, OUT_SPEC = 1, OUT_REDO = 2 };
enum RowFlag : unsigned char { ROW_NONE = 0, ROW_VALUES = 1, ROW_COLUMNS = 2, ROW_OVERFLOW = 3 };
struct RowOut {
    int mode;
    const int *crp;         // PLAIN / REDO: final row pointers
    const long long *soff;  // SPEC: speculative slot offsets [M+1]
    int *ccol;              // destination columns
    double *cval;           // destination values
    int *cnnz;              // SPEC: exact nnz found per row
    unsigned char *flag;    // SPEC: written; REDO: rows flagged ROW_OVERFLOW are redone
    int lo, hi;             // only rows lo <= i < hi are written (a row panel; 0, M: all rows)
};

// per-row data of A produced by the bounds kernel
struct RowInfo {
    long long *prod;   // intermediate products of the row
    int *tmin;         // first C tile id (INT_MAX for an empty row)
    int *tmax;         // last C tile id (-1 for an empty row)
    int *bins;         // NBIN slabs of M row ids, each in ascending row order
    int *cnnz;         // exact nnz per row (count pass)
    signed char *cls;  // row class (RowBin) of every row, -1 for an empty row
    int *bin_cnt;      // [NBIN][ceil(M/32)] rows of each class per 32-row chunk, then
                       // its exclusive scan (bin_scratch_ints(M) entries)
    int store;         // 1: the tile store is in use -- the count pass sizes each large row's
                       // list, min(tile span, sum of its B rows' tile counts), and adds the
                       // sizes up in Ctl::store_tiles (the arena the next call wants)
};

// C tiles of the large-class rows, kept by the count pass (which builds them
// anyway) so that the structure pass streams each row's tile list instead of
// repeating the OR walk over B's tiles.  Each large row reserves min(tile span,
// sum of its B rows' tile counts) entries of the arena (tcol/tent, `cap`
// entries, owned by the handle) with one atomic; a row that finds the arena full keeps nothing (cnt[i] = -1) and
// the structure pass walks B for it as before.  Row i's list:
// tcol/tent[off[i] .. off[i] + cnt[i]), tile ids ascending.
//
// A tile's column mask and its slot word are written and read together, so
// they share one 16-byte entry: one 128-bit store in the count pass, one
// 128-bit load in the structure pass.
struct alignas(16) TileEnt {
    unsigned long long mask;    // column mask
    long long info;             // first slot | (window ordinal + 1) << 32 (hsmu_tilelist.cuh)
};

struct TileStore {
    long long *off;             // [M] written by the count pass
    int *cnt;                   // [M] tiles stored per row, -1: none
    int *nwin;                  // [M] numeric windows of the row (0 for rows without a list)
    int *wbase;                 // [M+1] index of the row's first window: exclusive scan of nwin in row
                                // order (nullable: the structure pass reserves them itself)
    int *tcol;                  // arena: tile ids
    TileEnt *tent;              // arena: column mask and slot word of each tile
    long long cap;              // arena entries
    int all_stored;             // host: every large row got a list (no OR-walk rows left)
};

// scratch ints of RowInfo::bin_cnt for M rows
size_t bin_scratch_ints(int M);

// k_tiles.cu
void launch_tiles_count(const DevCSR &B, int *tcnt, int validate, Ctl *ctl, int grid, cudaStream_t st);
void launch_tiles_fill(const DevCSR &B, const int *tptr, int *tcol, unsigned long long *tmask, int *toff, Ctl *ctl,
                       int grid, cudaStream_t st);
void launch_validate(const DevCSR &A, Ctl *ctl, int grid, cudaStream_t st);

// k_rows.cu
void launch_bounds(const DevCSR &A, const DevCSR &B, RowInfo ri, Ctl *ctl, int grid, int *scan_tmp, cudaStream_t st);
// out[c] = products of rows c*PROD_CHUNK .. (c+1)*PROD_CHUNK-1 (ceil(M / PROD_CHUNK) entries)
constexpr int PROD_CHUNK = 64;
void launch_chunk_prod(int M, const long long *prod, long long *out, int grid, cudaStream_t st);
// exclusive scan of int counts (n entries) into out[0..n]; total (int64) into *total64;
// sets DERR_OVERFLOW if the total exceeds INT32_MAX.  tmp must hold scan_tmp_ints(n) ints.
// in == out (an in-place scan) is allowed.
size_t scan_tmp_ints(int n);
void launch_scan(const int *in, int *out, int n, long long *total64, int *tmp, Ctl *ctl, cudaStream_t st);
// same with int64 output (no overflow limit)
void launch_scan64(const int *in, long long *out, int n, long long *total64, int *tmp, cudaStream_t st);

// learned.cu
void launch_features(const DevCSR &A, const DevCSR &B, float4 *feat, long long *prod_out, int nsm, cudaStream_t st);
// wide_prod (nullable): incremented by the products of every warp-class row predicted clearly
// above FUSE_CAP entries; large_no_slot: rows of the large class get no slot (the caller keeps
// their tile lists)
void launch_capacity(const float *params, const float4 *feat, const long long *prod, const signed char *cls, int M,
                     int N, float margin, int *cap, int nsm, cudaStream_t st, unsigned long long *wide_prod,
                     bool large_no_slot);
void launch_compact(int M, const long long *soff, const int *crp, const unsigned char *flag, const int *scol,
                    const double *sval, int *ccol, double *cval, int nsm, cudaStream_t st);

// k_symbolic.cu
void launch_count(const DevCSR &A, const DevCSR &B, const DevTiles &Bt, RowInfo ri, Ctl *ctl, int nsm,
                  cudaStream_t st);
// the same in two launches: rows of the tiny and warp classes, then the large class
// (ts: nullable; when given, the large rows' C tiles are stored while the arena lasts)
void launch_count_small(const DevCSR &A, const DevCSR &B, const DevTiles &Bt, RowInfo ri, Ctl *ctl, int nsm,
                        cudaStream_t st);
void launch_count_large(const DevCSR &A, const DevTiles &Bt, RowInfo ri, const TileStore *ts, Ctl *ctl, int nsm,
                        cudaStream_t st);
// learned path, large rows: exact count and tile list in its speculative pass;
// every listed row is flagged ROW_OVERFLOW (out.flag) so that the pass after the
// exact scan writes it at its place in C (k_symbolic.cu)
void launch_spec_large(const DevCSR &A, const DevTiles &Bt, RowInfo ri, const TileStore &ts, RowOut out, Ctl *ctl,
                       int nsm, cudaStream_t st);

// k_structure.cu
// writes C's columns and numeric windows; rows that fit one warp also get their values
// class_rows: rows per class (BIN_*) when known on the host; kernels of empty classes are skipped
// ts (nullable, PLAIN mode): large rows are built from their stored tile lists
void launch_structure(const DevCSR &A, const DevCSR &B, const DevTiles &Bt, RowInfo ri, RowOut out, Window *win,
                      long long win_cap, Ctl *ctl, int arith, int nsm, cudaStream_t st,
                      const int *class_rows = nullptr, const TileStore *ts = nullptr);

// k_numeric.cu
// flag (nullable): speculative-pass windows of rows flagged ROW_OVERFLOW are skipped;
// scol/soff (nullable): speculative slots holding the columns of speculative-pass
// windows, which the kernel copies to ccol
// per-window cursors into the B rows (k_win_cursors): len/off/item_off/scan_tmp sized
// for win_cap windows (+1), total for 2 entries, cur for cap entries (Ctl::cur_bound)
struct WinCursors {
    int *len;
    long long *off;
    long long *total;
    int *scan_tmp;
    int *item_off;  // the cursor pass's work items per window, scanned in place
    int *cur;
    long long cap;
};
void launch_numeric(const DevCSR &A, const DevCSR &B, const DevTiles &Bt, const int *crp, int *ccol, double *cval,
                    const Window *win, long long win_cap, const unsigned char *flag, const int *scol,
                    const long long *soff, const WinCursors &wc, Ctl *ctl, int arith, int nsm, cudaStream_t st,
                    int wait_polls = 0, const TileStore *ts = nullptr);

int run_dmul_selftest(unsigned long long n, unsigned long long seed, unsigned long long *out, cudaStream_t st);
// FP64 lane operations per second of a full-grid chain probe
int run_fp64_rate(int iters, int nsm, double *lane_ops_per_s, cudaStream_t st);

// hsmu_status of the device error bits collected in Ctl::err (0 -> HSMU_OK)
int status_from_dev_err(int err);

// smem sizes are set once per device (cudaFuncSetAttribute)
int configure_kernels();

// k_transpose.cu: B = A^T (rows of B in ascending column order), scratch sized by the helpers
int launch_transpose(const DevCSR &A, int *trp, int *tcol, double *tval, int *scratch_i, double *scratch_d,
                     int *hist, int *scan_tmp, long long *total64, Ctl *ctl, int nsm, cudaStream_t st);
size_t transpose_scratch_ints(long long nnz);
size_t transpose_scratch_doubles(long long nnz);
size_t transpose_hist_ints(long long nnz);

}  // namespace hsmu
