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

// per-row data of A produced by the bounds kernel
struct RowInfo {
    long long *prod;   // intermediate products of the row
    int *tmin;         // first C tile id (INT_MAX for an empty row)
    int *tmax;         // last C tile id (-1 for an empty row)
    int *bins;         // NBIN slabs of M row ids
    int *cnnz;         // exact nnz per row (count pass)
};

// k_tiles.cu
void launch_tiles_count(const DevCSR &B, int *tcnt, int validate, Ctl *ctl, int grid, cudaStream_t st);
void launch_tiles_fill(const DevCSR &B, const int *tptr, int *tcol, unsigned long long *tmask, int *toff, Ctl *ctl,
                       int grid, cudaStream_t st);
void launch_validate(const DevCSR &A, Ctl *ctl, int grid, cudaStream_t st);

// k_rows.cu
void launch_bounds(const DevCSR &A, const DevCSR &B, const DevTiles &Bt, RowInfo ri, Ctl *ctl, int grid,
                   cudaStream_t st);
// exclusive scan of int counts (n entries) into out[0..n]; total (int64) into *total64;
// sets DERR_OVERFLOW if the total exceeds INT32_MAX.  tmp must hold scan_tmp_ints(n) ints.
size_t scan_tmp_ints(int n);
void launch_scan(const int *in, int *out, int n, long long *total64, int *tmp, Ctl *ctl, cudaStream_t st);

// k_symbolic.cu
void launch_count(const DevCSR &A, const DevCSR &B, const DevTiles &Bt, RowInfo ri, Ctl *ctl, int nsm,
                  cudaStream_t st);

// k_structure.cu
// writes C's columns and numeric windows; rows that fit one warp also get their values
void launch_structure(const DevCSR &A, const DevCSR &B, const DevTiles &Bt, RowInfo ri, const int *crp, int *ccol,
                      double *cval, Window *win, long long win_cap, Ctl *ctl, int arith, int nsm, cudaStream_t st);

// k_numeric.cu
void launch_numeric(const DevCSR &A, const DevCSR &B, const int *crp, const int *ccol, double *cval,
                    const Window *win, long long win_cap, Ctl *ctl, int arith, int nsm, cudaStream_t st);

int run_dmul_selftest(unsigned long long n, unsigned long long seed, unsigned long long *out, cudaStream_t st);

// smem sizes are set once per device (cudaFuncSetAttribute)
int configure_kernels();

}  // namespace hsmu
