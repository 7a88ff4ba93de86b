/*
 * Host FP64 Gustavson SpGEMM oracle for C = A*B (int32 CSR in, CSR out).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU engine: it
 * is built into liboracle.so and called from tests/, from the smoke check in
 * __graft_entry__.py and from the cpu_baseline / --impl reference legs of
 * bench.py.  The product path (the CUDA engine behind include/hsmu_gb.h)
 * never links, loads or calls it.
 *
 * What it restates from the reference (HSMU-SpGEMM, paths relative to that
 * project):
 *   - structure: C(i,:) is the union of the column sets of B(k,:) over the
 *     entries (i,k) of A, with no numerical dropping -- products that cancel
 *     to 0.0 stay as explicit entries, because the reference derives the
 *     structure symbolically from the OR of 64-column tile masks
 *     (src/compressed/compressed_tileOR.cuh:53-75, row nnz = sum of popcounts
 *     at :80-101);
 *   - column order: ascending within each row (rank sort in
 *     src/compressed/compressed_Ccol_symbolic.cuh:53-62, prefix compaction in
 *     src/external/spECK/dense_acc.cu:101-111);
 *   - values: every product is rounded to double first and then added to the
 *     row accumulator (atomicAdd(num_table + hash, aval * bval) in
 *     src/compressed/compressed_Cval.cuh:60-61).  The reference adds with
 *     shared-memory atomics, so its order is unspecified; this oracle fixes
 *     the order to the entries of A(i,:) in storage order (k ascending for a
 *     sorted A) and, within one k, B(k,:) in storage order.  The file must be
 *     compiled with -ffp-contract=off so that a*b+c is never fused.
 *   - intermediate-product count: sum over A entries of nnz(B(k,:))
 *     (src/NHC_spgemm.cuh:37-42), accumulated in 64 bits.
 *
 * Parallelism: OpenMP over rows, one dense sparse accumulator (SPA) per
 * thread.  The result does not depend on the thread count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_OK 0
#define ORC_ERR_ALLOC 2
#define ORC_ERR_OVERFLOW 4

static int set_threads(int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
    return omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

int oracle_max_threads(void) { return set_threads(0); }

/* Number of intermediate products, sum_i sum_{k in A(i,:)} nnz(B(k,:)).
 * Follows src/NHC_spgemm.cuh:37-42 (64-bit counter). */
uint64_t oracle_products(int M, const int *arp, const int *acol, const int *brp)
{
    uint64_t total = 0;
    for (int i = 0; i < M; i++)
        for (int p = arp[i]; p < arp[i + 1]; p++)
            total += (uint64_t)(brp[acol[p] + 1] - brp[acol[p]]);
    return total;
}

/* Symbolic phase: nnz of each listed output row (structural union of the
 * referenced B rows).  rows == NULL means rows 0..nrows-1.
 * out_nnz[r] receives nnz(C(rows[r],:)).  Returns 0 or ORC_ERR_ALLOC. */
int oracle_symbolic(int nrows, const int *rows, int N,
                    const int *arp, const int *acol, const int *brp, const int *bcol,
                    int64_t *out_nnz, int nthreads)
{
    int err = 0;
    set_threads(nthreads);
#pragma omp parallel
    {
        int *mark = (int *)malloc(sizeof(int) * (size_t)(N > 0 ? N : 1));
        if (!mark) {
#pragma omp atomic write
            err = ORC_ERR_ALLOC;
        } else {
            for (int j = 0; j < N; j++)
                mark[j] = -1;
#pragma omp for schedule(dynamic, 64)
            for (int r = 0; r < nrows; r++) {
                int i = rows ? rows[r] : r;
                int64_t cnt = 0;
                for (int p = arp[i]; p < arp[i + 1]; p++) {
                    int k = acol[p];
                    for (int q = brp[k]; q < brp[k + 1]; q++) {
                        int j = bcol[q];
                        if (mark[j] != r) {
                            mark[j] = r;
                            cnt++;
                        }
                    }
                }
                out_nnz[r] = cnt;
            }
            free(mark);
        }
    }
    return err;
}

static int cmp_int(const void *a, const void *b)
{
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

/* Numeric phase for the listed output rows.
 * crp[0..nrows] must be the exclusive scan of oracle_symbolic's counts for the
 * same row list (int64 offsets, so a sampled subset of a huge product works).
 * Writes sorted columns to ccol and values to cval.  For each output entry
 * the value is the left-to-right sum 0.0 + p_1 + p_2 + ... where the p_t are
 * the rounded products a_ik*b_kj in the order described at the top of the
 * file (fused != 0: each step is fma(a_ik, b_kj, partial sum) instead). */
static int numeric_impl(int nrows, const int *rows, int N,
                        const int *arp, const int *acol, const double *aval,
                        const int *brp, const int *bcol, const double *bval,
                        const int64_t *crp, int *ccol, double *cval, int nthreads, int fused)
{
    int err = 0;
    set_threads(nthreads);
#pragma omp parallel
    {
        int *mark = (int *)malloc(sizeof(int) * (size_t)(N > 0 ? N : 1));
        double *acc = (double *)malloc(sizeof(double) * (size_t)(N > 0 ? N : 1));
        if (!mark || !acc) {
#pragma omp atomic write
            err = ORC_ERR_ALLOC;
        } else {
            for (int j = 0; j < N; j++)
                mark[j] = -1;
#pragma omp for schedule(dynamic, 16)
            for (int r = 0; r < nrows; r++) {
                int i = rows ? rows[r] : r;
                int *cols = ccol + crp[r];
                int64_t cnt = 0;
                for (int p = arp[i]; p < arp[i + 1]; p++) {
                    int k = acol[p];
                    double a = aval[p];
                    for (int q = brp[k]; q < brp[k + 1]; q++) {
                        int j = bcol[q];
                        if (mark[j] != r) {
                            mark[j] = r;
                            acc[j] = 0.0;
                            cols[cnt++] = j;
                        }
                        if (fused)
                            acc[j] = fma(a, bval[q], acc[j]); /* one rounding per product */
                        else
                            acc[j] = acc[j] + a * bval[q]; /* rounded product, rounded sum */
                    }
                }
                qsort(cols, (size_t)cnt, sizeof(int), cmp_int);
                for (int64_t t = 0; t < cnt; t++)
                    cval[crp[r] + t] = acc[cols[t]];
            }
            free(mark);
            free(acc);
        }
    }
    return err;
}

int oracle_numeric(int nrows, const int *rows, int N,
                   const int *arp, const int *acol, const double *aval,
                   const int *brp, const int *bcol, const double *bval,
                   const int64_t *crp, int *ccol, double *cval, int nthreads)
{
    return numeric_impl(nrows, rows, N, arp, acol, aval, brp, bcol, bval, crp, ccol, cval, nthreads, 0);
}

/* Same as oracle_numeric, with every product fused into its accumulator:
 * c = fma(a, b, c), one rounding per product, in the same order.  This is the
 * arithmetic of the engine's fused-multiply-add mode (opts.arith = 1); the
 * reference rounds each product (see the top of the file), and the two differ
 * by at most one rounding of each product. */
int oracle_numeric_fma(int nrows, const int *rows, int N,
                       const int *arp, const int *acol, const double *aval,
                       const int *brp, const int *bcol, const double *bval,
                       const int64_t *crp, int *ccol, double *cval, int nthreads)
{
    return numeric_impl(nrows, rows, N, arp, acol, aval, brp, bcol, bval, crp, ccol, cval, nthreads, 1);
}

/* Sum of |a_ik|*|b_kj| per output entry, in the same layout as cval; used to
 * scale the value tolerance for entries whose terms cancel. */
int oracle_abs_numeric(int nrows, const int *rows, int N,
                       const int *arp, const int *acol, const double *aval,
                       const int *brp, const int *bcol, const double *bval,
                       const int64_t *crp, const int *ccol, double *cabs, int nthreads)
{
    int err = 0;
    set_threads(nthreads);
#pragma omp parallel
    {
        double *acc = (double *)malloc(sizeof(double) * (size_t)(N > 0 ? N : 1));
        if (!acc) {
#pragma omp atomic write
            err = ORC_ERR_ALLOC;
        } else {
#pragma omp for schedule(dynamic, 16)
            for (int r = 0; r < nrows; r++) {
                int i = rows ? rows[r] : r;
                for (int64_t t = crp[r]; t < crp[r + 1]; t++)
                    acc[ccol[t]] = 0.0;
                for (int p = arp[i]; p < arp[i + 1]; p++) {
                    int k = acol[p];
                    double a = aval[p] < 0 ? -aval[p] : aval[p];
                    for (int q = brp[k]; q < brp[k + 1]; q++) {
                        double b = bval[q] < 0 ? -bval[q] : bval[q];
                        acc[bcol[q]] += a * b;
                    }
                }
                for (int64_t t = crp[r]; t < crp[r + 1]; t++)
                    cabs[t] = acc[ccol[t]];
            }
            free(acc);
        }
    }
    return err;
}

/* CSR transpose (B = A^T) with columns sorted ascending in every output row,
 * as needed for the A*A^T configuration.  Counting sort; stable, so each
 * output row lists source rows in increasing order. */
int oracle_transpose(int M, int N, const int *arp, const int *acol, const double *aval,
                     int *trp, int *tcol, double *tval)
{
    memset(trp, 0, sizeof(int) * (size_t)(N + 1));
    for (int i = 0; i < M; i++)
        for (int p = arp[i]; p < arp[i + 1]; p++)
            trp[acol[p] + 1]++;
    for (int j = 0; j < N; j++)
        trp[j + 1] += trp[j];
    int *cur = (int *)malloc(sizeof(int) * (size_t)(N > 0 ? N : 1));
    if (!cur)
        return ORC_ERR_ALLOC;
    memcpy(cur, trp, sizeof(int) * (size_t)N);
    for (int i = 0; i < M; i++)
        for (int p = arp[i]; p < arp[i + 1]; p++) {
            int q = cur[acol[p]]++;
            tcol[q] = i;
            tval[q] = aval[p];
        }
    free(cur);
    return ORC_OK;
}
