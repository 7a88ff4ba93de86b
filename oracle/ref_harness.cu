// Harness that runs the reference HSMU-SpGEMM GPU path unmodified, for
// pinning the oracle and for timing the reference on the same GPU.
// TEST INFRASTRUCTURE ONLY: built by oracle/ref_build.py from the reference
// sources (staged into oracle/_ref/, never committed) and driven by
// oracle/ref_run.py.  Nothing in the engine links or calls it.
//
// usage: ref_harness A.bin B.bin|same C.bin|none reps   (none: time only, C is not written)
//   *.bin: int32 M, N, nnz, then int32 row_ptr[M+1], int32 col[nnz], f64 val[nnz]
// The call sequence mirrors the reference's driver (src/test.cu:62-91):
// HtD_value_col_ptr on A and B, NHC_spgemm, then the release functions; the
// driver's B for C = A*A is a second copy of A (src/test.cu:57-60), and so is
// ours.  Each call is timed with CUDA events around NHC_spgemm (setup, B
// conversion and all stages); the reference's own stage time (time2, which
// excludes setup and conversion) is printed by NHC_spgemm itself.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "src/NHC_spgemm.cuh"

static bool read_csr(const char *path, NHC_CSR *X) {
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    int hdr[3];
    if (fread(hdr, sizeof(int), 3, f) != 3) { fclose(f); return false; }
    X->M = hdr[0];
    X->N = hdr[1];
    X->nnz = hdr[2];
    X->rowPtr = new index_t[X->M + 1];
    X->col = new index_t[X->nnz > 0 ? X->nnz : 1];
    X->val = new value_t[X->nnz > 0 ? X->nnz : 1];
    bool ok = fread(X->rowPtr, sizeof(int), X->M + 1, f) == (size_t)(X->M + 1) &&
              fread(X->col, sizeof(int), X->nnz, f) == (size_t)X->nnz &&
              fread(X->val, sizeof(double), X->nnz, f) == (size_t)X->nnz;
    fclose(f);
    return ok;
}

static bool write_csr(const char *path, int M, int N, int nnz, const int *rp, const int *col, const double *val) {
    FILE *f = fopen(path, "wb");
    if (!f) return false;
    int hdr[3] = {M, N, nnz};
    bool ok = fwrite(hdr, sizeof(int), 3, f) == 3 && fwrite(rp, sizeof(int), M + 1, f) == (size_t)(M + 1) &&
              fwrite(col, sizeof(int), nnz, f) == (size_t)nnz && fwrite(val, sizeof(double), nnz, f) == (size_t)nnz;
    fclose(f);
    return ok;
}

int main(int argc, char **argv) {
    if (argc < 5) {
        fprintf(stderr, "usage: %s A.bin B.bin|same C.bin reps\n", argv[0]);
        return 2;
    }
    const int reps = atoi(argv[4]);
    NHC_CSR A, B;
    memset(&A, 0, sizeof(A));
    memset(&B, 0, sizeof(B));
    if (!read_csr(argv[1], &A) || !read_csr(strcmp(argv[2], "same") ? argv[2] : argv[1], &B)) {
        fprintf(stderr, "cannot read inputs\n");
        return 3;
    }
    if (B.N < threshold_value_selected) {
        fprintf(stderr, "B->N < %d selects the reference's small path, not the compressed path\n",
                threshold_value_selected);
        return 4;
    }
    char name[] = "harness";
    A.matrix_name = name;
    B.matrix_name = name;
    HtD_value_col_ptr(&A);
    HtD_value_col_ptr(&B);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = 0;
    for (int r = 0; r < reps; r++) {
        NHC_CSR C;
        memset(&C, 0, sizeof(C));
        C.M = A.M;
        C.N = B.N;
        compressed_bin cb{};
        NHC_bin nb{};
        NHC_mask_matrix mm{};
        cudaDeviceSynchronize();
        cudaEventRecord(e0);
        NHC_spgemm(&cb, &nb, &A, &B, &C, &mm);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaError_t err = cudaGetLastError();
        printf("HARNESS_CALL_MS %.6f nnz %d err %d\n", ms, C.nnz, (int)err);
        fflush(stdout);
        if (err != cudaSuccess) rc = 5;
        if (r == reps - 1 && err == cudaSuccess && strcmp(argv[3], "none") != 0) {
            std::vector<int> rp(C.M + 1), col(C.nnz > 0 ? C.nnz : 1);
            std::vector<double> val(C.nnz > 0 ? C.nnz : 1);
            cudaMemcpy(rp.data(), C.d_ptr, sizeof(int) * (C.M + 1), cudaMemcpyDeviceToHost);
            cudaMemcpy(col.data(), C.d_col, sizeof(int) * (size_t)C.nnz, cudaMemcpyDeviceToHost);
            cudaMemcpy(val.data(), C.d_val, sizeof(double) * (size_t)C.nnz, cudaMemcpyDeviceToHost);
            if (!write_csr(argv[3], C.M, C.N, C.nnz, rp.data(), col.data(), val.data())) rc = 6;
        }
        realse_NHC_tile(&B);
        realse_NHC_tile(&C);
        free_C_matrix(&C);
        realse_compressed_bin(&cb);
        free_bin(&nb);
    }
    realse_NHCcsr(&A);
    realse_NHCcsr(&B);
    return rc;
}
