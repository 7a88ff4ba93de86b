// A caller written against the reference's interface (the same steps as its
// driver, src/test.cu:30-91), compiled against include/hsmu_nhc_compat.h and
// linked with libhsmu_gb.so.  usage: compat_driver A.bin C.bin
//   *.bin: int32 M, N, nnz, then int32 row_ptr[M+1], int32 col[nnz], f64 val[nnz]
#include <cstdio>
#include <vector>

#include "hsmu_nhc_compat.h"

static bool read_csr(const char *path, NHC_CSR *X) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    int h[3];
    if (std::fread(h, sizeof(int), 3, f) != 3) return false;
    X->M = h[0];
    X->N = h[1];
    X->nnz = h[2];
    X->rowPtr = new index_t[X->M + 1];
    X->col = new index_t[X->nnz];
    X->val = new value_t[X->nnz];
    bool ok = std::fread(X->rowPtr, 4, X->M + 1, f) == (size_t)(X->M + 1) &&
              std::fread(X->col, 4, X->nnz, f) == (size_t)X->nnz && std::fread(X->val, 8, X->nnz, f) == (size_t)X->nnz;
    std::fclose(f);
    return ok;
}

int main(int argc, char **argv) {
    if (argc < 3) return 2;
    NHC_CSR A, B, C;
    NHC_mask_matrix mask_matrixB;
    NHC_bin c_bin;
    compressed_bin compressed_bin;
    std::memset(&A, 0, sizeof(A));
    std::memset(&B, 0, sizeof(B));
    std::memset(&C, 0, sizeof(C));
    if (!read_csr(argv[1], &A) || !read_csr(argv[1], &B)) return 3;  // B is a second copy of A
    C.M = A.M;
    C.N = B.N;
    HtD_value_col_ptr(&A);
    HtD_value_col_ptr(&B);
    for (int iter = 0; iter < 2; iter++) {
        NHC_spgemm(&compressed_bin, &c_bin, &A, &B, &C, &mask_matrixB);
        if (iter == 0) {  // release between calls, as the reference's own loop does
            realse_NHC_tile(&B);
            realse_NHC_tile(&C);
            free_C_matrix(&C);
            realse_compressed_bin(&compressed_bin);
            free_bin(&c_bin);
        }
    }
    std::vector<int> col(C.nnz);
    std::vector<double> val(C.nnz);
    cudaMemcpy(col.data(), C.d_col, 4 * (size_t)C.nnz, cudaMemcpyDeviceToHost);
    cudaMemcpy(val.data(), C.d_val, 8 * (size_t)C.nnz, cudaMemcpyDeviceToHost);
    FILE *f = std::fopen(argv[2], "wb");
    int h[3] = {C.M, C.N, C.nnz};
    std::fwrite(h, 4, 3, f);
    std::fwrite(C.rowPtr, 4, C.M + 1, f);  // the host copy of the row pointers
    std::fwrite(col.data(), 4, C.nnz, f);
    std::fwrite(val.data(), 8, C.nnz, f);
    std::fclose(f);
    realse_NHCcsr(&A);
    realse_NHCcsr(&B);
    free_C_matrix(&C);
    realse_NHC_tile(&B);
    realse_NHC_tile(&C);
    realse_compressed_bin(&compressed_bin);
    free_bin(&c_bin);
    std::printf("ok nnz %d\n", C.nnz);
    return 0;
}
