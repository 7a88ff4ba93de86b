// Device generators of the AMG Galerkin workload's operators (inputs of the
// batched engine's measured configuration): the 7-point Poisson matrix of a
// side^3 grid and the 2x2x2 aggregation prolongator P with its transpose.
// Generating on the device keeps hundreds of operators with 1e9 entries in
// total off the host; hsmu_gb/gen.py (poisson7, aggregation_prolongator)
// builds the same matrices on the host and the tests compare the two.
#include <cuda_runtime.h>

#include "hsmu_common.cuh"
#include "hsmu_gb.h"
#include "hsmu_kernels.h"

namespace hsmu {

__global__ void k_poisson7_len(int s, int *len) {
    const long long n = (long long)s * s * s;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % s), y = (int)((i / s) % s), z = (int)(i / ((long long)s * s));
        len[i] = 1 + (z > 0) + (y > 0) + (x > 0) + (x < s - 1) + (y < s - 1) + (z < s - 1);
    }
}

__global__ void k_poisson7_fill(int s, const int *rp, int *col, double *val) {
    const long long n = (long long)s * s * s;
    const int ss = s * s;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % s), y = (int)((i / s) % s), z = (int)(i / ss);
        int q = rp[i];
        const int ii = (int)i;
        // ascending column order
        if (z > 0) { col[q] = ii - ss; val[q++] = -1.0; }
        if (y > 0) { col[q] = ii - s; val[q++] = -1.0; }
        if (x > 0) { col[q] = ii - 1; val[q++] = -1.0; }
        col[q] = ii; val[q++] = 6.0;
        if (x < s - 1) { col[q] = ii + 1; val[q++] = -1.0; }
        if (y < s - 1) { col[q] = ii + s; val[q++] = -1.0; }
        if (z < s - 1) { col[q] = ii + ss; val[q++] = -1.0; }
    }
}

__global__ void k_agg_p(int s, int *rp, int *col, double *val) {
    const long long n = (long long)s * s * s;
    const int cs = (s + 1) / 2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i <= n; i += (long long)gridDim.x * blockDim.x) {
        rp[i] = (int)i;
        if (i < n) {
            const int x = (int)(i % s), y = (int)((i / s) % s), z = (int)(i / ((long long)s * s));
            col[i] = x / 2 + cs * (y / 2 + cs * (z / 2));
            val[i] = 1.0;
        }
    }
}

__device__ __forceinline__ int agg_extent(int c, int s) { return min(2, s - 2 * c); }

__global__ void k_agg_pt_len(int s, int *len) {
    const int cs = (s + 1) / 2;
    const long long nc = (long long)cs * cs * cs;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nc; c += (long long)gridDim.x * blockDim.x) {
        const int cx = (int)(c % cs), cy = (int)((c / cs) % cs), cz = (int)(c / ((long long)cs * cs));
        len[c] = agg_extent(cx, s) * agg_extent(cy, s) * agg_extent(cz, s);
    }
}

__global__ void k_agg_pt_fill(int s, const int *rp, int *col, double *val) {
    const int cs = (s + 1) / 2;
    const long long nc = (long long)cs * cs * cs;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nc; c += (long long)gridDim.x * blockDim.x) {
        const int cx = (int)(c % cs), cy = (int)((c / cs) % cs), cz = (int)(c / ((long long)cs * cs));
        int q = rp[c];
        for (int dz = 0; dz < agg_extent(cz, s); dz++)
            for (int dy = 0; dy < agg_extent(cy, s); dy++)
                for (int dx = 0; dx < agg_extent(cx, s); dx++) {
                    col[q] = (2 * cx + dx) + s * ((2 * cy + dy) + s * (2 * cz + dz));
                    val[q++] = 1.0;
                }
    }
}

namespace {

int scan_lengths(int *rp, int n, cudaStream_t st) {
    int *tmp = nullptr;
    long long *tot = nullptr;
    Ctl *ctl = nullptr;
    int rc = HSMU_OK;
    if (cudaMallocAsync(reinterpret_cast<void **>(&tmp), scan_tmp_ints(n) * sizeof(int), st) ||
        cudaMallocAsync(reinterpret_cast<void **>(&tot), sizeof(long long), st) ||
        cudaMallocAsync(reinterpret_cast<void **>(&ctl), sizeof(Ctl), st)) {
        rc = HSMU_ERR_ALLOC;
    } else {
        cudaMemsetAsync(ctl, 0, sizeof(Ctl), st);
        launch_scan(rp, rp, n, tot, tmp, ctl, st);
        if (cudaGetLastError() != cudaSuccess) rc = HSMU_ERR_CUDA;
    }
    if (tmp) cudaFreeAsync(tmp, st);
    if (tot) cudaFreeAsync(tot, st);
    if (ctl) cudaFreeAsync(ctl, st);
    return rc;
}

int read_int(const int *d, int *h, cudaStream_t st) {
    if (cudaMemcpyAsync(h, d, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return HSMU_ERR_CUDA;
    return HSMU_OK;
}

}  // namespace
}  // namespace hsmu

using namespace hsmu;

extern "C" int hsmu_gen_poisson7(int side, hsmu_csr *A, void *stream) {
    if (!A || side < 1 || side > 670) return HSMU_ERR_INVALID;  // 7 * side^3 must fit int32
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int n = side * side * side;
    int *rp = nullptr, *col = nullptr;
    double *val = nullptr;
    int nnz = 0, rc;
    if (cudaMallocAsync(reinterpret_cast<void **>(&rp), sizeof(int) * (n + 1), st)) return HSMU_ERR_ALLOC;
    k_poisson7_len<<<1024, 256, 0, st>>>(side, rp);
    rc = scan_lengths(rp, n, st);
    if (!rc) rc = read_int(rp + n, &nnz, st);
    if (!rc && (cudaMallocAsync(reinterpret_cast<void **>(&col), sizeof(int) * (size_t)nnz, st) ||
                cudaMallocAsync(reinterpret_cast<void **>(&val), sizeof(double) * (size_t)nnz, st)))
        rc = HSMU_ERR_ALLOC;
    if (!rc) {
        k_poisson7_fill<<<1024, 256, 0, st>>>(side, rp, col, val);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) rc = HSMU_ERR_CUDA;
    }
    if (rc) {
        cudaFreeAsync(rp, st);
        if (col) cudaFreeAsync(col, st);
        if (val) cudaFreeAsync(val, st);
        cudaStreamSynchronize(st);
        return rc;
    }
    *A = hsmu_csr{n, n, nnz, 1, rp, col, val};
    return HSMU_OK;
}

extern "C" int hsmu_gen_aggregation(int side, hsmu_csr *P, hsmu_csr *Pt, void *stream) {
    if (!P || !Pt || side < 1 || side > 670) return HSMU_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int n = side * side * side;
    const int cs = (side + 1) / 2;
    const int nc = cs * cs * cs;
    int *prp = nullptr, *pcol = nullptr, *trp = nullptr, *tcol = nullptr;
    double *pval = nullptr, *tval = nullptr;
    int rc = HSMU_OK;
    if (cudaMallocAsync(reinterpret_cast<void **>(&prp), sizeof(int) * (n + 1), st) ||
        cudaMallocAsync(reinterpret_cast<void **>(&pcol), sizeof(int) * n, st) ||
        cudaMallocAsync(reinterpret_cast<void **>(&pval), sizeof(double) * n, st) ||
        cudaMallocAsync(reinterpret_cast<void **>(&trp), sizeof(int) * (nc + 1), st) ||
        cudaMallocAsync(reinterpret_cast<void **>(&tcol), sizeof(int) * n, st) ||
        cudaMallocAsync(reinterpret_cast<void **>(&tval), sizeof(double) * n, st))
        rc = HSMU_ERR_ALLOC;
    if (!rc) {
        k_agg_p<<<1024, 256, 0, st>>>(side, prp, pcol, pval);
        k_agg_pt_len<<<1024, 256, 0, st>>>(side, trp);
        rc = scan_lengths(trp, nc, st);
    }
    if (!rc) {
        k_agg_pt_fill<<<1024, 256, 0, st>>>(side, trp, tcol, tval);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) rc = HSMU_ERR_CUDA;
    }
    if (rc) {
        for (void *p : {(void *)prp, (void *)pcol, (void *)pval, (void *)trp, (void *)tcol, (void *)tval})
            if (p) cudaFreeAsync(p, st);
        cudaStreamSynchronize(st);
        return rc;
    }
    *P = hsmu_csr{n, nc, n, 1, prp, pcol, pval};
    *Pt = hsmu_csr{nc, n, n, 1, trp, tcol, tval};
    return HSMU_OK;
}
