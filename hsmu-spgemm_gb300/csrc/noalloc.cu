// hsmu_btiles_build_noalloc: the B -> 64-column bit tile conversion without
// any device allocation.
//
// Who needs it: callers whose device memory is owned by someone else -- an
// application that reserves all GPU memory up front in its own pool, or a
// runtime with a fixed memory budget that forbids cudaMalloc/cudaFree (and
// allocating library calls) on its compute path.  Such a caller can still
// provide the input B and the output tile arrays from its own memory, but
// cannot let the library allocate the conversion's scratch.
//
// The conversion's scratch -- the block sums of the device scan that turns
// per-row tile counts into tile_ptr, the scan total, and the control word
// that collects device-side errors -- lives in the file-scope device array
// below.  Its size fixes the maximum number of B rows (NOALLOC_MAX_ROWS);
// every GPU that loads the library holds the array (about 64 KB) until the
// process exits.  The per-row tile counts are written into tile_ptr itself
// and scanned in place, so they need no scratch.
//
// Set-up: the device address of the array is looked up with
// cudaGetSymbolAddress once per device, by the first call made while that
// device is current (so make the first call on each device before any
// stream capture).  The address is cached for the life of the process:
// cudaDeviceReset (or any reset of the device's primary context) reloads
// the module and invalidates it, so do not call this entry point again on a
// device after resetting it.  All calls share the array and it keeps the previous
// call's contents: each call clears the control word itself, and calls that
// overlap on the GPU (different streams, or different host threads on the
// same device) race on it -- serialise them.
#include <cuda_runtime.h>

#include <mutex>

#include "hsmu_common.cuh"
#include "hsmu_gb.h"
#include "hsmu_kernels.h"

namespace hsmu {

constexpr int NOALLOC_MAX_ROWS = 1 << 24;
constexpr int NOALLOC_MAX_DEVICES = 64;
// scan block sums (scan_tmp_ints(NOALLOC_MAX_ROWS) ints) + total + control block
constexpr size_t NOALLOC_SCAN_INTS = (size_t)((NOALLOC_MAX_ROWS + 2047) / 2048) * 2 + 2;
constexpr size_t NOALLOC_BYTES = NOALLOC_SCAN_INTS * sizeof(int) + sizeof(long long) + sizeof(Ctl);

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

namespace {
std::mutex g_setup_mu;
void *g_scratch_ptr[NOALLOC_MAX_DEVICES] = {};

// device address of g_noalloc_scratch on the current device (set-up on first use)
int scratch_for_current_device(unsigned char **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return HSMU_ERR_NO_DEVICE;
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return HSMU_ERR_INVALID;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return HSMU_ERR_CUDA;
        g_scratch_ptr[dev] = p;
    }
    *out = static_cast<unsigned char *>(g_scratch_ptr[dev]);
    return HSMU_OK;
}
}  // namespace

}  // namespace hsmu

using namespace hsmu;

extern "C" int hsmu_btiles_build_noalloc(const hsmu_csr *B, int32_t *tile_ptr, int32_t *tile_col, uint64_t *mask,
                                         int32_t *tile_off, void *stream) {
    if (!B || B->M < 0 || B->N < 0 || B->nnz < 0 || !B->row_ptr || !tile_ptr) return HSMU_ERR_INVALID;
    if (B->nnz > 0 && (!B->col || !tile_col || !mask || !tile_off)) return HSMU_ERR_INVALID;
    if (B->M > NOALLOC_MAX_ROWS) return HSMU_ERR_OVERFLOW;  // more rows than the static scratch holds
    unsigned char *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != HSMU_OK) return rc;
    int *scan_tmp = reinterpret_cast<int *>(scratch);
    long long *total = reinterpret_cast<long long *>(scratch + NOALLOC_SCAN_INTS * sizeof(int));
    Ctl *ctl = reinterpret_cast<Ctl *>(scratch + NOALLOC_SCAN_INTS * sizeof(int) + sizeof(long long));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return HSMU_ERR_CUDA;
    const DevCSR Bd{B->M, B->N, (long long)B->nnz, B->row_ptr, B->col, B->val};
    // the control word keeps the previous call's bits: clear it first
    if (cudaMemsetAsync(ctl, 0, sizeof(Ctl), st) != cudaSuccess) return HSMU_ERR_CUDA;
    // B is checked (row pointers non-decreasing within [0, nnz], columns sorted, unique and
    // in range) before any tile kernel indexes through it: a bad row pointer would make the
    // fill pass write past the caller's nnz-sized tile arrays
    launch_validate(Bd, ctl, nsm * 8, st);
    if (cudaGetLastError() != cudaSuccess) return HSMU_ERR_CUDA;
    int err = 0;
    if (cudaMemcpyAsync(&err, &ctl->err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return HSMU_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return HSMU_ERR_CUDA;
    if (err) return status_from_dev_err(err);
    // counts into tile_ptr[0..M), in-place exclusive scan (tile_ptr[M] = total), then the fill
    launch_tiles_count(Bd, tile_ptr, 0, ctl, nsm * 8, st);
    launch_scan(tile_ptr, tile_ptr, B->M, total, scan_tmp, ctl, st);
    launch_tiles_fill(Bd, tile_ptr, tile_col, reinterpret_cast<unsigned long long *>(mask), tile_off, ctl, nsm * 8, st);
    if (cudaGetLastError() != cudaSuccess) return HSMU_ERR_CUDA;
    if (cudaMemcpyAsync(&err, &ctl->err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return HSMU_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return HSMU_ERR_CUDA;
    return status_from_dev_err(err);
}
