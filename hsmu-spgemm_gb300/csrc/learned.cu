// Learned row scheduler: an FP32 MLP predicts every C row's nnz from cheap
// row features, so the exact symbolic count pass can be skipped.
//
// Plain engine:   bounds -> exact count -> scan -> allocate -> structure/values
// Learned engine: bounds -> features -> MLP -> speculative slots -> scan ->
//                 allocate -> structure/values into the slots (exact counts
//                 found on the way) -> scan of exact counts -> compaction ->
//                 redo of the rows that did not fit -> values of wide rows
// The structure pass builds every row's exact column set anyway, so it is
// also the exact count: every prediction is checked there, and a row whose
// nnz exceeds its slot is simply redone at its exact place after the scan.
// The output is identical to the plain engine's, bit for bit.  The model's
// job is to size the slots tightly (a safe bound such as the product count
// overallocates by ~18x on FEM matrices).
//
// Features (per row, log2(1 + x)): A-row nnz, sum of referenced B-row lengths
// (= intermediate products), longest referenced B row, column span of the
// C row (last - first column).  Target: log2(nnz of the C row).  Network:
// 4 -> 32 -> 32 -> 1, ReLU, inputs and target standardised with constants
// stored next to the weights.  Training (hand-written kernels): per block of
// 256 samples each thread runs forward and backward for one sample, the
// activations go to shared memory and the weight gradients are formed there
// as small outer-product sums (a 32x256 by 256x32 product for W2), then added
// to the global gradient; Adam updates the parameters.
//
// Parameter layout (floats): W1[32][4] b1[32] W2[32][32] b2[32] W3[32] b3[1]
// (MLP_NPARAM trainable), then mu[4] sd[4] ymu ysd (normalisation).
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstring>

#include "hsmu_common.cuh"
#include "hsmu_gb.h"
#include "hsmu_kernels.h"
#include "hsmu_rowops.cuh"

namespace hsmu {

constexpr int H = 32;
constexpr int NF = 4;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + H * NF, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H,
              OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + H, MLP_NPARAM = OFF_B3 + 1;
constexpr int OFF_MU = MLP_NPARAM, OFF_SD = OFF_MU + NF, OFF_YMU = OFF_SD + NF, OFF_YSD = OFF_YMU + 1,
              MLP_NTOTAL = OFF_YSD + 1;
static_assert(MLP_NTOTAL == HSMU_MLP_FLOATS, "parameter layout and the C ABI disagree");

// ---------------------------------------------------------------- features
template <int G>
__global__ void __launch_bounds__(256) k_features(int M, const int *__restrict__ arp, const int *__restrict__ acol,
                                                  const int *__restrict__ brp, const int *__restrict__ bcol,
                                                  float4 *__restrict__ feat, long long *__restrict__ prod_out) {
    constexpr int RPW = WARP / G;  // rows per warp per step
    const int sub = threadIdx.x & (G - 1);
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int rb = gw * RPW; rb < M; rb += nw * RPW) {  // uniform across the warp
        const int i = rb + (lane_id() / G);
        long long prod = 0;
        int mx = 0, cmin = INT_MAX, cmax = -1;
        if (i < M) {
            for (int p = arp[i] + sub; p < arp[i + 1]; p += G) {
                const int k = __ldg(acol + p);
                const int s = __ldg(brp + k), e = __ldg(brp + k + 1);
                prod += e - s;
                mx = max(mx, e - s);
                if (e > s) {
                    cmin = min(cmin, __ldg(bcol + s));
                    cmax = max(cmax, __ldg(bcol + e - 1));
                }
            }
        }
#pragma unroll
        for (int d = G / 2; d > 0; d >>= 1) {
            prod += __shfl_xor_sync(FULL, prod, d, G);
            mx = max(mx, __shfl_xor_sync(FULL, mx, d, G));
            cmin = min(cmin, __shfl_xor_sync(FULL, cmin, d, G));
            cmax = max(cmax, __shfl_xor_sync(FULL, cmax, d, G));
        }
        if (i < M && sub == 0) {
            const int na = arp[i + 1] - arp[i];
            const float span = cmax >= cmin ? (float)(cmax - cmin) : 0.f;
            feat[i] = make_float4(log2f(1.f + (float)na), log2f(1.f + (float)prod), log2f(1.f + (float)mx),
                                  log2f(1.f + span));
            if (prod_out) prod_out[i] = prod;
        }
    }
}

void launch_features(const DevCSR &A, const DevCSR &B, float4 *feat, long long *prod_out, int nsm, cudaStream_t st) {
    const double avg = A.M ? (double)A.nnz / A.M : 0.0;
    const int grid = nsm * 8;
    if (avg <= 6) k_features<4><<<grid, 256, 0, st>>>(A.M, A.rp, A.col, B.rp, B.col, feat, prod_out);
    else if (avg <= 24) k_features<16><<<grid, 256, 0, st>>>(A.M, A.rp, A.col, B.rp, B.col, feat, prod_out);
    else k_features<32><<<grid, 256, 0, st>>>(A.M, A.rp, A.col, B.rp, B.col, feat, prod_out);
}

// ---------------------------------------------------------------- MLP
__device__ __forceinline__ float mlp_eval(const float *P, float4 f, float *h1, float *h2, float *z1, float *z2) {
    const float x[NF] = {(f.x - P[OFF_MU + 0]) / P[OFF_SD + 0], (f.y - P[OFF_MU + 1]) / P[OFF_SD + 1],
                         (f.z - P[OFF_MU + 2]) / P[OFF_SD + 2], (f.w - P[OFF_MU + 3]) / P[OFF_SD + 3]};
#pragma unroll
    for (int j = 0; j < H; j++) {
        float a = P[OFF_B1 + j];
#pragma unroll
        for (int i = 0; i < NF; i++) a = fmaf(P[OFF_W1 + j * NF + i], x[i], a);
        if (z1) z1[j] = a;
        h1[j] = fmaxf(a, 0.f);
    }
#pragma unroll 4
    for (int j = 0; j < H; j++) {
        float a = P[OFF_B2 + j];
#pragma unroll
        for (int i = 0; i < H; i++) a = fmaf(P[OFF_W2 + j * H + i], h1[i], a);
        if (z2) z2[j] = a;
        h2[j] = fmaxf(a, 0.f);
    }
    float o = P[OFF_B3];
#pragma unroll
    for (int i = 0; i < H; i++) o = fmaf(P[OFF_W3 + i], h2[i], o);
    return o;  // standardised log2(nnz)
}

__global__ void __launch_bounds__(256) k_mlp_forward(const float *__restrict__ params, const float4 *__restrict__ X,
                                                     int n, float *__restrict__ y) {
    __shared__ float P[MLP_NTOTAL];
    for (int q = threadIdx.x; q < MLP_NTOTAL; q += blockDim.x) P[q] = params[q];
    __syncthreads();
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        float h1[H], h2[H];
        const float o = mlp_eval(P, X[s], h1, h2, nullptr, nullptr);
        y[s] = o * P[OFF_YSD] + P[OFF_YMU];
    }
}

constexpr int GB = 256;  // samples per block in the gradient kernel

struct GradSmem {
    float h1[GB][H + 1];
    float dh1[GB][H + 1];
    float dh2[GB][H + 1];
    float h2[GB][H + 1];
    float x[GB][NF];
    float d[GB];
    float P[MLP_NTOTAL];
};

// Loss = 0.5 * sum over samples of (out - (y - ymu) / ysd)^2; adds d loss / d params
// (first MLP_NPARAM entries of grad) and the loss to *loss.
__global__ void __launch_bounds__(GB) k_mlp_grad(const float *__restrict__ params, const float4 *__restrict__ X,
                                                 const float *__restrict__ Y, int n, float *__restrict__ grad,
                                                 float *__restrict__ loss) {
    extern __shared__ float s_dynf[];
    GradSmem &S = *reinterpret_cast<GradSmem *>(s_dynf);
    for (int q = threadIdx.x; q < MLP_NTOTAL; q += blockDim.x) S.P[q] = params[q];
    __syncthreads();
    const float *P = S.P;
    float my_loss = 0.f;
    for (int base = blockIdx.x * GB; base < n; base += gridDim.x * GB) {
        const int s = base + threadIdx.x;
        const int t = threadIdx.x;
        if (s < n) {
            const float4 f = X[s];
            float h1[H], h2[H], z1[H], z2[H];
            const float o = mlp_eval(P, f, h1, h2, z1, z2);
            const float tgt = (Y[s] - P[OFF_YMU]) / P[OFF_YSD];
            const float d = o - tgt;
            my_loss += 0.5f * d * d;
            S.d[t] = d;
            S.x[t][0] = (f.x - P[OFF_MU + 0]) / P[OFF_SD + 0];
            S.x[t][1] = (f.y - P[OFF_MU + 1]) / P[OFF_SD + 1];
            S.x[t][2] = (f.z - P[OFF_MU + 2]) / P[OFF_SD + 2];
            S.x[t][3] = (f.w - P[OFF_MU + 3]) / P[OFF_SD + 3];
            float dh2[H];
#pragma unroll
            for (int j = 0; j < H; j++) {
                dh2[j] = z2[j] > 0.f ? d * P[OFF_W3 + j] : 0.f;
                S.h1[t][j] = h1[j];
                S.h2[t][j] = h2[j];
                S.dh2[t][j] = dh2[j];
            }
#pragma unroll 4
            for (int i = 0; i < H; i++) {
                float a = 0.f;
#pragma unroll
                for (int j = 0; j < H; j++) a = fmaf(P[OFF_W2 + j * H + i], dh2[j], a);
                S.dh1[t][i] = z1[i] > 0.f ? a : 0.f;
            }
        } else {
            S.d[t] = 0.f;
#pragma unroll
            for (int j = 0; j < H; j++) S.h1[t][j] = S.h2[t][j] = S.dh2[t][j] = S.dh1[t][j] = 0.f;
            for (int i = 0; i < NF; i++) S.x[t][i] = 0.f;
        }
        __syncthreads();
        // weight gradients as sums over the block's samples
        for (int q = threadIdx.x; q < MLP_NPARAM; q += blockDim.x) {
            float a = 0.f;
            if (q < OFF_B1) {  // W1[j][i] = sum dh1[j] x[i]
                const int j = q / NF, i = q % NF;
                for (int r = 0; r < GB; r++) a = fmaf(S.dh1[r][j], S.x[r][i], a);
            } else if (q < OFF_W2) {  // b1
                const int j = q - OFF_B1;
                for (int r = 0; r < GB; r++) a += S.dh1[r][j];
            } else if (q < OFF_B2) {  // W2[j][i] = sum dh2[j] h1[i]
                const int j = (q - OFF_W2) / H, i = (q - OFF_W2) % H;
                for (int r = 0; r < GB; r++) a = fmaf(S.dh2[r][j], S.h1[r][i], a);
            } else if (q < OFF_W3) {  // b2
                const int j = q - OFF_B2;
                for (int r = 0; r < GB; r++) a += S.dh2[r][j];
            } else if (q < OFF_B3) {  // W3[i] = sum d h2[i]
                const int i = q - OFF_W3;
                for (int r = 0; r < GB; r++) a = fmaf(S.d[r], S.h2[r][i], a);
            } else {  // b3
                for (int r = 0; r < GB; r++) a += S.d[r];
            }
            atomicAdd(grad + q, a);
        }
        __syncthreads();
    }
    my_loss = warp_sum(my_loss);
    if (lane_id() == 0) atomicAdd(loss, my_loss);
}

__global__ void k_adam(float *__restrict__ params, const float *__restrict__ grad, float *__restrict__ m,
                       float *__restrict__ v, int np, float lr, float b1, float b2, float eps, float scale, int step) {
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < np; q += gridDim.x * blockDim.x) {
        const float g = grad[q] * scale;
        const float mq = b1 * m[q] + (1.f - b1) * g;
        const float vq = b2 * v[q] + (1.f - b2) * g * g;
        m[q] = mq;
        v[q] = vq;
        params[q] -= lr * (mq / c1) / (sqrtf(vq / c2) + eps);
    }
}

// ---------------------------------------------------------------- speculative slots
// capacity of row i: exact bound for rows with <= TINY_MAX products (they
// always fit), min(products, N, 2^(prediction + margin)) otherwise; large rows
// that keep a tile list take none (large_no_slot).  wide_prod: the products of
// the warp-class rows predicted clearly wider than the fused warp path (what
// the prediction can save is their count pass).
__global__ void __launch_bounds__(256) k_capacity(const float *__restrict__ params, const float4 *__restrict__ feat,
                                                  const long long *__restrict__ prod, int M, int N, float margin,
                                                  int *__restrict__ cap, unsigned long long *wide_prod,
                                                  const signed char *__restrict__ cls, bool large_no_slot) {
    __shared__ float P[MLP_NTOTAL];
    __shared__ unsigned long long s_wide;
    for (int q = threadIdx.x; q < MLP_NTOTAL; q += blockDim.x) P[q] = params[q];
    if (threadIdx.x == 0) s_wide = 0;
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
        const long long pr = prod[i];
        const long long bound = pr < (long long)N ? pr : (long long)N;
        long long c = bound;
        bool w = false;  // predicted clearly wider than the fused warp path (routing only)
        if (pr > TINY_MAX) {
            float h1[H], h2[H];
            const float y = mlp_eval(P, feat[i], h1, h2, nullptr, nullptr) * P[OFF_YSD] + P[OFF_YMU];
            const float e = fminf(y + margin, 31.f);
            const long long pc = (long long)ceilf(exp2f(fmaxf(e, 0.f)));
            c = pc < bound ? pc : bound;
            if (c < 1) c = 1;
            w = y > log2f((float)FUSE_CAP) + 0.5f && bound > FUSE_CAP;  // half a step of slack
        }
        const bool large = cls[i] == BIN_L;
        if (large && large_no_slot) c = 0;  // a large row with a tile list takes no slot
        cap[i] = (int)c;
        if (w && !large) atomicAdd(&s_wide, (unsigned long long)pr);
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_wide && wide_prod) atomicAdd(wide_prod, s_wide);
}

// copy rows fused in their speculative slots (columns and values, at most a
// few hundred entries each) to their final place; the columns of wider rows
// are copied by the value kernel, window by window
__global__ void __launch_bounds__(256) k_compact(int M, const long long *__restrict__ soff,
                                                 const int *__restrict__ crp, const unsigned char *__restrict__ flag,
                                                 const int *__restrict__ scol, const double *__restrict__ sval,
                                                 int *__restrict__ ccol, double *__restrict__ cval) {
    const int lane = lane_id();
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = gw; i < M; i += nw) {
        if (flag[i] != ROW_VALUES) continue;
        const long long src = soff[i];
        const int dst = crp[i], n = crp[i + 1] - dst;
        for (int q = lane; q < n; q += WARP) {
            ccol[dst + q] = scol[src + q];
            cval[dst + q] = sval[src + q];
        }
    }
}

void launch_capacity(const float *params, const float4 *feat, const long long *prod, const signed char *cls, int M,
                     int N, float margin, int *cap, int nsm, cudaStream_t st, unsigned long long *wide_prod,
                     bool large_no_slot) {
    k_capacity<<<nsm * 4, 256, 0, st>>>(params, feat, prod, M, N, margin, cap, wide_prod, cls, large_no_slot);
}

void launch_compact(int M, const long long *soff, const int *crp, const unsigned char *flag, const int *scol,
                    const double *sval, int *ccol, double *cval, int nsm, cudaStream_t st) {
    k_compact<<<nsm * 8, 256, 0, st>>>(M, soff, crp, flag, scol, sval, ccol, cval);
}

}  // namespace hsmu

using namespace hsmu;

namespace {
int cuerr(cudaError_t e) { return e == cudaSuccess ? HSMU_OK : (e == cudaErrorMemoryAllocation ? HSMU_ERR_ALLOC : HSMU_ERR_CUDA); }
}  // namespace

extern "C" {

int hsmu_row_features(hsmu_handle h, const hsmu_csr *A, const hsmu_csr *B, float *feat, int64_t *products,
                      void *stream) {
    (void)h;
    if (!A || !B || !feat || A->N != B->M) return HSMU_ERR_INVALID;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const DevCSR Ad{A->M, A->N, (long long)A->nnz, A->row_ptr, A->col, A->val};
    const DevCSR Bd{B->M, B->N, (long long)B->nnz, B->row_ptr, B->col, B->val};
    launch_features(Ad, Bd, reinterpret_cast<float4 *>(feat), reinterpret_cast<long long *>(products), nsm,
                    static_cast<cudaStream_t>(stream));
    return cuerr(cudaGetLastError());
}

int hsmu_mlp_forward(const float *params, const float *feat, int n, float *out, void *stream) {
    if (!params || (n > 0 && (!feat || !out)) || n < 0) return HSMU_ERR_INVALID;
    if (n == 0) return HSMU_OK;
    k_mlp_forward<<<min(1024, (n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        params, reinterpret_cast<const float4 *>(feat), n, out);
    return cuerr(cudaGetLastError());
}

int hsmu_mlp_grad(const float *params, const float *feat, const float *target, int n, float *grad, float *loss,
                  void *stream) {
    if (!params || !grad || !loss || n < 0 || (n > 0 && (!feat || !target))) return HSMU_ERR_INVALID;
    static bool configured = false;
    if (!configured) {
        if (cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(GradSmem)))
            return HSMU_ERR_CUDA;
        configured = true;
    }
    if (n == 0) return HSMU_OK;
    k_mlp_grad<<<min(304, (n + GB - 1) / GB), GB, sizeof(GradSmem), static_cast<cudaStream_t>(stream)>>>(
        params, reinterpret_cast<const float4 *>(feat), target, n, grad, loss);
    return cuerr(cudaGetLastError());
}

int hsmu_mlp_adam(float *params, const float *grad, float *m, float *v, float lr, float scale, int step,
                  void *stream) {
    if (!params || !grad || !m || !v || step < 1) return HSMU_ERR_INVALID;
    k_adam<<<(MLP_NPARAM + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(params, grad, m, v, MLP_NPARAM, lr,
                                                                                   0.9f, 0.999f, 1e-8f, scale, step);
    return cuerr(cudaGetLastError());
}

}  // extern "C"
