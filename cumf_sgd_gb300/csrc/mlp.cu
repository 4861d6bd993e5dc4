// mlp.cu - the learned warm start: user features and a small MLP that maps them to an
// initial user-factor row, trained and run on the tensor cores (tc_gemm.cu).
//
// Features of user u (k + 3 values), from the user's ratings and the item factors Q:
//   x[0:k] = sum_i (r_ui - mean_u) q_i / deg_u      (rating-centred mean of the rated items)
//   x[k]   = log(1 + deg_u) / 4,  x[k+1] = (mean_u - 3) / 2,  x[k+2] = var_u / 2
// The centred mean is zero for a user with one rating, so users with few ratings stay inside
// the range the network was trained on (an uncentred mean of one item's factors does not).
// MLP: d_in -> H (GELU) -> H (GELU) -> d_out, bf16 weights and activations, fp32
// accumulation (tcgen05), fp32 master weights updated with Adam.  Every matrix product of the
// forward and backward passes is a TN product C = A B^T on the tcgen05 GEMM:
//   forward   H1 = gelu(X W1^T + b1), H2 = gelu(H1 W2^T + b2), Y = H2 W3^T + b3
//   backward  dW = dZ^T A  ->  (dZ^T)(A^T)^T on transposed copies; dA = dZ W -> dZ (W^T)^T
// Loss: mean over rows of the squared error summed over the output dimension.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <string>
#include <vector>

#include "cumf_sgd.h"
#include "internal.h"
#include "rng.h"
#include "train_common.h"

namespace cumf {

cudaError_t launch_tc_gemm(const void *A, const void *B, int M, int N, int K, const float *bias, int act,
                           void *out, int out_f32, int ldo, float *pre_out, int *status, cudaStream_t s);

namespace {

constexpr int kT = 256;

int grid_of(int64_t n) {
    int64_t g = (n + kT - 1) / kT;
    if (g > 152 * 64) g = 152 * 64;
    return (int)(g < 1 ? 1 : g);
}

// ---- feature gather --------------------------------------------------------------------

__global__ void user_stats_kernel(const cumf_node *R, int64_t nnz, int32_t m, int32_t n, float *deg, float *sum,
                                  float *sum2) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        const cumf_node x = R[i];
        if ((uint32_t)x.u >= (uint32_t)m || (uint32_t)x.v >= (uint32_t)n) continue;
        atomicAdd(deg + x.u, 1.f);
        atomicAdd(sum + x.u, x.r);
        atomicAdd(sum2 + x.u, x.r * x.r);
    }
}

// One warp per rating: acc[u][0:k] += (r - mean_u) q_v / deg_u.
__global__ void user_qsum_kernel(const cumf_node *R, int64_t nnz, int32_t m, int32_t n, const float *Q, int k,
                                 const float *deg, const float *sum, float *X, int ldx) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = w0; i < nnz; i += nw) {
        const cumf_node x = R[i];
        if ((uint32_t)x.u >= (uint32_t)m || (uint32_t)x.v >= (uint32_t)n) continue;
        const float d = deg[x.u];
        const float c = (x.r - sum[x.u] / d) / d;
        const float *q = Q + (int64_t)x.v * k;
        float *dst = X + (int64_t)x.u * ldx;
        if ((k & 3) == 0 && (ldx & 3) == 0) {  // 16-byte vector atomics (sm_90+)
            const float4 *q4 = reinterpret_cast<const float4 *>(q);
            float4 *d4 = reinterpret_cast<float4 *>(dst);
            for (int j = lane; j < (k >> 2); j += 32) {
                const float4 a = q4[j];
                atomicAdd(d4 + j, make_float4(c * a.x, c * a.y, c * a.z, c * a.w));
            }
        } else {
            for (int j = lane; j < k; j += 32) atomicAdd(dst + j, c * q[j]);
        }
    }
}

__global__ void user_scalar_kernel(int32_t m, int k, const float *deg, const float *sum, const float *sum2, float *X,
                                   int ldx) {
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < m; u += (int64_t)gridDim.x * blockDim.x) {
        const float d = deg[u];
        const float mean = d > 0 ? sum[u] / d : 0.f;
        const float var = d > 0 ? fmaxf(sum2[u] / d - mean * mean, 0.f) : 0.f;
        float *x = X + u * ldx;
        x[k] = logf(1.f + d) * 0.25f;
        x[k + 1] = d > 0 ? (mean - 3.f) * 0.5f : 0.f;
        x[k + 2] = var * 0.5f;
    }
}

// ---- elementwise helpers ---------------------------------------------------------------

// rows x cols fp32 (row stride lds) -> rows x ldd bf16, zero padding for cols..ldd.
__global__ void to_bf16_pad_kernel(const float *S, int64_t rows, int cols, int lds, __nv_bfloat16 *D, int ldd) {
    const int64_t total = rows * ldd;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / ldd;
        const int c = (int)(i - r * ldd);
        D[i] = __float2bfloat16_rn(c < cols ? S[r * lds + c] : 0.f);
    }
}

// D[c][r] = S[r][c] for a rows x cols bf16 matrix (tiled through shared memory).
// Row tiles run along gridDim.x (up to 2^31 - 1), column tiles along gridDim.y.
__global__ void transpose_bf16_kernel(const __nv_bfloat16 *S, int rows, int cols, __nv_bfloat16 *D) {
    __shared__ __nv_bfloat16 tile[32][33];
    const int bx = blockIdx.y * 32, by = blockIdx.x * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int r = by + j, c = bx + threadIdx.x;
        tile[j][threadIdx.x] = (r < rows && c < cols) ? S[(int64_t)r * cols + c] : __float2bfloat16_rn(0.f);
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int c = bx + j, r = by + threadIdx.x;
        if (c < cols && r < rows) D[(int64_t)c * rows + r] = tile[threadIdx.x][j];
    }
}

__device__ __forceinline__ float gelu_grad(float x) {
    const float c = 0.7978845608028654f;
    const float u = c * (x + 0.044715f * x * x * x);
    const float t = tanhf(u);
    return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * c * (1.f + 3.f * 0.044715f * x * x);
}

// dZ = dA * gelu'(pre) -> bf16; rows beyond `valid` are zero.
__global__ void gelu_back_kernel(const float *dA, const float *pre, int64_t rows, int64_t valid, int cols,
                                 __nv_bfloat16 *dZ) {
    const int64_t total = rows * cols;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / cols;
        dZ[i] = __float2bfloat16_rn(r < valid ? dA[i] * gelu_grad(pre[i]) : 0.f);
    }
}

// dY = 2 (Y - T) / B (bf16, zero for padding rows) and the loss partial sums.
__global__ void mse_grad_kernel(const float *Y, const float *T, int64_t rows, int64_t valid, int cols, float inv_b,
                                __nv_bfloat16 *dY, double *loss) {
    double acc = 0;
    const int64_t total = rows * cols;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / cols;
        float g = 0.f;
        if (r < valid) {
            const float d = Y[i] - T[i];
            acc += (double)d * d;
            g = 2.f * d * inv_b;
        }
        dY[i] = __float2bfloat16_rn(g);
    }
    for (int o = 16; o >= 1; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, acc);
}

// bias gradient: column sums of a rows x cols bf16 matrix.
__global__ void colsum_kernel(const __nv_bfloat16 *Z, int64_t rows, int cols, float *out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float s = 0.f;
    for (int64_t r = 0; r < rows; ++r) s += __bfloat162float(Z[r * cols + c]);
    out[c] = s;
}

__global__ void adam_kernel(float *w, const float *g, float *m1, float *m2, int64_t n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float a = b1 * m1[i] + (1.f - b1) * gi;
        const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
        m1[i] = a;
        m2[i] = b;
        w[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
    }
}

__global__ void init_weights_kernel(float *w, int64_t n, float scale, uint64_t key) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        // uniform(-scale, scale) from the counter hash
        const float u = init_uniform(key, (uint64_t)i);  // (0, 1]
        w[i] = (2.f * u - 1.f) * scale;
    }
}

__global__ void gather_rows_kernel(const float *S, int ld, const int32_t *idx, int64_t rows, float *D) {
    const int64_t total = rows * ld;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / ld;
        D[i] = S[(int64_t)idx[r] * ld + (i - r * ld)];
    }
}

}  // namespace

struct Mlp {
    int d_in, dp, h, d_out;  // dp = d_in padded to a multiple of 64
    // fp32 parameters (flattened: W1[h][d_in], b1[h], W2[h][h], b2[h], W3[d_out][h], b3[d_out])
    DevBuf params, grads, m1, m2;
    int64_t count = 0;
    int64_t off_w1, off_b1, off_w2, off_b2, off_w3, off_b3;
    // bf16 operand copies: W1p[h][dp], W2[h][h], W3[d_out][h] and transposes W2T[h][h], W3T[h][d_out]
    DevBuf w1b, w2b, w3b, w2t, w3t;
    DevBuf status;
    int64_t step = 0;
    // workspace for one batch of up to cap rows
    int64_t cap = 0;
    DevBuf xb, h1, h2, pre1, pre2, y, dy, dyt, h2t, h1t, xbt, dh2, dp2, dp2t, dh1, dp1, dp1t, loss;
    DevBuf gw1p;  // gradient of W1 in padded layout [h][dp]
};

namespace {

int mlp_ensure(Mlp *mp, int64_t rows) {
    if (rows <= mp->cap) return CUMF_OK;
    const int64_t r = (rows + 127) / 128 * 128;
    const size_t b2 = 2;
    const int h = mp->h, dp = mp->dp, dout = mp->d_out;
    CUMF_CUDA(mp->xb.alloc(r * dp * b2));
    CUMF_CUDA(mp->h1.alloc(r * h * b2));
    CUMF_CUDA(mp->h2.alloc(r * h * b2));
    CUMF_CUDA(mp->pre1.alloc(r * h * 4));
    CUMF_CUDA(mp->pre2.alloc(r * h * 4));
    CUMF_CUDA(mp->y.alloc(r * dout * 4));
    CUMF_CUDA(mp->dy.alloc(r * dout * b2));
    CUMF_CUDA(mp->dyt.alloc(r * dout * b2));
    CUMF_CUDA(mp->h2t.alloc(r * h * b2));
    CUMF_CUDA(mp->h1t.alloc(r * h * b2));
    CUMF_CUDA(mp->xbt.alloc(r * dp * b2));
    CUMF_CUDA(mp->dh2.alloc(r * h * 4));
    CUMF_CUDA(mp->dp2.alloc(r * h * b2));
    CUMF_CUDA(mp->dp2t.alloc(r * h * b2));
    CUMF_CUDA(mp->dh1.alloc(r * h * 4));
    CUMF_CUDA(mp->dp1.alloc(r * h * b2));
    CUMF_CUDA(mp->dp1t.alloc(r * h * b2));
    mp->cap = r;
    return CUMF_OK;
}

cudaError_t transpose(const void *S, int rows, int cols, void *D, cudaStream_t s) {
    dim3 grid((rows + 31) / 32, (cols + 31) / 32), block(32, 8);
    if (grid.y > 65535) return cudaErrorInvalidValue;
    transpose_bf16_kernel<<<grid, block, 0, s>>>(reinterpret_cast<const __nv_bfloat16 *>(S), rows, cols,
                                                  reinterpret_cast<__nv_bfloat16 *>(D));
    return cudaGetLastError();
}

// bf16 operand copies of the fp32 master weights.
int mlp_refresh(Mlp *mp, cudaStream_t s) {
    const float *P = mp->params.as<float>();
    const int h = mp->h, dout = mp->d_out;
    to_bf16_pad_kernel<<<grid_of((int64_t)h * mp->dp), kT, 0, s>>>(P + mp->off_w1, h, mp->d_in, mp->d_in,
                                                                     mp->w1b.as<__nv_bfloat16>(), mp->dp);
    to_bf16_pad_kernel<<<grid_of((int64_t)h * h), kT, 0, s>>>(P + mp->off_w2, h, h, h, mp->w2b.as<__nv_bfloat16>(), h);
    to_bf16_pad_kernel<<<grid_of((int64_t)dout * h), kT, 0, s>>>(P + mp->off_w3, dout, h, h,
                                                                   mp->w3b.as<__nv_bfloat16>(), h);
    CUMF_CUDA(cudaGetLastError());
    CUMF_CUDA(transpose(mp->w2b.p, h, h, mp->w2t.p, s));
    CUMF_CUDA(transpose(mp->w3b.p, dout, h, mp->w3t.p, s));
    return CUMF_OK;
}

// Forward over rows [0, rows) of X (fp32, rows x d_in); Y (fp32 rows x d_out) in mp->y.
int mlp_forward_ws(Mlp *mp, const float *X, int64_t rows, cudaStream_t s) {
    if (int rc = mlp_ensure(mp, rows)) return rc;
    const float *P = mp->params.as<float>();
    const int h = mp->h;
    const int64_t rp = (rows + 127) / 128 * 128;  // padding rows are zero
    CUMF_CUDA(cudaMemsetAsync(mp->xb.p, 0, rp * mp->dp * 2, s));
    to_bf16_pad_kernel<<<grid_of(rows * mp->dp), kT, 0, s>>>(X, rows, mp->d_in, mp->d_in, mp->xb.as<__nv_bfloat16>(),
                                                               mp->dp);
    CUMF_CUDA(cudaGetLastError());
    int *st = mp->status.as<int>();
    CUMF_CUDA(launch_tc_gemm(mp->xb.p, mp->w1b.p, (int)rp, h, mp->dp, P + mp->off_b1, 1, mp->h1.p, 0, h,
                             mp->pre1.as<float>(), st, s));
    CUMF_CUDA(launch_tc_gemm(mp->h1.p, mp->w2b.p, (int)rp, h, h, P + mp->off_b2, 1, mp->h2.p, 0, h,
                             mp->pre2.as<float>(), st, s));
    CUMF_CUDA(launch_tc_gemm(mp->h2.p, mp->w3b.p, (int)rp, mp->d_out, h, P + mp->off_b3, 0, mp->y.p, 1, mp->d_out,
                             nullptr, st, s));
    return CUMF_OK;
}

// Loss and gradients (into mp->grads) for rows [0, rows) with targets T (fp32 rows x d_out).
int mlp_backward_ws(Mlp *mp, const float *T, int64_t rows, cudaStream_t s) {
    const int h = mp->h, dout = mp->d_out, dp = mp->dp;
    const int64_t rp = (rows + 127) / 128 * 128;
    float *G = mp->grads.as<float>();
    int *st = mp->status.as<int>();
    CUMF_CUDA(cudaMemsetAsync(mp->loss.p, 0, sizeof(double), s));
    mse_grad_kernel<<<grid_of(rp * dout), kT, 0, s>>>(mp->y.as<float>(), T, rp, rows, dout, 1.f / (float)rows,
                                                       mp->dy.as<__nv_bfloat16>(), mp->loss.as<double>());
    CUMF_CUDA(cudaGetLastError());
    // layer 3: dW3 = dY^T H2, db3 = colsum(dY), dH2 = dY W3
    CUMF_CUDA(transpose(mp->dy.p, (int)rp, dout, mp->dyt.p, s));
    CUMF_CUDA(transpose(mp->h2.p, (int)rp, h, mp->h2t.p, s));
    CUMF_CUDA(launch_tc_gemm(mp->dyt.p, mp->h2t.p, dout, h, (int)rp, nullptr, 0, G + mp->off_w3, 1, h, nullptr, st, s));
    colsum_kernel<<<(dout + 127) / 128, 128, 0, s>>>(mp->dy.as<__nv_bfloat16>(), rp, dout, G + mp->off_b3);
    CUMF_CUDA(launch_tc_gemm(mp->dy.p, mp->w3t.p, (int)rp, h, dout, nullptr, 0, mp->dh2.p, 1, h, nullptr, st, s));
    gelu_back_kernel<<<grid_of(rp * h), kT, 0, s>>>(mp->dh2.as<float>(), mp->pre2.as<float>(), rp, rows, h,
                                                     mp->dp2.as<__nv_bfloat16>());
    // layer 2
    CUMF_CUDA(transpose(mp->dp2.p, (int)rp, h, mp->dp2t.p, s));
    CUMF_CUDA(transpose(mp->h1.p, (int)rp, h, mp->h1t.p, s));
    CUMF_CUDA(launch_tc_gemm(mp->dp2t.p, mp->h1t.p, h, h, (int)rp, nullptr, 0, G + mp->off_w2, 1, h, nullptr, st, s));
    colsum_kernel<<<(h + 127) / 128, 128, 0, s>>>(mp->dp2.as<__nv_bfloat16>(), rp, h, G + mp->off_b2);
    CUMF_CUDA(launch_tc_gemm(mp->dp2.p, mp->w2t.p, (int)rp, h, h, nullptr, 0, mp->dh1.p, 1, h, nullptr, st, s));
    gelu_back_kernel<<<grid_of(rp * h), kT, 0, s>>>(mp->dh1.as<float>(), mp->pre1.as<float>(), rp, rows, h,
                                                     mp->dp1.as<__nv_bfloat16>());
    // layer 1 (padded input columns give zero gradient columns, dropped on copy)
    CUMF_CUDA(transpose(mp->dp1.p, (int)rp, h, mp->dp1t.p, s));
    CUMF_CUDA(transpose(mp->xb.p, (int)rp, dp, mp->xbt.p, s));
    CUMF_CUDA(launch_tc_gemm(mp->dp1t.p, mp->xbt.p, h, dp, (int)rp, nullptr, 0, mp->gw1p.p, 1, dp, nullptr, st, s));
    CUMF_CUDA(cudaMemcpy2DAsync(G + mp->off_w1, mp->d_in * sizeof(float), mp->gw1p.p, dp * sizeof(float),
                                mp->d_in * sizeof(float), h, cudaMemcpyDeviceToDevice, s));
    colsum_kernel<<<(h + 127) / 128, 128, 0, s>>>(mp->dp1.as<__nv_bfloat16>(), rp, h, G + mp->off_b1);
    CUMF_CUDA(cudaGetLastError());
    return CUMF_OK;
}

int mlp_check_status(Mlp *mp, cudaStream_t s) {
    int st = 0;
    CUMF_CUDA(cudaMemcpyAsync(&st, mp->status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUMF_CUDA(cudaStreamSynchronize(s));
    if (st) return fail(CUMF_ERR_TIMEOUT, "a tensor-core GEMM gave up waiting");
    return CUMF_OK;
}

}  // namespace

}  // namespace cumf

using namespace cumf;

extern "C" {

int cumf_mlp_create(int d_in, int hidden, int d_out, uint64_t seed, void **out) {
    if (!out || d_in <= 0 || hidden <= 0 || d_out <= 0 || hidden % 64 || d_out % 64)
        return fail(CUMF_ERR_ARG, "mlp_create: hidden and d_out must be positive multiples of 64");
    Mlp *mp = new Mlp();
    mp->d_in = d_in;
    mp->dp = (d_in + 63) / 64 * 64;
    mp->h = hidden;
    mp->d_out = d_out;
    int64_t o = 0;
    mp->off_w1 = o; o += (int64_t)hidden * d_in;
    mp->off_b1 = o; o += hidden;
    mp->off_w2 = o; o += (int64_t)hidden * hidden;
    mp->off_b2 = o; o += hidden;
    mp->off_w3 = o; o += (int64_t)d_out * hidden;
    mp->off_b3 = o; o += d_out;
    mp->count = o;
    auto cleanup = [&](int rc) { delete mp; return rc; };
    if (cudaError_t e = mp->params.alloc(o * 4)) return cleanup(cuda_fail(e, "mlp params"));
    if (cudaError_t e = mp->grads.alloc(o * 4)) return cleanup(cuda_fail(e, "mlp grads"));
    if (cudaError_t e = mp->m1.alloc(o * 4)) return cleanup(cuda_fail(e, "mlp adam"));
    if (cudaError_t e = mp->m2.alloc(o * 4)) return cleanup(cuda_fail(e, "mlp adam"));
    if (cudaError_t e = mp->w1b.alloc((size_t)hidden * mp->dp * 2)) return cleanup(cuda_fail(e, "mlp w1"));
    if (cudaError_t e = mp->w2b.alloc((size_t)hidden * hidden * 2)) return cleanup(cuda_fail(e, "mlp w2"));
    if (cudaError_t e = mp->w3b.alloc((size_t)d_out * hidden * 2)) return cleanup(cuda_fail(e, "mlp w3"));
    if (cudaError_t e = mp->w2t.alloc((size_t)hidden * hidden * 2)) return cleanup(cuda_fail(e, "mlp w2t"));
    if (cudaError_t e = mp->w3t.alloc((size_t)d_out * hidden * 2)) return cleanup(cuda_fail(e, "mlp w3t"));
    if (cudaError_t e = mp->gw1p.alloc((size_t)hidden * mp->dp * 4)) return cleanup(cuda_fail(e, "mlp gw1"));
    if (cudaError_t e = mp->status.alloc(sizeof(int))) return cleanup(cuda_fail(e, "mlp status"));
    if (cudaError_t e = mp->loss.alloc(sizeof(double))) return cleanup(cuda_fail(e, "mlp loss"));
    cudaMemset(mp->status.p, 0, sizeof(int));
    cudaMemset(mp->m1.p, 0, o * 4);
    cudaMemset(mp->m2.p, 0, o * 4);
    cudaMemset(mp->params.p, 0, o * 4);  // biases start at zero
    // Weights U(-a, a) with a = sqrt(6 / (fan_in + fan_out)) (Glorot uniform).
    float *P = mp->params.as<float>();
    const struct { int64_t off, n; int fi, fo; } layers[3] = {
        {mp->off_w1, (int64_t)hidden * d_in, d_in, hidden},
        {mp->off_w2, (int64_t)hidden * hidden, hidden, hidden},
        {mp->off_w3, (int64_t)d_out * hidden, hidden, d_out}};
    for (int l = 0; l < 3; ++l)
        init_weights_kernel<<<grid_of(layers[l].n), kT>>>(P + layers[l].off, layers[l].n,
                                                           sqrtf(6.f / (layers[l].fi + layers[l].fo)),
                                                           init_key(seed, 10 + l));
    if (int rc = mlp_refresh(mp, 0)) return cleanup(rc);
    if (cudaError_t e = cudaDeviceSynchronize()) return cleanup(cuda_fail(e, "mlp init"));
    *out = mp;
    return CUMF_OK;
}

int cumf_mlp_destroy(void *mlp) {
    delete static_cast<Mlp *>(mlp);
    return CUMF_OK;
}

int64_t cumf_mlp_param_count(void *mlp) { return mlp ? static_cast<Mlp *>(mlp)->count : 0; }

int cumf_mlp_get_params(void *mlp, float *host, int64_t count, int which) {
    Mlp *mp = static_cast<Mlp *>(mlp);
    if (!mp || !host || count != mp->count || which < 0 || which > 1) return fail(CUMF_ERR_ARG, "mlp_get_params");
    CUMF_CUDA(cudaMemcpy(host, which ? mp->grads.p : mp->params.p, count * 4, cudaMemcpyDeviceToHost));
    return CUMF_OK;
}

int cumf_mlp_set_params(void *mlp, const float *host, int64_t count) {
    Mlp *mp = static_cast<Mlp *>(mlp);
    if (!mp || !host || count != mp->count) return fail(CUMF_ERR_ARG, "mlp_set_params");
    CUMF_CUDA(cudaMemcpy(mp->params.p, host, count * 4, cudaMemcpyHostToDevice));
    if (int rc = mlp_refresh(mp, 0)) return rc;
    CUMF_CUDA(cudaDeviceSynchronize());
    return CUMF_OK;
}

int cumf_mlp_forward(void *mlp, const float *d_X, int64_t rows, float *d_Y, void *stream) {
    Mlp *mp = static_cast<Mlp *>(mlp);
    if (!mp || !d_X || !d_Y || rows < 0) return fail(CUMF_ERR_ARG, "mlp_forward: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t chunk = 1 << 16;
    for (int64_t r0 = 0; r0 < rows; r0 += chunk) {
        const int64_t r = std::min(chunk, rows - r0);
        if (int rc = mlp_forward_ws(mp, d_X + r0 * mp->d_in, r, s)) return rc;
        CUMF_CUDA(cudaMemcpyAsync(d_Y + r0 * mp->d_out, mp->y.p, r * mp->d_out * 4, cudaMemcpyDeviceToDevice, s));
    }
    return mlp_check_status(mp, s);
}

int cumf_mlp_loss_grad(void *mlp, const float *d_X, const float *d_T, int64_t rows, double *loss, void *stream) {
    Mlp *mp = static_cast<Mlp *>(mlp);
    if (!mp || !d_X || !d_T || rows <= 0) return fail(CUMF_ERR_ARG, "mlp_loss_grad: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    if (int rc = mlp_forward_ws(mp, d_X, rows, s)) return rc;
    if (int rc = mlp_backward_ws(mp, d_T, rows, s)) return rc;
    double l = 0;
    CUMF_CUDA(cudaMemcpyAsync(&l, mp->loss.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    if (int rc = mlp_check_status(mp, s)) return rc;
    if (loss) *loss = l / (double)rows;
    return CUMF_OK;
}

int cumf_mlp_train(void *mlp, const float *d_X, const float *d_T, int64_t rows, int epochs, int batch, float lr,
                   uint64_t seed, double *final_loss, void *stream) {
    Mlp *mp = static_cast<Mlp *>(mlp);
    if (!mp || !d_X || !d_T || rows <= 0 || epochs < 0 || batch <= 0)
        return fail(CUMF_ERR_ARG, "mlp_train: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    DevBuf xs, ts, perm_d;
    CUMF_CUDA(xs.alloc((size_t)batch * mp->d_in * 4));
    CUMF_CUDA(ts.alloc((size_t)batch * mp->d_out * 4));
    CUMF_CUDA(perm_d.alloc((size_t)rows * 4));
    std::vector<int32_t> perm(rows);
    GlibcRand rng((uint32_t)seed);
    double last = 0;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int e = 0; e < epochs; ++e) {
        for (int64_t i = 0; i < rows; ++i) perm[i] = (int32_t)i;
        glibc_random_shuffle(perm.data(), rows, rng);
        CUMF_CUDA(cudaMemcpyAsync(perm_d.p, perm.data(), rows * 4, cudaMemcpyHostToDevice, s));
        double sum = 0;
        int64_t seen = 0;
        for (int64_t r0 = 0; r0 < rows; r0 += batch) {
            const int64_t r = std::min<int64_t>(batch, rows - r0);
            gather_rows_kernel<<<grid_of(r * mp->d_in), kT, 0, s>>>(d_X, mp->d_in, perm_d.as<int32_t>() + r0, r,
                                                                     xs.as<float>());
            gather_rows_kernel<<<grid_of(r * mp->d_out), kT, 0, s>>>(d_T, mp->d_out, perm_d.as<int32_t>() + r0, r,
                                                                      ts.as<float>());
            if (int rc = mlp_forward_ws(mp, xs.as<float>(), r, s)) return rc;
            if (int rc = mlp_backward_ws(mp, ts.as<float>(), r, s)) return rc;
            ++mp->step;
            const float c1 = 1.f - powf(b1, (float)mp->step), c2 = 1.f - powf(b2, (float)mp->step);
            adam_kernel<<<grid_of(mp->count), kT, 0, s>>>(mp->params.as<float>(), mp->grads.as<float>(),
                                                          mp->m1.as<float>(), mp->m2.as<float>(), mp->count, lr, b1,
                                                          b2, eps, c1, c2);
            CUMF_CUDA(cudaGetLastError());
            if (int rc = mlp_refresh(mp, s)) return rc;
            if (e == epochs - 1) {
                double l = 0;
                CUMF_CUDA(cudaMemcpyAsync(&l, mp->loss.p, sizeof(double), cudaMemcpyDeviceToHost, s));
                CUMF_CUDA(cudaStreamSynchronize(s));
                sum += l;
                seen += r;
            }
        }
        if (e == epochs - 1 && seen) last = sum / (double)seen;
    }
    if (int rc = mlp_check_status(mp, s)) return rc;
    if (final_loss) *final_loss = last;
    return CUMF_OK;
}

int cumf_user_features(const cumf_node *d_R, int64_t nnz, const float *d_Q, int32_t n, int k, int32_t m,
                       float *d_X, void *stream) {
    if (!d_Q || !d_X || m <= 0 || n <= 0 || k <= 0 || nnz < 0 || (nnz > 0 && !d_R))
        return fail(CUMF_ERR_ARG, "user_features: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    DevBuf deg, sum, sum2;
    CUMF_CUDA(deg.alloc((size_t)m * 4));
    CUMF_CUDA(sum.alloc((size_t)m * 4));
    CUMF_CUDA(sum2.alloc((size_t)m * 4));
    CUMF_CUDA(cudaMemsetAsync(deg.p, 0, (size_t)m * 4, s));
    CUMF_CUDA(cudaMemsetAsync(sum.p, 0, (size_t)m * 4, s));
    CUMF_CUDA(cudaMemsetAsync(sum2.p, 0, (size_t)m * 4, s));
    // The centred mean accumulates in a k-wide buffer (16-byte aligned rows for the vector
    // atomics), then lands in the (k+3)-wide feature rows beside the scalar features.
    const int ldx = k + 3;
    DevBuf acc;
    CUMF_CUDA(acc.alloc((size_t)m * k * 4));
    CUMF_CUDA(cudaMemsetAsync(acc.p, 0, (size_t)m * k * 4, s));
    if (nnz > 0) {
        user_stats_kernel<<<grid_of(nnz), kT, 0, s>>>(d_R, nnz, m, n, deg.as<float>(), sum.as<float>(),
                                                       sum2.as<float>());
        user_qsum_kernel<<<grid_of(nnz * 32), kT, 0, s>>>(d_R, nnz, m, n, d_Q, k, deg.as<float>(), sum.as<float>(),
                                                           acc.as<float>(), k);
    }
    CUMF_CUDA(cudaMemcpy2DAsync(d_X, (size_t)ldx * 4, acc.p, (size_t)k * 4, (size_t)k * 4, m,
                                cudaMemcpyDeviceToDevice, s));
    user_scalar_kernel<<<grid_of(m), kT, 0, s>>>(m, k, deg.as<float>(), sum.as<float>(), sum2.as<float>(), d_X, ldx);
    CUMF_CUDA(cudaGetLastError());
    CUMF_CUDA(cudaStreamSynchronize(s));
    return CUMF_OK;
}

}  // extern "C"
