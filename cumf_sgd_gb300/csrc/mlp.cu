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
#include <cub/cub.cuh>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <mutex>
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

// Stream-ordered scratch of the feature extraction from a pool of this library that keeps up
// to 256 MB between calls (the default pool returns its memory at every synchronisation, and
// mapping it again cost more than the feature kernels at 50,000 users).
cudaError_t feature_scratch(void **p, size_t bytes, cudaStream_t s) {
    static std::mutex mu;
    static cudaMemPool_t pools[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaMallocAsync(p, bytes, s);
    cudaMemPool_t pool;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!pools[dev]) {
            cudaMemPoolProps props;
            memset(&props, 0, sizeof(props));
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            if ((e = cudaMemPoolCreate(&pools[dev], &props)) != cudaSuccess) return e;
            uint64_t keep = 256ull << 20;
            if ((e = cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess)
                return e;
        }
        pool = pools[dev];
    }
    return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

// Sort keys of the ratings: the user, or m for a rating outside [0, m) x [0, n) (sorted last
// and left out); values: the rating's index.
__global__ void user_keys_kernel(const cumf_node *R, uint32_t nnz, int32_t m, int32_t n, uint32_t *key,
                                 uint32_t *idx) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += gridDim.x * blockDim.x) {
        const cumf_node x = R[i];
        const bool ok = (uint32_t)x.u < (uint32_t)m && (uint32_t)x.v < (uint32_t)n;
        key[i] = ok ? (uint32_t)x.u : (uint32_t)m;
        idx[i] = i;
    }
}

// seg[u] = the first sorted position whose key is >= u, u = 0..m (binary search).
__global__ void user_segments_kernel(const uint32_t *key, uint32_t nnz, int32_t m, int64_t *seg) {
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u <= m; u += (int64_t)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = nnz;
        while (lo < hi) {
            const uint32_t mid = lo + (hi - lo) / 2;
            if (key[mid] < (uint32_t)u) lo = mid + 1;
            else hi = mid;
        }
        seg[u] = lo;
    }
}

// One warp per user over the user's ratings in their original order (a stable sort by user):
// the rating sum and sum of squares by a fixed-order warp reduction, then
// sum (r - mean) q / deg accumulated rating by rating in registers, 32 * KPL columns per
// pass; X[u] = (that sum, log(1 + deg)/4, (mean - 3)/2, var/2).  The ratings are fetched 32
// at a time (one per lane, then broadcast) and the item rows of four ratings are loaded
// before they are added, in rating order.  No atomics: the features are the same bits on
// every run.
template <int KPL>
__global__ void user_rows_kernel(const cumf_node *R, const uint32_t *order, const int64_t *seg, int32_t m,
                                 const float *Q, int k, float *X, int ldx) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = w0; u < m; u += nw) {
        const int64_t a = seg[u], b = seg[u + 1];
        float s = 0.f, s2 = 0.f;
        for (int64_t t = a + lane; t < b; t += 32) {
            const float r = R[order[t]].r;
            s += r;
            s2 += r * r;
        }
        for (int o = 16; o >= 1; o >>= 1) {
            s += __shfl_xor_sync(0xffffffffu, s, o);
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        }
        const float d = (float)(b - a);
        const float mean = d > 0 ? s / d : 0.f;
        float *xu = X + u * ldx;
        for (int c0 = 0; c0 < k; c0 += 32 * KPL) {
            float acc[KPL];
#pragma unroll
            for (int j = 0; j < KPL; ++j) acc[j] = 0.f;
            bool col[KPL];
#pragma unroll
            for (int j = 0; j < KPL; ++j) col[j] = c0 + lane + 32 * j < k;
            for (int64_t t0 = a; t0 < b; t0 += 32) {
                float cl = 0.f;
                int vl = 0;
                if (t0 + lane < b) {
                    const cumf_node x = R[order[t0 + lane]];
                    cl = (x.r - s / d) / d;
                    vl = x.v;
                }
                const int cnt = (int)(b - t0 < 32 ? b - t0 : 32);
                for (int j0 = 0; j0 < cnt; j0 += 4) {
                    float c4[4], q4[4][KPL];
#pragma unroll
                    for (int h = 0; h < 4; ++h) {
                        c4[h] = __shfl_sync(0xffffffffu, cl, (j0 + h) & 31);
                        const int v = __shfl_sync(0xffffffffu, vl, (j0 + h) & 31);
                        const float *q = Q + (int64_t)v * k + c0 + lane;
#pragma unroll
                        for (int j = 0; j < KPL; ++j) q4[h][j] = (j0 + h < cnt && col[j]) ? q[32 * j] : 0.f;
                    }
#pragma unroll
                    for (int h = 0; h < 4; ++h)
                        if (j0 + h < cnt) {
#pragma unroll
                            for (int j = 0; j < KPL; ++j) acc[j] += c4[h] * q4[h][j];
                        }
                }
            }
#pragma unroll
            for (int j = 0; j < KPL; ++j)
                if (col[j]) xu[c0 + lane + 32 * j] = acc[j];
        }
        if (lane == 0) {
            xu[k] = logf(1.f + d) * 0.25f;
            xu[k + 1] = d > 0 ? (mean - 3.f) * 0.5f : 0.f;
            xu[k + 2] = (d > 0 ? fmaxf(s2 / d - mean * mean, 0.f) : 0.f) * 0.5f;
        }
    }
}

// x[u] = (acc[u][0:k], log(1 + deg)/4, (mean - 3)/2, var/2) for the m users (ldx = k + 3).
__global__ void user_finish_kernel(int32_t m, int k, const float *acc, const float *deg, const float *sum,
                                   const float *sum2, float *X, int ldx) {
    const int64_t total = (int64_t)m * ldx;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t u = i / ldx;
        const int c = (int)(i - u * ldx);
        if (c < k) {
            X[i] = acc[u * k + c];
            continue;
        }
        const float d = deg[u];
        const float mean = d > 0 ? sum[u] / d : 0.f;
        if (c == k)
            X[i] = logf(1.f + d) * 0.25f;
        else if (c == k + 1)
            X[i] = d > 0 ? (mean - 3.f) * 0.5f : 0.f;
        else
            X[i] = (d > 0 ? fmaxf(sum2[u] / d - mean * mean, 0.f) : 0.f) * 0.5f;
    }
}

// ---- elementwise helpers ---------------------------------------------------------------

// ---- 32 x 32 tile kernels: an elementwise result written row-major and transposed --------
//
// The weight-gradient products dW = dZ^T A take both operands K-major (K = the batch rows), so
// every bf16 activation or gradient that feeds one is also needed transposed.  The kernels
// below produce both copies from one read of their inputs: a block computes a 32 x 32 tile,
// writes it row-major, stages it in shared memory (fp32, conflict-free) and writes the
// transpose; gradient tiles also leave their 32-row column sums for the bias gradient.
constexpr int kTile = 32;
constexpr int kTileRows = 8;  // threads per column of a tile (blockDim = 32 x 8)

// Dt[c][r] = tile[r - r0][c - c0] for the tile's valid rows r < nr and columns c < nc.
__device__ __forceinline__ void store_tile_t(const float (*tile)[kTile + 1], __nv_bfloat16 *Dt, int64_t ldt, int r0,
                                             int c0, int nr, int nc) {
    for (int j = threadIdx.y; j < kTile; j += kTileRows) {
        const int c = c0 + j, r = r0 + threadIdx.x;
        if (c < nc && r < nr) Dt[(int64_t)c * ldt + r] = __float2bfloat16_rn(tile[threadIdx.x][j]);
    }
}

// partial[tile row][c] = the tile's column c summed over its 32 rows: each thread's own rows
// (y, y + 8, y + 16, y + 24, in order, in `mine`), then the 8 thread sums in order.  Call after
// a barrier that follows the writes of lanes[][] (lanes[threadIdx.y][threadIdx.x] = mine).
__device__ __forceinline__ void tile_colsum(const float (*lanes)[kTile + 1], float *partial, int cols, int c0) {
    if (threadIdx.y == 0 && c0 + (int)threadIdx.x < cols) {
        float sum = 0.f;
        for (int y = 0; y < kTileRows; ++y) sum += lanes[y][threadIdx.x];
        partial[(int64_t)blockIdx.x * cols + c0 + threadIdx.x] = sum;
    }
}

// D (rp x ldd bf16) and, when Dt != NULL, Dt (ldd x rp) from the fp32 rows of S (cols wide):
// row r < valid is S[perm[*batch_idx * batch + r]] (perm NULL: S[r]); other rows and the
// columns cols..ldd are zero.
struct ConvertJob {
    const float *S;
    int cols;
    const int32_t *perm;
    const int *batch_idx;
    int64_t batch;
    int valid, rp, ldd;
    __nv_bfloat16 *D, *Dt;
};
struct ConvertJobs {
    ConvertJob job[3];  // blockIdx.z picks one; tiles outside its rp x ldd return
};

__global__ void __launch_bounds__(kTile * kTileRows) convert_t_kernel(const __grid_constant__ ConvertJobs jobs) {
    const ConvertJob &jb = jobs.job[blockIdx.z];
    const float *S = jb.S;
    const int cols = jb.cols, valid = jb.valid, rp = jb.rp, ldd = jb.ldd;
    __nv_bfloat16 *D = jb.D, *Dt = jb.Dt;
    __shared__ float tile[kTile][kTile + 1];
    const int r0 = blockIdx.x * kTile, c0 = blockIdx.y * kTile;
    if (r0 >= rp || c0 >= ldd) return;
    const int32_t *idx = jb.perm ? jb.perm + (int64_t)*jb.batch_idx * jb.batch : nullptr;
    for (int j = threadIdx.y; j < kTile; j += kTileRows) {
        const int r = r0 + j, c = c0 + threadIdx.x;
        float v = 0.f;
        if (r < valid && c < cols) v = S[(int64_t)(idx ? idx[r] : r) * cols + c];
        const __nv_bfloat16 b = __float2bfloat16_rn(v);
        if (r < rp && c < ldd) D[(int64_t)r * ldd + c] = b;
        tile[j][threadIdx.x] = __bfloat162float(b);
    }
    if (!Dt) return;
    __syncthreads();
    store_tile_t(tile, Dt, rp, r0, c0, rp, ldd);
}

// D^T (cols x rows) of a bf16 matrix D (rows x cols).
__global__ void __launch_bounds__(kTile * kTileRows) transpose_t_kernel(const __nv_bfloat16 *D, int rows, int cols,
                                                                        __nv_bfloat16 *Dt) {
    __shared__ float tile[kTile][kTile + 1];
    const int r0 = blockIdx.x * kTile, c0 = blockIdx.y * kTile;
    for (int j = threadIdx.y; j < kTile; j += kTileRows) {
        const int r = r0 + j, c = c0 + threadIdx.x;
        tile[j][threadIdx.x] = (r < rows && c < cols) ? __bfloat162float(D[(int64_t)r * cols + c]) : 0.f;
    }
    __syncthreads();
    store_tile_t(tile, Dt, rows, r0, c0, rows, cols);
}

__device__ __forceinline__ float gelu_grad(float x) {
    const float c = 0.7978845608028654f;
    const float u = c * (x + 0.044715f * x * x * x);
    const float t = tanhf(u);
    return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * c * (1.f + 3.f * 0.044715f * x * x);
}

// dZ = dA * gelu'(pre) -> bf16 (rows beyond `valid` zero), its transpose dZt, and the tile
// column sums of dZ (the bias gradient's partial sums).
__global__ void __launch_bounds__(kTile * kTileRows) gelu_back_t_kernel(const float *dA, const float *pre, int rp,
                                                                        int valid, int cols, __nv_bfloat16 *dZ,
                                                                        __nv_bfloat16 *dZt, float *partial) {
    __shared__ float tile[kTile][kTile + 1];
    __shared__ float lanes[kTileRows][kTile + 1];
    const int r0 = blockIdx.x * kTile, c0 = blockIdx.y * kTile;
    float mine = 0.f;
    for (int j = threadIdx.y; j < kTile; j += kTileRows) {
        const int r = r0 + j, c = c0 + threadIdx.x;
        const int64_t i = (int64_t)r * cols + c;
        const float g = (r < valid && c < cols) ? dA[i] * gelu_grad(pre[i]) : 0.f;
        const __nv_bfloat16 b = __float2bfloat16_rn(g);
        if (r < rp && c < cols) dZ[i] = b;
        const float bv = __bfloat162float(b);
        tile[j][threadIdx.x] = bv;
        mine += bv;
    }
    lanes[threadIdx.y][threadIdx.x] = mine;
    __syncthreads();
    tile_colsum(lanes, partial, cols, c0);
    store_tile_t(tile, dZt, rp, r0, c0, rp, cols);
}

// dY = 2 (Y - T) / B (bf16, zero for padding rows), its transpose, the tile column sums and
// the loss (sum of squared errors).  Row r < valid of T is T[perm[*batch_idx * batch + r]]
// (perm NULL: T[r]).
__global__ void __launch_bounds__(kTile * kTileRows) mse_grad_t_kernel(const float *Y, const float *T,
                                                                       const int32_t *perm, const int *batch_idx,
                                                                       int64_t batch, int rp, int valid, int cols,
                                                                       float inv_b, __nv_bfloat16 *dY,
                                                                       __nv_bfloat16 *dYt, float *partial,
                                                                       double *loss) {
    __shared__ float tile[kTile][kTile + 1];
    __shared__ float lanes[kTileRows][kTile + 1];
    __shared__ double s_loss[kTileRows];
    const int r0 = blockIdx.x * kTile, c0 = blockIdx.y * kTile;
    const int32_t *idx = perm ? perm + (int64_t)*batch_idx * batch : nullptr;
    double acc = 0;
    float mine = 0.f;
    for (int j = threadIdx.y; j < kTile; j += kTileRows) {
        const int r = r0 + j, c = c0 + threadIdx.x;
        float g = 0.f;
        if (r < valid && c < cols) {
            const float d = Y[(int64_t)r * cols + c] - T[(int64_t)(idx ? idx[r] : r) * cols + c];
            acc += (double)d * d;
            g = 2.f * d * inv_b;
        }
        const __nv_bfloat16 b = __float2bfloat16_rn(g);
        if (r < rp && c < cols) dY[(int64_t)r * cols + c] = b;
        const float bv = __bfloat162float(b);
        tile[j][threadIdx.x] = bv;
        mine += bv;
    }
    lanes[threadIdx.y][threadIdx.x] = mine;
    for (int o = 16; o >= 1; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) s_loss[threadIdx.y] = acc;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0 && loss) {
        double t = 0;
        for (int w = 0; w < kTileRows; ++w) t += s_loss[w];
        atomicAdd(loss, t);
    }
    tile_colsum(lanes, partial, cols, c0);
    store_tile_t(tile, dYt, rp, r0, c0, rp, cols);
}

// Bias gradient: out[c] = the tile column sums of column c (tile_colsum).  Block: 32 columns x
// 8 lanes; lane y adds tiles y, y + 8, ... in order, then the 8 lane sums are added in order.
__global__ void __launch_bounds__(kTile * kTileRows) colsum_finish_kernel(const float *partial, int tiles, int cols,
                                                                          float *out) {
    __shared__ float lanes[kTileRows][kTile + 1];
    const int c = blockIdx.x * kTile + threadIdx.x;
    float sum = 0.f;
    if (c < cols)
        for (int t = threadIdx.y; t < tiles; t += kTileRows) sum += partial[(int64_t)t * cols + c];
    lanes[threadIdx.y][threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.y == 0 && c < cols) {
        float total = 0.f;
        for (int y = 0; y < kTileRows; ++y) total += lanes[y][threadIdx.x];
        out[c] = total;
    }
}

// After a step: the next batch of the permutation, Adam's step count, the step's loss added to
// the epoch's.  One thread; this state lives on the device so that a captured step can replay.
__global__ void step_end_kernel(int64_t *step, int *batch_idx, const double *loss, double *loss_sum) {
    ++*step;
    ++*batch_idx;
    *loss_sum += *loss;
}

// Adam step number *step + 1 (bias corrections 1 - b^t computed once per block).
__global__ void adam_kernel(float *w, const float *g, float *m1, float *m2, int64_t n, float lr, float b1, float b2,
                            float eps, const int64_t *step) {
    __shared__ float corr[2];
    if (threadIdx.x == 0) {
        const float t = (float)(*step + 1);
        corr[0] = 1.f - powf(b1, t);
        corr[1] = 1.f - powf(b2, t);
    }
    __syncthreads();
    const float c1 = corr[0], c2 = corr[1];
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
    // workspace for batches of up to cap_fwd rows (forward) / cap rows (backward)
    int64_t cap = 0;      // rows of the backward buffers
    int64_t cap_fwd = 0;  // rows of the forward buffers
    DevBuf xb, h1, h2, pre1, pre2, y, dy, dyt, h2t, h1t, xbt, dh2, dp2, dp2t, dh1, dp1, dp1t, loss;
    DevBuf gw1p;  // gradient of W1 in padded layout [h][dp]
    DevBuf colws; // (cap / 32) x max(h, d_out) tile column sums
};

namespace {

// Workspace for batches of up to `rows` rows: the forward buffers, and with `train` also
// those of the backward pass (the activations' transposes, pre-activations, gradients).
int mlp_ensure(Mlp *mp, int64_t rows, bool train) {
    const int64_t r = (rows + 127) / 128 * 128;
    const size_t b2 = 2;
    const int h = mp->h, dp = mp->dp, dout = mp->d_out;
    if (rows > mp->cap_fwd) {
        CUMF_CUDA(mp->xb.alloc(r * dp * b2));
        CUMF_CUDA(mp->h1.alloc(r * h * b2));
        CUMF_CUDA(mp->h2.alloc(r * h * b2));
        CUMF_CUDA(mp->y.alloc(r * dout * 4));
        mp->cap_fwd = r;
    }
    if (!train || rows <= mp->cap) return CUMF_OK;
    CUMF_CUDA(mp->pre1.alloc(r * h * 4));
    CUMF_CUDA(mp->pre2.alloc(r * h * 4));
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
    CUMF_CUDA(mp->colws.alloc((r / kTile) * (h > dout ? h : dout) * 4));
    mp->cap = r;
    return CUMF_OK;
}

const dim3 kTileBlock(kTile, kTileRows);

dim3 tiles_of(int64_t rows, int cols) { return dim3((unsigned)((rows + kTile - 1) / kTile), (unsigned)((cols + kTile - 1) / kTile)); }

ConvertJob convert_job(const float *S, int cols, const int32_t *perm, const int *batch_idx, int64_t batch, int valid,
                       int rp, int ldd, void *D, void *Dt) {
    return ConvertJob{S, cols, perm, batch_idx, batch, valid, rp, ldd, static_cast<__nv_bfloat16 *>(D),
                      static_cast<__nv_bfloat16 *>(Dt)};
}

// n (1..3) conversions in one launch.
cudaError_t convert(const ConvertJob *job, int n, cudaStream_t s) {
    ConvertJobs jobs{};
    unsigned gx = 1, gy = 1;
    for (int i = 0; i < n; ++i) {
        jobs.job[i] = job[i];
        const dim3 g = tiles_of(job[i].rp, job[i].ldd);
        gx = g.x > gx ? g.x : gx;
        gy = g.y > gy ? g.y : gy;
    }
    convert_t_kernel<<<dim3(gx, gy, n), kTileBlock, 0, s>>>(jobs);
    return cudaGetLastError();
}

cudaError_t transpose(const void *D, int rows, int cols, void *Dt, cudaStream_t s) {
    transpose_t_kernel<<<tiles_of(rows, cols), kTileBlock, 0, s>>>(static_cast<const __nv_bfloat16 *>(D), rows, cols,
                                                                   static_cast<__nv_bfloat16 *>(Dt));
    return cudaGetLastError();
}

cudaError_t colsum_finish(Mlp *mp, int64_t rp, int cols, float *out, cudaStream_t s) {
    colsum_finish_kernel<<<(cols + kTile - 1) / kTile, kTileBlock, 0, s>>>(mp->colws.as<float>(), (int)(rp / kTile),
                                                                            cols, out);
    return cudaGetLastError();
}

// bf16 operand copies of the fp32 master weights.
int mlp_refresh(Mlp *mp, cudaStream_t s) {
    const float *P = mp->params.as<float>();
    const int h = mp->h, dout = mp->d_out;
    const ConvertJob jobs[3] = {
        convert_job(P + mp->off_w1, mp->d_in, nullptr, nullptr, 0, h, h, mp->dp, mp->w1b.p, nullptr),
        convert_job(P + mp->off_w2, h, nullptr, nullptr, 0, h, h, h, mp->w2b.p, mp->w2t.p),
        convert_job(P + mp->off_w3, h, nullptr, nullptr, 0, dout, dout, h, mp->w3b.p, mp->w3t.p)};
    CUMF_CUDA(convert(jobs, 3, s));
    return CUMF_OK;
}

// Forward over rows [0, rows) of X (fp32, rows x d_in; with perm, row r is X[perm[*batch_idx *
// batch + r]]); Y (fp32 rows x d_out) in mp->y.  train: also X's bf16 transpose and the
// pre-activations, which the backward pass uses.
int mlp_forward_ws(Mlp *mp, const float *X, int64_t rows, cudaStream_t s, bool train, const int32_t *perm = nullptr,
                   const int *batch_idx = nullptr, int64_t batch = 0) {
    if (int rc = mlp_ensure(mp, rows, train)) return rc;
    const float *P = mp->params.as<float>();
    const int h = mp->h;
    const int64_t rp = (rows + 127) / 128 * 128;  // padding rows are zero
    const ConvertJob job = convert_job(X, mp->d_in, perm, batch_idx, batch, (int)rows, (int)rp, mp->dp, mp->xb.p,
                                       train ? mp->xbt.p : nullptr);
    CUMF_CUDA(convert(&job, 1, s));
    int *st = mp->status.as<int>();
    CUMF_CUDA(launch_tc_gemm(mp->xb.p, mp->w1b.p, (int)rp, h, mp->dp, P + mp->off_b1, 1, mp->h1.p, 0, h,
                             train ? mp->pre1.as<float>() : nullptr, st, s));
    CUMF_CUDA(launch_tc_gemm(mp->h1.p, mp->w2b.p, (int)rp, h, h, P + mp->off_b2, 1, mp->h2.p, 0, h,
                             train ? mp->pre2.as<float>() : nullptr, st, s));
    CUMF_CUDA(launch_tc_gemm(mp->h2.p, mp->w3b.p, (int)rp, mp->d_out, h, P + mp->off_b3, 0, mp->y.p, 1, mp->d_out,
                             nullptr, st, s));
    return CUMF_OK;
}

// Loss and gradients (into mp->grads) for rows [0, rows) with targets T (fp32 rows x d_out,
// through perm as in mlp_forward_ws), after mlp_forward_ws on the same rows.
int mlp_backward_ws(Mlp *mp, const float *T, int64_t rows, cudaStream_t s, const int32_t *perm = nullptr,
                    const int *batch_idx = nullptr, int64_t batch = 0) {
    const int h = mp->h, dout = mp->d_out, dp = mp->dp;
    const int64_t rp = (rows + 127) / 128 * 128;
    float *G = mp->grads.as<float>();
    float *part = mp->colws.as<float>();
    int *st = mp->status.as<int>();
    CUMF_CUDA(cudaMemsetAsync(mp->loss.p, 0, sizeof(double), s));
    // layer 3: dY (and dY^T, db3), dW3 = dY^T H2, dH2 = dY W3
    mse_grad_t_kernel<<<tiles_of(rp, dout), kTileBlock, 0, s>>>(
        mp->y.as<float>(), T, perm, batch_idx, batch, (int)rp, (int)rows, dout, 1.f / (float)rows,
        mp->dy.as<__nv_bfloat16>(), mp->dyt.as<__nv_bfloat16>(), part, mp->loss.as<double>());
    CUMF_CUDA(cudaGetLastError());
    CUMF_CUDA(colsum_finish(mp, rp, dout, G + mp->off_b3, s));
    CUMF_CUDA(transpose(mp->h2.p, (int)rp, h, mp->h2t.p, s));
    CUMF_CUDA(launch_tc_gemm(mp->dyt.p, mp->h2t.p, dout, h, (int)rp, nullptr, 0, G + mp->off_w3, 1, h, nullptr, st, s));
    CUMF_CUDA(launch_tc_gemm(mp->dy.p, mp->w3t.p, (int)rp, h, dout, nullptr, 0, mp->dh2.p, 1, h, nullptr, st, s));
    // layer 2
    gelu_back_t_kernel<<<tiles_of(rp, h), kTileBlock, 0, s>>>(mp->dh2.as<float>(), mp->pre2.as<float>(), (int)rp,
                                                              (int)rows, h, mp->dp2.as<__nv_bfloat16>(),
                                                              mp->dp2t.as<__nv_bfloat16>(), part);
    CUMF_CUDA(cudaGetLastError());
    CUMF_CUDA(colsum_finish(mp, rp, h, G + mp->off_b2, s));
    CUMF_CUDA(transpose(mp->h1.p, (int)rp, h, mp->h1t.p, s));
    CUMF_CUDA(launch_tc_gemm(mp->dp2t.p, mp->h1t.p, h, h, (int)rp, nullptr, 0, G + mp->off_w2, 1, h, nullptr, st, s));
    CUMF_CUDA(launch_tc_gemm(mp->dp2.p, mp->w2t.p, (int)rp, h, h, nullptr, 0, mp->dh1.p, 1, h, nullptr, st, s));
    // layer 1 (padded input columns give zero gradient columns, dropped on copy)
    gelu_back_t_kernel<<<tiles_of(rp, h), kTileBlock, 0, s>>>(mp->dh1.as<float>(), mp->pre1.as<float>(), (int)rp,
                                                              (int)rows, h, mp->dp1.as<__nv_bfloat16>(),
                                                              mp->dp1t.as<__nv_bfloat16>(), part);
    CUMF_CUDA(cudaGetLastError());
    CUMF_CUDA(colsum_finish(mp, rp, h, G + mp->off_b1, s));
    CUMF_CUDA(launch_tc_gemm(mp->dp1t.p, mp->xbt.p, h, dp, (int)rp, nullptr, 0, mp->gw1p.p, 1, dp, nullptr, st, s));
    CUMF_CUDA(cudaMemcpy2DAsync(G + mp->off_w1, mp->d_in * sizeof(float), mp->gw1p.p, dp * sizeof(float),
                                mp->d_in * sizeof(float), h, cudaMemcpyDeviceToDevice, s));
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
    TraceRange trace("warm start: MLP inference");
    Mlp *mp = static_cast<Mlp *>(mlp);
    if (!mp || !d_X || !d_Y || rows < 0) return fail(CUMF_ERR_ARG, "mlp_forward: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t chunk = 1 << 16;
    for (int64_t r0 = 0; r0 < rows; r0 += chunk) {
        const int64_t r = std::min(chunk, rows - r0);
        if (int rc = mlp_forward_ws(mp, d_X + r0 * mp->d_in, r, s, false)) return rc;
        CUMF_CUDA(cudaMemcpyAsync(d_Y + r0 * mp->d_out, mp->y.p, r * mp->d_out * 4, cudaMemcpyDeviceToDevice, s));
    }
    return mlp_check_status(mp, s);
}

int cumf_mlp_loss_grad(void *mlp, const float *d_X, const float *d_T, int64_t rows, double *loss, void *stream) {
    Mlp *mp = static_cast<Mlp *>(mlp);
    if (!mp || !d_X || !d_T || rows <= 0) return fail(CUMF_ERR_ARG, "mlp_loss_grad: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    if (int rc = mlp_forward_ws(mp, d_X, rows, s, true)) return rc;
    if (int rc = mlp_backward_ws(mp, d_T, rows, s)) return rc;
    double l = 0;
    CUMF_CUDA(cudaMemcpyAsync(&l, mp->loss.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    if (int rc = mlp_check_status(mp, s)) return rc;
    if (loss) *loss = l / (double)rows;
    return CUMF_OK;
}

int cumf_mlp_train(void *mlp, const float *d_X, const float *d_T, int64_t rows, int epochs, int batch, float lr,
                   uint64_t seed, double *final_loss, void *stream) {
    TraceRange trace("warm start: MLP training");
    Mlp *mp = static_cast<Mlp *>(mlp);
    if (!mp || !d_X || !d_T || rows <= 0 || epochs < 0 || batch <= 0)
        return fail(CUMF_ERR_ARG, "mlp_train: bad arguments");
    if (rows > 0x7fffffffll) return fail(CUMF_ERR_ARG, "mlp_train: more than 2^31 - 1 rows");
    if (final_loss) *final_loss = 0;
    if (epochs == 0) return CUMF_OK;
    if (batch > rows) batch = (int)rows;
    const int64_t full = rows / batch, tail = rows % batch;
    if (int rc = mlp_ensure(mp, batch, true)) return rc;  // the workspace, before any capture

    // Device state of the replayed step: Adam's step count and corrections, the batch index
    // into the epoch's permutation, the epoch's loss.
    struct State {
        int64_t step;
        int batch_idx;
        int pad;
        double loss_sum;
    };
    DevBuf perm_d, state;
    CUMF_CUDA(perm_d.alloc((size_t)rows * 4));
    CUMF_CUDA(state.alloc(sizeof(State)));
    State *st = state.as<State>();
    struct Host {
        void *p[2] = {nullptr, nullptr};
        ~Host() {
            for (void *x : p)
                if (x) cudaFreeHost(x);
        }
    } perm_h;
    for (int k = 0; k < 2; ++k) CUMF_CUDA(cudaMallocHost(&perm_h.p[k], (size_t)rows * 4));
    // A private stream (capture is not possible on the legacy default stream), ordered after
    // the caller's stream and before its later work.
    struct Res {
        cudaStream_t ws = nullptr;
        cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
        cudaGraphExec_t exec[2] = {nullptr, nullptr};
        ~Res() {
            for (cudaGraphExec_t x : exec)
                if (x) cudaGraphExecDestroy(x);
            for (cudaEvent_t x : ev)
                if (x) cudaEventDestroy(x);
            if (ws) cudaStreamDestroy(ws);
        }
    } res;
    CUMF_CUDA(cudaStreamCreateWithFlags(&res.ws, cudaStreamNonBlocking));
    for (cudaEvent_t &x : res.ev) CUMF_CUDA(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
    cudaStream_t user = (cudaStream_t)stream, ws = res.ws;
    CUMF_CUDA(cudaEventRecord(res.ev[0], user));
    CUMF_CUDA(cudaStreamWaitEvent(ws, res.ev[0], 0));
    const State init = {mp->step, 0, 0, 0.0};
    CUMF_CUDA(cudaMemcpyAsync(st, &init, sizeof(State), cudaMemcpyHostToDevice, ws));
    CUMF_CUDA(cudaStreamSynchronize(ws));  // `init` is a host local

    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    // One training step of r rows at the batch the device index names.
    auto enqueue_step = [&](int64_t r) -> int {
        const int32_t *perm = perm_d.as<int32_t>();
        if (int rc = mlp_forward_ws(mp, d_X, r, ws, true, perm, &st->batch_idx, batch)) return rc;
        if (int rc = mlp_backward_ws(mp, d_T, r, ws, perm, &st->batch_idx, batch)) return rc;
        adam_kernel<<<grid_of(mp->count), kT, 0, ws>>>(mp->params.as<float>(), mp->grads.as<float>(),
                                                       mp->m1.as<float>(), mp->m2.as<float>(), mp->count, lr, b1, b2,
                                                       eps, &st->step);
        if (int rc = mlp_refresh(mp, ws)) return rc;
        step_end_kernel<<<1, 1, 0, ws>>>(&st->step, &st->batch_idx, mp->loss.as<double>(), &st->loss_sum);
        CUMF_CUDA(cudaGetLastError());
        return CUMF_OK;
    };
    // Capture the full-batch step and the last, shorter one; replay them every epoch.
    auto capture = [&](int64_t r, cudaGraphExec_t *exec) -> int {
        CUMF_CUDA(cudaStreamBeginCapture(ws, cudaStreamCaptureModeRelaxed));
        const int rc = enqueue_step(r);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(ws, &g);
        if (rc != CUMF_OK || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            return rc != CUMF_OK ? rc : cuda_fail(e, "mlp_train: capture");
        }
        const cudaError_t ei = cudaGraphInstantiate(exec, g, 0);
        cudaGraphDestroy(g);
        CUMF_CUDA(ei);
        return CUMF_OK;
    };
    if (full > 0)
        if (int rc = capture(batch, &res.exec[0])) return rc;
    if (tail > 0)
        if (int rc = capture(tail, &res.exec[1])) return rc;

    // Permutations from one glibc rand() stream, epoch by epoch; the next epoch's is drawn on
    // the host while the device runs the current one (two pinned buffers).
    GlibcRand rng((uint32_t)seed);
    auto draw = [&](int32_t *perm) {
        for (int64_t i = 0; i < rows; ++i) perm[i] = (int32_t)i;
        glibc_random_shuffle(perm, rows, rng);
    };
    draw(static_cast<int32_t *>(perm_h.p[0]));
    for (int e = 0; e < epochs; ++e) {
        const int k = e & 1;
        CUMF_CUDA(cudaMemsetAsync(&st->batch_idx, 0, sizeof(int), ws));
        CUMF_CUDA(cudaMemsetAsync(&st->loss_sum, 0, sizeof(double), ws));
        CUMF_CUDA(cudaMemcpyAsync(perm_d.p, perm_h.p[k], (size_t)rows * 4, cudaMemcpyHostToDevice, ws));
        CUMF_CUDA(cudaEventRecord(res.ev[1 + k], ws));  // perm_h[k] may be redrawn after this
        for (int64_t i = 0; i < full; ++i) CUMF_CUDA(cudaGraphLaunch(res.exec[0], ws));
        if (tail > 0) CUMF_CUDA(cudaGraphLaunch(res.exec[1], ws));
        if (e + 1 < epochs) {
            CUMF_CUDA(cudaEventSynchronize(res.ev[1 + (k ^ 1)]));
            draw(static_cast<int32_t *>(perm_h.p[k ^ 1]));
        }
    }
    mp->step += (int64_t)epochs * (full + (tail > 0 ? 1 : 0));
    double sum = 0;
    CUMF_CUDA(cudaMemcpyAsync(&sum, &st->loss_sum, sizeof(double), cudaMemcpyDeviceToHost, ws));
    if (int rc = mlp_check_status(mp, ws)) return rc;  // synchronizes ws
    CUMF_CUDA(cudaEventRecord(res.ev[3], ws));
    CUMF_CUDA(cudaStreamWaitEvent(user, res.ev[3], 0));
    if (final_loss) *final_loss = sum / (double)rows;
    return CUMF_OK;
}

int cumf_user_features(const cumf_node *d_R, int64_t nnz, const float *d_Q, int32_t n, int k, int32_t m,
                       float *d_X, void *stream) {
    TraceRange trace("warm start: user features");
    if (!d_Q || !d_X || m <= 0 || n <= 0 || k <= 0 || nnz < 0 || (nnz > 0 && !d_R))
        return fail(CUMF_ERR_ARG, "user_features: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    if (nnz < 0xffffffffll && m < 0x7fffffff) {
        // The ratings stably sorted by user (32-bit keys and indices), then one warp per user.
        const uint32_t N = (uint32_t)nnz;
        int end_bit = 1;
        while (end_bit < 32 && ((uint32_t)m >> end_bit) != 0) ++end_bit;
        size_t tmp_bytes = 0;
        CUMF_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, (const uint32_t *)nullptr, (uint32_t *)nullptr,
                                                  (const uint32_t *)nullptr, (uint32_t *)nullptr, N, 0, end_bit, s));
        auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
        const size_t kb = up((size_t)N * 4 + 4), sb = up(((size_t)m + 1) * 8);
        void *buf = nullptr;
        CUMF_CUDA(feature_scratch(&buf, 4 * kb + sb + up(tmp_bytes), s));
        char *p = static_cast<char *>(buf);
        uint32_t *key = reinterpret_cast<uint32_t *>(p), *idx = reinterpret_cast<uint32_t *>(p + kb);
        uint32_t *key2 = reinterpret_cast<uint32_t *>(p + 2 * kb), *idx2 = reinterpret_cast<uint32_t *>(p + 3 * kb);
        int64_t *seg = reinterpret_cast<int64_t *>(p + 4 * kb);
        void *tmp = p + 4 * kb + sb;
        cudaError_t e = cudaSuccess;
        if (N > 0) {
            user_keys_kernel<<<grid_of(N), kT, 0, s>>>(d_R, N, m, n, key, idx);
            e = cudaGetLastError();
            if (e == cudaSuccess)
                e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, key, key2, idx, idx2, N, 0, end_bit, s);
        }
        if (e == cudaSuccess) {
            user_segments_kernel<<<grid_of((int64_t)m + 1), kT, 0, s>>>(key2, N, m, seg);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) {
            const int g = grid_of((int64_t)m * 32);
            if (k <= 32) user_rows_kernel<1><<<g, kT, 0, s>>>(d_R, idx2, seg, m, d_Q, k, d_X, k + 3);
            else if (k <= 64) user_rows_kernel<2><<<g, kT, 0, s>>>(d_R, idx2, seg, m, d_Q, k, d_X, k + 3);
            else if (k <= 128) user_rows_kernel<4><<<g, kT, 0, s>>>(d_R, idx2, seg, m, d_Q, k, d_X, k + 3);
            else user_rows_kernel<8><<<g, kT, 0, s>>>(d_R, idx2, seg, m, d_Q, k, d_X, k + 3);
            e = cudaGetLastError();
        }
        const cudaError_t ef = cudaFreeAsync(buf, s);
        CUMF_CUDA(e);
        CUMF_CUDA(ef);
        CUMF_CUDA(cudaStreamSynchronize(s));
        return CUMF_OK;
    }
    // 2^32 ratings or more: vector atomics into per-user rows.  One stream-ordered scratch: the
    // centred mean accumulates in k-wide rows (16-byte aligned for the vector atomics), then
    // degree, rating sum and sum of squares per user.
    const size_t acc_bytes = (size_t)m * k * 4, scratch = acc_bytes + 3 * (size_t)m * 4;
    void *buf = nullptr;
    CUMF_CUDA(cudaMallocAsync(&buf, scratch, s));
    float *acc = static_cast<float *>(buf);
    float *deg = acc + (size_t)m * k, *sum = deg + m, *sum2 = sum + m;
    cudaError_t e = cudaMemsetAsync(buf, 0, scratch, s);
    if (e == cudaSuccess && nnz > 0) {
        user_stats_kernel<<<grid_of(nnz), kT, 0, s>>>(d_R, nnz, m, n, deg, sum, sum2);
        user_qsum_kernel<<<grid_of(nnz * 32), kT, 0, s>>>(d_R, nnz, m, n, d_Q, k, deg, sum, acc, k);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        user_finish_kernel<<<grid_of((int64_t)m * (k + 3)), kT, 0, s>>>(m, k, acc, deg, sum, sum2, d_X, k + 3);
        e = cudaGetLastError();
    }
    const cudaError_t ef = cudaFreeAsync(buf, s);
    CUMF_CUDA(e);
    CUMF_CUDA(ef);
    CUMF_CUDA(cudaStreamSynchronize(s));
    return CUMF_OK;
}

}  // extern "C"
