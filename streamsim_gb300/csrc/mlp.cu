// mlp.cu — the warm-start network: MLP 12 -> 128 -> 128 -> 64, GELU,
// BF16 weights with an FP32 master copy, FP32 accumulation, trained by the
// library's own forward, backward and Adam kernels.
//
// Layout: parameters are one FP32 vector (W1[128x12], b1[128], W2[128x128],
// b2[128], W3[64x128], b3[64], row-major, W[out][in]); a BF16 copy of the
// weights is what the forward and backward GEMMs read.  Activations are
// row-major [n][features] FP32.  The loss is the mean squared error over
// all n x 64 outputs.
//
// GEMMs are one tiled kernel (64 x 64 output tile per CTA, 16-deep K
// slices staged in shared memory, 4 x 4 outputs per thread) with optional
// transposes, a BF16 operand, a bias + GELU epilogue, and split-K for the
// weight gradients (K = batch): each split writes its own partial and a
// second kernel sums the partials in a fixed order, so a training step is
// deterministic.
#include <cuda_bf16.h>

#include <cmath>

#include "internal.h"

namespace facetcu {
namespace mlp {


namespace {

constexpr int TM = 64, TN = 64, TK = 16;

__device__ __forceinline__ float gelu(float z)
{
    return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float z)
{
    const float cdf = 0.5f * (1.0f + erff(z * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * z * z);
    return cdf + z * pdf;
}

template <typename T> __device__ __forceinline__ float ld(const T* p);
template <> __device__ __forceinline__ float ld<float>(const float* p) { return *p; }
template <> __device__ __forceinline__ float ld<__nv_bfloat16>(const __nv_bfloat16* p)
{
    return __bfloat162float(*p);
}

// C[m][n] (+)= sum_k opA(m,k) * opB(k,n)   (split-K: C += z * M * N)
// opA(m,k) = TA ? A[k*lda + m] : A[m*lda + k]
// opB(k,n) = TB ? B[n*ldb + k] : B[k*ldb + n]
// epilogue: EPI 0 = store; 1 = + bias[n], store Z and GELU(Z) to C2.
template <bool TA, bool TB, typename TBT, int EPI>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const float* __restrict__ A,
                                              int lda, const TBT* __restrict__ B, int ldb,
                                              float* __restrict__ C, int ldc,
                                              const float* __restrict__ bias, float* __restrict__ C2,
                                              int k_per_split)
{
    __shared__ float As[TK][TM + 4];
    __shared__ float Bs[TK][TN + 4];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
    const int kb = blockIdx.z * k_per_split;
    const int ke = min(K, kb + k_per_split);
    float acc[4][4] = {};
    for (int k0 = kb; k0 < ke; k0 += TK) {
        for (int i = threadIdx.x; i < TM * TK; i += 256) {
            const int mm = TA ? i % TM : i / TK;
            const int kk = TA ? i / TM : i % TK;
            const int m = m0 + mm, k = k0 + kk;
            As[kk][mm] = (m < M && k < ke) ? (TA ? A[size_t(k) * lda + m] : A[size_t(m) * lda + k])
                                            : 0.0f;
        }
        for (int i = threadIdx.x; i < TN * TK; i += 256) {
            const int nn = TB ? i / TK : i % TN;
            const int kk = TB ? i % TK : i / TN;
            const int n = n0 + nn, k = k0 + kk;
            Bs[kk][nn] = (n < N && k < ke)
                             ? (TB ? ld(B + size_t(n) * ldb + k) : ld(B + size_t(k) * ldb + n))
                             : 0.0f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                a[i] = As[kk][ty * 4 + i];
                b[i] = Bs[kk][tx * 4 + i];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * b[j];
        }
        __syncthreads();
    }
    float* Cz = C + size_t(blockIdx.z) * M * ldc;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + ty * 4 + i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int n = n0 + tx * 4 + j;
            if (n >= N) continue;
            if (EPI == 0) {
                Cz[size_t(m) * ldc + n] = acc[i][j];
            } else {
                const float z = acc[i][j] + bias[n];
                Cz[size_t(m) * ldc + n] = z;
                C2[size_t(m) * ldc + n] = gelu(z);
            }
        }
    }
}

// out[i] = sum_z part[z * n + i], fixed order.
__global__ void k_sum_splits(const float* part, int splits, size_t n, float* out, float scale)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 0.0f;
    for (int z = 0; z < splits; ++z) s += part[size_t(z) * n + i];
    out[i] = s * scale;
}

// Column sums of X[n][cols] in fixed order: one thread per column, rows
// split in `splits` chunks written to part[split][col].
__global__ void k_colsum_part(const float* X, int rows, int cols, int rows_per_split, float* part)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.y;
    if (c >= cols) return;
    const int r0 = z * rows_per_split, r1 = min(rows, r0 + rows_per_split);
    float s = 0.0f;
    for (int r = r0; r < r1; ++r) s += X[size_t(r) * cols + c];
    part[size_t(z) * cols + c] = s;
}

// dY = 2 (Y - T) / (n * 64); loss partials per block.
__global__ void k_mse_grad(const float* Y, const float* T, size_t count, float scale, float* dY,
                           double* loss_part)
{
    __shared__ double red[256];
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (i < count) {
        const float d = Y[i] - T[i];
        dY[i] = 2.0f * d * scale;
        l = double(d) * double(d);
    }
    red[threadIdx.x] = l;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss_part[blockIdx.x] = red[0];
}

__global__ void k_sum_double(const double* part, int n, double* out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += part[i];
    *out = s;
}

// dZ = dA * gelu'(Z)
__global__ void k_gelu_back(const float* dA, const float* Z, size_t n, float* dZ)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) dZ[i] = dA[i] * gelu_grad(Z[i]);
}

__global__ void k_to_bf16(const float* p, size_t n, __nv_bfloat16* q)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) q[i] = __float2bfloat16_rn(p[i]);
}

// Adam (Kingma & Ba 2015) with bias correction.
__global__ void k_adam(float* p, const float* g, float* m, float* v, size_t n, float lr, float b1,
                       float b2, float eps, float c1, float c2)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Gather a minibatch: rows idx[i] of X (cols c) into out.
__global__ void k_gather_rows(const float* X, const uint32_t* idx, int n, int cols, float* out)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= size_t(n) * cols) return;
    const size_t r = i / cols, c = i % cols;
    out[i] = X[size_t(idx[r]) * cols + c];
}

// Minibatch indices from a counter-based hash (splitmix64 of seed, step, i).
__global__ void k_batch_indices(uint64_t seed, uint64_t step, int n, uint64_t population,
                                uint32_t* idx)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (step * 0x100000001ull + uint64_t(i) + 1ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    idx[i] = uint32_t(z % population);
}

inline unsigned blocks(size_t n, unsigned b) { return unsigned((n + b - 1) / b); }

}  // namespace

// ---- host side ---------------------------------------------------------------
static_assert(kParams == kParameterCount, "parameter layout");

void init_params(Net& net, uint32_t seed, cudaStream_t s)
{
    // Glorot-uniform weights, zero biases, from a host RNG (xorshift64*).
    std::vector<float> p(kParams, 0.0f);
    uint64_t state = 0x2545F4914F6CDD1Dull ^ (uint64_t(seed) * 0x9E3779B97F4A7C15ull);
    auto uni = [&]() {
        state ^= state >> 12;
        state ^= state << 25;
        state ^= state >> 27;
        const uint64_t r = state * 2685821657736338717ull;
        return double(r >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](int off, int fan_out, int fan_in) {
        const double lim = std::sqrt(6.0 / double(fan_in + fan_out));
        for (int i = 0; i < fan_out * fan_in; ++i) p[off + i] = float((2.0 * uni() - 1.0) * lim);
    };
    fill(kOffW1, kH, kIn);
    fill(kOffW2, kH, kH);
    fill(kOffW3, kOut, kH);
    net.params.reserve(kParams * 4);
    FCU_CHECK(cudaMemcpyAsync(net.params.ptr, p.data(), kParams * 4, cudaMemcpyHostToDevice, s));
    net.adam_m.reserve(kParams * 4);
    net.adam_v.reserve(kParams * 4);
    net.grad.reserve(kParams * 4);
    FCU_CHECK(cudaMemsetAsync(net.adam_m.ptr, 0, kParams * 4, s));
    FCU_CHECK(cudaMemsetAsync(net.adam_v.ptr, 0, kParams * 4, s));
    net.bf16.reserve(kParams * 2);
    k_to_bf16<<<blocks(kParams, 256), 256, 0, s>>>(net.params.as<float>(), kParams,
                                                   net.bf16.as<__nv_bfloat16>());
    FCU_LAUNCH("k_to_bf16");
    net.ready = true;
    net.steps_done = 0;
}

void set_params(Net& net, const float* host, cudaStream_t s)
{
    if (!net.ready) init_params(net, 1, s);
    FCU_CHECK(cudaMemcpyAsync(net.params.ptr, host, kParams * 4, cudaMemcpyHostToDevice, s));
    FCU_CHECK(cudaMemsetAsync(net.adam_m.ptr, 0, kParams * 4, s));
    FCU_CHECK(cudaMemsetAsync(net.adam_v.ptr, 0, kParams * 4, s));
    k_to_bf16<<<blocks(kParams, 256), 256, 0, s>>>(net.params.as<float>(), kParams,
                                                   net.bf16.as<__nv_bfloat16>());
    FCU_LAUNCH("k_to_bf16");
    net.steps_done = 0;
}

namespace {

template <bool TA, bool TB, typename TBT, int EPI>
void gemm(int M, int N, int K, const float* A, int lda, const TBT* B, int ldb, float* C, int ldc,
          const float* bias, float* C2, int splits, cudaStream_t s)
{
    const int kps = ((K + splits - 1) / splits + TK - 1) / TK * TK;
    dim3 grid(unsigned((N + TN - 1) / TN), unsigned((M + TM - 1) / TM), unsigned(splits));
    k_gemm<TB ? TA : TA, TB, TBT, EPI><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias,
                                                           C2, kps);
    FCU_LAUNCH("k_gemm");
}

}  // namespace

// Forward pass of n rows (activations kept in sc for a backward pass).
static void forward(Net& net, const float* X, int n, Scratch& sc, float* Y, cudaStream_t s)
{
    const __nv_bfloat16* w = net.bf16.as<__nv_bfloat16>();
    const float* p = net.params.as<float>();
    float* z1 = static_cast<float*>(sc.z1.reserve(size_t(n) * kH * 4));
    float* a1 = static_cast<float*>(sc.a1.reserve(size_t(n) * kH * 4));
    float* z2 = static_cast<float*>(sc.z2.reserve(size_t(n) * kH * 4));
    float* a2 = static_cast<float*>(sc.a2.reserve(size_t(n) * kH * 4));
    // Z1 = X W1^T + b1 ; A1 = gelu(Z1)
    gemm<false, true, __nv_bfloat16, 1>(n, kH, kIn, X, kIn, w + kOffW1, kIn, z1, kH, p + kOffB1,
                                        a1, 1, s);
    gemm<false, true, __nv_bfloat16, 1>(n, kH, kH, a1, kH, w + kOffW2, kH, z2, kH, p + kOffB2, a2,
                                        1, s);
    // Y = A2 W3^T + b3 (no activation): use EPI 1 into a scratch then copy?
    // The output layer has no GELU: EPI 0, then add the bias in the loss or
    // here with a tiny kernel.
    gemm<false, true, __nv_bfloat16, 0>(n, kOut, kH, a2, kH, w + kOffW3, kH, Y, kOut, nullptr,
                                        nullptr, 1, s);
}

static __global__ void k_add_bias(float* Y, const float* b, size_t rows, int cols)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < rows * cols) Y[i] += b[i % cols];
}

void forward_full(Net& net, const float* X, int n, Scratch& sc, float* Y, cudaStream_t s)
{
    forward(net, X, n, sc, Y, s);
    k_add_bias<<<blocks(size_t(n) * kOut, 256), 256, 0, s>>>(Y, net.params.as<float>() + kOffB3,
                                                             size_t(n), kOut);
    FCU_LAUNCH("k_add_bias");
}

// Inference over any number of rows: chunks of kInferChunk rows keep the
// activation scratch at 1 GB and the GEMM grid within its y limit.
void infer(Net& net, const float* X, size_t n, Scratch& sc, float* Y, cudaStream_t s)
{
    for (size_t r0 = 0; r0 < n; r0 += kInferChunk) {
        const int rows = int(std::min(n - r0, kInferChunk));
        forward_full(net, X + r0 * kIn, rows, sc, Y + r0 * kOut, s);
    }
}

// Loss and gradient (into net.grad) of one batch; returns the mean loss.
double loss_and_grad(Net& net, const float* X, const float* T, int n, Scratch& sc, cudaStream_t s,
                     bool want_loss)
{
    float* Y = static_cast<float*>(sc.y.reserve(size_t(n) * kOut * 4));
    forward_full(net, X, n, sc, Y, s);
    float* dY = static_cast<float*>(sc.dy.reserve(size_t(n) * kOut * 4));
    const size_t cnt = size_t(n) * kOut;
    const unsigned lb = blocks(cnt, 256);
    double* lossp = static_cast<double*>(sc.lossp.reserve((lb + 1) * 8));
    k_mse_grad<<<lb, 256, 0, s>>>(Y, T, cnt, 1.0f / float(cnt), dY, lossp);
    FCU_LAUNCH("k_mse_grad");
    const __nv_bfloat16* w = net.bf16.as<__nv_bfloat16>();
    float* g = net.grad.as<float>();
    const int splits = std::max(1, std::min(64, n / 512));
    float* part = static_cast<float*>(sc.part.reserve(size_t(splits) * kH * kH * 4 + 64));
    float* da = static_cast<float*>(sc.da.reserve(size_t(n) * kH * 4));
    float* dz = static_cast<float*>(sc.dz.reserve(size_t(n) * kH * 4));
    const int rps = (n + splits - 1) / splits;
    // layer 3: dW3[o][h] = sum_r dY[r][o] A2[r][h]; db3 = colsum dY
    gemm<true, false, float, 0>(kOut, kH, n, dY, kOut, sc.a2.as<float>(), kH, part, kH, nullptr,
                                nullptr, splits, s);
    k_sum_splits<<<blocks(kW3, 256), 256, 0, s>>>(part, splits, kW3, g + kOffW3, 1.0f);
    k_colsum_part<<<dim3(blocks(kOut, 128), splits), 128, 0, s>>>(dY, n, kOut, rps, part);
    k_sum_splits<<<1, 128, 0, s>>>(part, splits, kB3, g + kOffB3, 1.0f);
    // dA2 = dY W3 ; dZ2 = dA2 gelu'(Z2)
    gemm<false, false, __nv_bfloat16, 0>(n, kH, kOut, dY, kOut, w + kOffW3, kH, da, kH, nullptr,
                                         nullptr, 1, s);
    k_gelu_back<<<blocks(size_t(n) * kH, 256), 256, 0, s>>>(da, sc.z2.as<float>(), size_t(n) * kH,
                                                            dz);
    // layer 2: dW2 = dZ2^T A1 ; db2 = colsum dZ2
    gemm<true, false, float, 0>(kH, kH, n, dz, kH, sc.a1.as<float>(), kH, part, kH, nullptr,
                                nullptr, splits, s);
    k_sum_splits<<<blocks(kW2, 256), 256, 0, s>>>(part, splits, kW2, g + kOffW2, 1.0f);
    k_colsum_part<<<dim3(blocks(kH, 128), splits), 128, 0, s>>>(dz, n, kH, rps, part);
    k_sum_splits<<<1, 128, 0, s>>>(part, splits, kB2, g + kOffB2, 1.0f);
    // dA1 = dZ2 W2 ; dZ1 = dA1 gelu'(Z1)
    gemm<false, false, __nv_bfloat16, 0>(n, kH, kH, dz, kH, w + kOffW2, kH, da, kH, nullptr,
                                         nullptr, 1, s);
    k_gelu_back<<<blocks(size_t(n) * kH, 256), 256, 0, s>>>(da, sc.z1.as<float>(), size_t(n) * kH,
                                                            dz);
    // layer 1: dW1 = dZ1^T X ; db1 = colsum dZ1
    gemm<true, false, float, 0>(kH, kIn, n, dz, kH, X, kIn, part, kIn, nullptr, nullptr, splits, s);
    k_sum_splits<<<blocks(kW1, 256), 256, 0, s>>>(part, splits, kW1, g + kOffW1, 1.0f);
    k_colsum_part<<<dim3(blocks(kH, 128), splits), 128, 0, s>>>(dz, n, kH, rps, part);
    k_sum_splits<<<1, 128, 0, s>>>(part, splits, kB1, g + kOffB1, 1.0f);
    FCU_LAUNCH("mlp backward");
    if (!want_loss) return 0.0;
    double* total = lossp + lb;
    k_sum_double<<<1, 1, 0, s>>>(lossp, int(lb), total);
    double host = 0.0;
    FCU_CHECK(cudaMemcpyAsync(&host, total, 8, cudaMemcpyDeviceToHost, s));
    FCU_CHECK(cudaStreamSynchronize(s));
    return host / double(cnt);
}

void adam_step(Net& net, float lr, cudaStream_t s)
{
    net.steps_done += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, float(net.steps_done));
    const float c2 = 1.0f - std::pow(b2, float(net.steps_done));
    k_adam<<<blocks(kParams, 256), 256, 0, s>>>(net.params.as<float>(), net.grad.as<float>(),
                                                net.adam_m.as<float>(), net.adam_v.as<float>(),
                                                kParams, lr, b1, b2, 1e-8f, c1, c2);
    FCU_LAUNCH("k_adam");
    k_to_bf16<<<blocks(kParams, 256), 256, 0, s>>>(net.params.as<float>(), kParams,
                                                   net.bf16.as<__nv_bfloat16>());
    FCU_LAUNCH("k_to_bf16");
}

// Train on n samples resident on the device (X[n][12], T[n][64]).
double train(Net& net, const float* X, const float* T, uint64_t n, uint32_t steps, uint32_t batch,
             float lr, uint32_t seed, Scratch& sc, cudaStream_t s)
{
    uint32_t* idx = static_cast<uint32_t*>(sc.idx.reserve(size_t(batch) * 4));
    float* xb = static_cast<float*>(sc.xb.reserve(size_t(batch) * kIn * 4));
    float* tb = static_cast<float*>(sc.tb.reserve(size_t(batch) * kOut * 4));
    double last = 0.0;
    for (uint32_t st = 0; st < steps; ++st) {
        k_batch_indices<<<blocks(batch, 256), 256, 0, s>>>(seed, st, int(batch), n, idx);
        k_gather_rows<<<blocks(size_t(batch) * kIn, 256), 256, 0, s>>>(X, idx, int(batch), kIn, xb);
        k_gather_rows<<<blocks(size_t(batch) * kOut, 256), 256, 0, s>>>(T, idx, int(batch), kOut, tb);
        const bool report = st + 1 == steps;
        const double l = loss_and_grad(net, xb, tb, int(batch), sc, s, report);
        if (report) last = l;
        adam_step(net, lr, s);
    }
    FCU_CHECK(cudaStreamSynchronize(s));
    return last;
}

// ---- features and warm start ----------------------------------------------
// Per (sun k, side s): the first-order radiosity B1 (one sweep from zero) of
// 8 band groups (bands 0, 9, ..., 63) scaled by ref_b = sky_b + beam_b, the
// reflectance and transmittance of band 32, the sky-view fraction
// sky_s / denom_s (1 when denom = 0) and the side normal's y (up) component.
__global__ void k_features(const float* B1, uint32_t S, uint32_t bands, uint32_t suns,
                           const float* rho, const float* tau, const float* sky,
                           const float* beam, const uint32_t* denom, const uint32_t* skyc,
                           const facetcu_vertex* V, float* X)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= size_t(S) * suns) return;
    const uint32_t k = uint32_t(i / S), s = uint32_t(i % S);
    float* x = X + i * kIn;
    for (int g = 0; g < 8; ++g) {
        const uint32_t b = uint32_t(g * 9);
        const float ref = sky[b] + beam[b];
        x[g] = B1[(size_t(k) * bands + b) * S + s] / (ref > 0.0f ? ref : 1.0f);
    }
    const uint32_t mid = bands / 2;
    x[8] = rho[size_t(mid) * S + s];
    x[9] = tau[size_t(mid) * S + s];
    x[10] = denom[s] ? float(skyc[s]) / float(denom[s]) : 1.0f;
    const float ny = V[3 * (s >> 1)].normal[1];
    x[11] = (s & 1u) ? -ny : ny;
}

// x0[k*bands + b][s] = B1 + Y[(k*S + s)][b] * ref_b  (Y = predicted (B - B1) / ref)
__global__ void k_warm_combine(const float* B1, const float* Y, uint32_t S, uint32_t bands,
                               uint32_t suns, const float* sky, const float* beam, float* x0)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const size_t total = size_t(S) * bands * suns;
    if (i >= total) return;
    const size_t col = i / S;
    const uint32_t s = uint32_t(i % S);
    const uint32_t b = uint32_t(col % bands), k = uint32_t(col / bands);
    const float ref = sky[b] + beam[b];
    const float y = Y[(size_t(k) * S + s) * kOut + b];
    x0[i] = fmaxf(0.0f, B1[i] + y * ref);
}

// T[(k*S + s)][b] = (B - B1) / ref_b  (training targets)
__global__ void k_targets(const float* B, const float* B1, uint32_t S, uint32_t bands,
                          uint32_t suns, const float* sky, const float* beam, float* T)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const size_t total = size_t(S) * bands * suns;
    if (i >= total) return;
    const size_t col = i / S;
    const uint32_t s = uint32_t(i % S);
    const uint32_t b = uint32_t(col % bands), k = uint32_t(col / bands);
    const float ref = sky[b] + beam[b];
    T[(size_t(k) * S + s) * kOut + b] = (B[i] - B1[i]) / (ref > 0.0f ? ref : 1.0f);
}

void features(const float* B1, uint32_t S, uint32_t bands, uint32_t suns, const float* rho,
              const float* tau, const float* sky, const float* beam, const uint32_t* denom,
              const uint32_t* skyc, const facetcu_vertex* V, float* X, cudaStream_t s)
{
    k_features<<<blocks(size_t(S) * suns, 256), 256, 0, s>>>(B1, S, bands, suns, rho, tau, sky,
                                                             beam, denom, skyc, V, X);
    FCU_LAUNCH("k_features");
}

void warm_combine(const float* B1, const float* Y, uint32_t S, uint32_t bands, uint32_t suns,
                  const float* sky, const float* beam, float* x0, cudaStream_t s)
{
    k_warm_combine<<<blocks(size_t(S) * bands * suns, 256), 256, 0, s>>>(B1, Y, S, bands, suns,
                                                                         sky, beam, x0);
    FCU_LAUNCH("k_warm_combine");
}

void targets(const float* B, const float* B1, uint32_t S, uint32_t bands, uint32_t suns,
             const float* sky, const float* beam, float* T, cudaStream_t s)
{
    k_targets<<<blocks(size_t(S) * bands * suns, 256), 256, 0, s>>>(B, B1, S, bands, suns, sky,
                                                                    beam, T);
    FCU_LAUNCH("k_targets");
}

}  // namespace mlp
}  // namespace facetcu
