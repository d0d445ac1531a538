// mlp_tc.cu — the warm-start network's inference on the 5th-generation
// tensor cores (tcgen05), BF16 operands, FP32 accumulation in tensor memory.
//
// One CTA computes 128 rows of one layer, out[128 x N] = act(in[128 x K]
// W^T + b), with N = 128 (hidden layers) or 64 (output layer):
//   * one thread loads the CTA's rows of the BF16 input and the whole BF16
//     weight matrix into shared memory with 2-D TMA tiles
//     (cp.async.bulk.tensor, 64 x 128 boxes of 128-byte rows, 128-byte
//     swizzle), completing on an mbarrier;
//   * the same thread issues the K / 16 tcgen05.mma (kind::f16, M = 128,
//     N, K = 16) that accumulate into N columns of tensor memory, and
//     tcgen05.commit arrives on a second mbarrier when they are done;
//   * the four warps read the accumulator back (tcgen05.ld, 32 lanes x 32
//     columns each), add the bias, apply GELU on hidden layers and store
//     BF16 activations (hidden) or FP32 outputs.
// Every wait is bounded (1 s): a wait that runs out sets the error flag,
// waits once more (bounded) for the work in flight and frees the tensor
// memory before the CTA exits.  With FACETCU_TEST_STALL_TENSOR_WAIT=1 in the
// environment (read at each call; for tests of that path) the load barrier
// expects 16 bytes more than the loads deliver, so its wait runs out and
// the call reports FACETCU_DEVICE_TIMEOUT.
//
// The input rows are BF16 padded to 64 features (128 bytes); the first
// layer's weight matrix is padded the same way.  Hidden activations are
// BF16 (the SIMT path of mlp.cu keeps FP32 activations; the difference is a
// BF16 rounding per layer, ~1e-2 of the output scale).
#include <cstdlib>

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include "internal.h"

namespace facetcu {
namespace mlp {
namespace {

constexpr int kTileM = 128;        // rows per CTA (the MMA's M)
constexpr int kBoxK = 64;          // BF16 elements per TMA box row: 128 bytes
constexpr int kBoxBytesRow = 128;  // bytes per box row
constexpr int kTmemCols = 128;     // tensor-memory columns per CTA (>= N, a power of two)
constexpr int kPadIn = 64;         // padded input features (128-byte rows)
constexpr unsigned long long kWaitNs = 1000000000ull;

template <int N, int KB>
struct TcLayout {
    static constexpr int kA = KB * kTileM * kBoxBytesRow;  // input boxes
    static constexpr int kB = KB * N * kBoxBytesRow;       // weight boxes
    static constexpr int kBytes = kA + kB + 64 + 1024;     // + barriers, + alignment slack
};

__device__ __forceinline__ uint32_t su32(const void* p)
{
    return uint32_t(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ unsigned long long gtime()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity)
{
    const uint32_t a = su32(bar);
    const unsigned long long t0 = gtime();
    for (uint32_t i = 0;; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
        if ((i & 63u) == 63u && gtime() - t0 > kWaitNs) return false;
    }
}

// SMEM matrix descriptor of a K-major BF16 tile in the 128-byte swizzle
// layout TMA writes: start address >> 4 (bits 0-13), leading-dimension
// byte offset 16 >> 4 (unused for swizzled K-major tiles), stride byte
// offset 1024 >> 4 (8 rows of 128 bytes, bits 32-45), version 1 (bit 46),
// base offset 0 (tiles are 1024-byte aligned), swizzle mode 2 = 128-byte
// (bits 61-63).  A K step of 16 elements advances the start address by 32
// bytes inside the swizzle atom.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr)
{
    uint64_t d = uint64_t((addr & 0x3FFFFu) >> 4);
    d |= uint64_t(16 >> 4) << 16;
    d |= uint64_t(1024 >> 4) << 32;
    d |= uint64_t(1) << 46;
    d |= uint64_t(2) << 61;
    return d;
}

// Instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator (bits
// 4-5 = 1), BF16 A and B (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15,
// 16 = 0), N >> 3 (bits 17-22), M >> 4 (bits 24-28).
template <int N>
__host__ __device__ constexpr uint32_t idesc()
{
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) |
           (uint32_t(kTileM >> 4) << 24);
}

__device__ __forceinline__ void tma_load(void* dst, const CUtensorMap* map, int x, int y,
                                         uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(su32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(su32(bar))
        : "memory");
}

__device__ __forceinline__ float gelu(float z)
{
    return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f));
}

// out[r][n] = act(sum_k in[r][k] W[n][k] + bias[n]) for the CTA's 128 rows;
// KB boxes of 64 features, KS MMA steps of 16 features (KS <= 4 KB).
template <int N, int KB, int KS, bool kGelu, typename OutT>
__global__ void __launch_bounds__(128) k_mlp_tc(const __grid_constant__ CUtensorMap amap,
                                                const __grid_constant__ CUtensorMap bmap,
                                                const float* __restrict__ bias,
                                                OutT* __restrict__ out, uint32_t n,
                                                uint32_t* error, uint32_t extra_tx)
{
    static_assert(N % 32 == 0 && N <= kTmemCols && N >= 32, "N");
    static_assert(KS >= 1 && KS <= 4 * KB, "K steps");
    using Lay = TcLayout<N, KB>;
    extern __shared__ __align__(1024) unsigned char raw[];
    unsigned char* sm = raw + ((1024u - (su32(raw) & 1023u)) & 1023u);
    unsigned char* sA = sm;
    unsigned char* sB = sm + Lay::kA;
    uint64_t* bar_load = reinterpret_cast<uint64_t*>(sm + Lay::kA + Lay::kB);
    uint64_t* bar_mma = bar_load + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar_load + 2);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t row0 = blockIdx.x * kTileM;

    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(bar_load)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(bar_mma)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         su32(tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    bool issued = false;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar_load)),
                     "r"(uint32_t(Lay::kA + Lay::kB) + extra_tx)
                     : "memory");
#pragma unroll
        for (int kb = 0; kb < KB; ++kb) {
            tma_load(sA + kb * kTileM * kBoxBytesRow, &amap, kb * kBoxK, int(row0), bar_load);
            tma_load(sB + kb * N * kBoxBytesRow, &bmap, kb * kBoxK, 0, bar_load);
        }
        if (mbar_wait(bar_load, 0)) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int k = 0; k < KS; ++k) {
                const int kb = k / 4, kk = k % 4;
                const uint64_t a = sdesc(su32(sA + kb * kTileM * kBoxBytesRow + kk * 32));
                const uint64_t b = sdesc(su32(sB + kb * N * kBoxBytesRow + kk * 32));
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(a), "l"(b), "r"(idesc<N>()), "r"(uint32_t(k))
                    : "memory");
            }
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    su32(bar_mma))
                : "memory");
            issued = true;
        } else {
            atomicExch(error, 1u);
            mbar_wait(bar_load, 0);  // the loads in flight, once more (bounded)
        }
    }
    // every thread waits for the accumulator (a CTA whose loads timed out
    // never commits: its threads time out here and skip the epilogue)
    bool ready = mbar_wait(bar_mma, 0);
    ready = __all_sync(0xffffffffu, ready);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ready) {
        const uint32_t r = row0 + uint32_t(warp * 32 + lane);
#pragma unroll
        for (int c = 0; c < N / 32; ++c) {
            uint32_t v[32];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, "
                "%10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, "
                "%26, %27, %28, %29, %30, %31}, [%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                  "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
                  "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]),
                  "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
                  "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
                  "=r"(v[30]), "=r"(v[31])
                : "r"(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c * 32)));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (r < n) {
                // bias and activation, then 16-byte stores of the row's 32 columns
                float z[32];
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    z[j] = __uint_as_float(v[j]) + __ldg(bias + c * 32 + j);
                    if (kGelu) z[j] = gelu(z[j]);
                }
                uint4* dst = reinterpret_cast<uint4*>(out + size_t(r) * N + c * 32);
                if constexpr (sizeof(OutT) == 2) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        uint32_t w[4];
#pragma unroll
                        for (int t = 0; t < 4; ++t) {
                            const __nv_bfloat162 b2 =
                                __floats2bfloat162_rn(z[8 * q + 2 * t], z[8 * q + 2 * t + 1]);
                            w[t] = *reinterpret_cast<const uint32_t*>(&b2);
                        }
                        dst[q] = make_uint4(w[0], w[1], w[2], w[3]);
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        dst[q] = make_uint4(__float_as_uint(z[4 * q]), __float_as_uint(z[4 * q + 1]),
                                            __float_as_uint(z[4 * q + 2]),
                                            __float_as_uint(z[4 * q + 3]));
                }
            }
        }
    } else if (threadIdx.x == 0) {
        atomicExch(error, 1u);
        if (issued) mbar_wait(bar_mma, 0);  // the MMAs in flight, once more (bounded)
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTmemCols)
                     : "memory");
    }
}

// x[n][12] FP32 -> BF16 rows of 64 (features 12..63 zero)
__global__ void k_pack_inputs(const float* __restrict__ x, size_t n, __nv_bfloat16* __restrict__ xb)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n * kPadIn) return;
    const size_t r = i / kPadIn, c = i % kPadIn;
    xb[i] = __float2bfloat16_rn(c < size_t(kIn) ? x[r * kIn + c] : 0.0f);
}

// W1 [128][12] BF16 -> [128][64] (zero-padded)
__global__ void k_pad_w1(const __nv_bfloat16* __restrict__ w1, __nv_bfloat16* __restrict__ w1p)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kH * kPadIn) return;
    const int r = i / kPadIn, c = i % kPadIn;
    w1p[i] = c < kIn ? w1[r * kIn + c] : __float2bfloat16_rn(0.0f);
}

PFN_cuTensorMapEncodeTiled_v12000 encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    if (!fn) throw Error(FACETCU_CUDA_ERROR, "cuTensorMapEncodeTiled is not available");
    return fn;
}

// 2-D BF16 tensor [rows][cols] (row stride cols * 2 bytes), boxes of
// 64 x box_rows with 128-byte swizzle.
CUtensorMap tensor_map(const void* base, uint64_t cols, uint64_t rows, uint32_t box_rows)
{
    if (reinterpret_cast<uintptr_t>(base) % 16 != 0 || (cols * 2) % 16 != 0)
        throw Error(FACETCU_INVALID_ARGUMENT, "tensor map: 16-byte alignment");
    CUtensorMap m;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * 2};
    const cuuint32_t box[2] = {uint32_t(kBoxK), box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base),
                                 dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                 CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        throw Error(FACETCU_CUDA_ERROR, "cuTensorMapEncodeTiled failed: " + std::to_string(int(r)));
    return m;
}

template <int N, int KB, int KS, bool kGelu, typename OutT>
void layer(const CUtensorMap& a, const CUtensorMap& b, const float* bias, OutT* out, size_t n,
           uint32_t* error, uint32_t extra_tx, cudaStream_t s)
{
    auto kern = k_mlp_tc<N, KB, KS, kGelu, OutT>;
    constexpr int bytes = TcLayout<N, KB>::kBytes;
    static const bool attr = [&] {
        FCU_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        return true;
    }();
    (void)attr;
    const unsigned grid = unsigned((n + kTileM - 1) / kTileM);
    kern<<<grid, 128, bytes, s>>>(a, b, bias, out, uint32_t(n), error, extra_tx);
    FCU_LAUNCH("k_mlp_tc");
}

}  // namespace

void infer_tensor(Net& net, const float* X, size_t n, TensorScratch& ts, float* Y, cudaStream_t s)
{
    if (n == 0) return;
    if (n > (size_t(1) << 30)) throw Error(FACETCU_OVERFLOW_ERROR, "too many rows for the tensor path");
    const __nv_bfloat16* w = net.bf16.as<__nv_bfloat16>();
    const float* p = net.params.as<float>();
    __nv_bfloat16* xb = static_cast<__nv_bfloat16*>(ts.xb.reserve(n * kPadIn * 2));
    __nv_bfloat16* a1 = static_cast<__nv_bfloat16*>(ts.a1.reserve(n * kH * 2));
    __nv_bfloat16* a2 = static_cast<__nv_bfloat16*>(ts.a2.reserve(n * kH * 2));
    __nv_bfloat16* w1p = static_cast<__nv_bfloat16*>(ts.w1p.reserve(size_t(kH) * kPadIn * 2));
    uint32_t* err = static_cast<uint32_t*>(ts.error.reserve(16));
    FCU_CHECK(cudaMemsetAsync(err, 0, 4, s));
    k_pack_inputs<<<unsigned((n * kPadIn + 255) / 256), 256, 0, s>>>(X, n, xb);
    FCU_LAUNCH("k_pack_inputs");
    k_pad_w1<<<(kH * kPadIn + 255) / 256, 256, 0, s>>>(w + kOffW1, w1p);
    FCU_LAUNCH("k_pad_w1");
    const CUtensorMap mx = tensor_map(xb, kPadIn, n, kTileM);
    const CUtensorMap m1 = tensor_map(a1, kH, n, kTileM);
    const CUtensorMap m2 = tensor_map(a2, kH, n, kTileM);
    const CUtensorMap mw1 = tensor_map(w1p, kPadIn, kH, kH);
    const CUtensorMap mw2 = tensor_map(w + kOffW2, kH, kH, kH);
    const CUtensorMap mw3 = tensor_map(w + kOffW3, kH, kOut, kOut);
    const char* stall = std::getenv("FACETCU_TEST_STALL_TENSOR_WAIT");
    const uint32_t extra = stall && stall[0] == '1' ? 16u : 0u;
    // A1 = gelu(X W1^T + b1): one K step (12 features + 4 zeros)
    layer<kH, 1, 1, true, __nv_bfloat16>(mx, mw1, p + kOffB1, a1, n, err, extra, s);
    // A2 = gelu(A1 W2^T + b2)
    layer<kH, 2, 8, true, __nv_bfloat16>(m1, mw2, p + kOffB2, a2, n, err, extra, s);
    // Y = A2 W3^T + b3
    layer<kOut, 2, 8, false, float>(m2, mw3, p + kOffB3, Y, n, err, extra, s);
}

uint32_t tensor_error(TensorScratch& ts, cudaStream_t s)
{
    if (!ts.error.ptr) return 0;
    uint32_t h = 0;
    FCU_CHECK(cudaMemcpyAsync(&h, ts.error.ptr, 4, cudaMemcpyDeviceToHost, s));
    FCU_CHECK(cudaStreamSynchronize(s));
    return h;
}

}  // namespace mlp
}  // namespace facetcu
