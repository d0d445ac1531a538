// sort.cu — device exclusive scan and stable LSD radix sort.
//
// Both are written for the graph build: the scan turns per-pixel fragment
// counts into list offsets, the sort groups (side, side) pair keys so that
// the symmetric CSR comes out row-sorted and deterministic (the reference
// uses a hash map on the CPU, facetrtcore.cpp:1358-1412, and a 64-bit-key
// GPU hash compacted on the host, facetrt_vulkan.cpp:979-1037).
#include "internal.h"

namespace facetcu {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;  // 2048

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---- scan ---------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* warp_sums, T& block_total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T w = lane < kThreads / 32 ? warp_sums[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kThreads / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    const T before = warp == 0 ? T(0) : warp_sums[warp - 1];
    block_total = warp_sums[kThreads / 32 - 1];
    return before + x - v;
}

// Tile sums (u64) of a u32 (or u64) array.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_tile_sums(const T* in, size_t n,
                                                        unsigned long long* sums)
{
    __shared__ unsigned long long ws[kThreads / 32];
    const size_t base = size_t(blockIdx.x) * kTile;
    unsigned long long acc = 0;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const size_t idx = base + size_t(i) * kThreads + threadIdx.x;
        if (idx < n) acc += in[idx];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) ws[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < kThreads / 32; ++w) t += ws[w];
        sums[blockIdx.x] = t;
    }
}

// Exclusive scan of each tile plus the tile offset.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_tile_scan(const T* in, T* out, size_t n,
                                                        const unsigned long long* offsets)
{
    __shared__ T tile[kTile];
    __shared__ T ws[kThreads / 32];
    const size_t base = size_t(blockIdx.x) * kTile;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const int j = i * kThreads + threadIdx.x;
        const size_t idx = base + j;
        tile[j] = idx < n ? in[idx] : T(0);
    }
    __syncthreads();
    T local[kItems];
    T sum = 0;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        local[i] = tile[threadIdx.x * kItems + i];
        sum += local[i];
    }
    T total;
    T run = block_exclusive_scan<T>(sum, ws, total) + T(offsets ? offsets[blockIdx.x] : 0ULL);
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        tile[threadIdx.x * kItems + i] = run;
        run += local[i];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const int j = i * kThreads + threadIdx.x;
        const size_t idx = base + j;
        if (idx < n) out[idx] = tile[j];
    }
}

// ---- radix sort -----------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_digit_histogram(const uint64_t* keys, size_t n,
                                                              int shift, uint32_t* hist,
                                                              uint32_t blocks)
{
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const size_t base = size_t(blockIdx.x) * kTile;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const size_t idx = base + size_t(i) * kThreads + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[size_t(threadIdx.x) * blocks + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kThreads) k_digit_scatter(
    const uint64_t* keys, const uint32_t* values, uint64_t* keys_out, uint32_t* values_out,
    size_t n, int shift, const uint32_t* offsets, uint32_t blocks)
{
    __shared__ uint32_t s_base[256];
    __shared__ uint32_t s_warp[kThreads / 32][256];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    s_base[t] = offsets[size_t(t) * blocks + blockIdx.x];
    const size_t base = size_t(blockIdx.x) * kTile;
    const unsigned lt = lanemask_lt();
    for (int r = 0; r < kItems; ++r) {
        const size_t idx = base + size_t(r) * kThreads + t;
        const bool valid = idx < n;
        const uint64_t key = valid ? keys[idx] : 0ull;
        const uint32_t val = (valid && values) ? values[idx] : 0u;
        const uint32_t digit = valid ? uint32_t((key >> shift) & 255u) : 256u;
#pragma unroll
        for (int w = 0; w < kThreads / 32; ++w) s_warp[w][t] = 0;
        __syncthreads();
        const unsigned peers = __match_any_sync(0xffffffffu, digit);
        const uint32_t rank = __popc(peers & lt);
        if (valid && rank == 0) s_warp[warp][digit] = __popc(peers);
        __syncthreads();
        uint32_t run = s_base[t];
#pragma unroll
        for (int w = 0; w < kThreads / 32; ++w) {
            const uint32_t c = s_warp[w][t];
            s_warp[w][t] = run;
            run += c;
        }
        s_base[t] = run;
        __syncthreads();
        if (valid) {
            const uint32_t pos = s_warp[warp][digit] + rank;
            keys_out[pos] = key;
            if (values) values_out[pos] = val;
        }
        __syncthreads();
    }
}

}  // namespace

void exclusive_scan_u32(const uint32_t* in, uint32_t* out, size_t n,
                        unsigned long long* total_dev, Workspace& ws, cudaStream_t s)
{
    if (n == 0) {
        if (total_dev) FCU_CHECK(cudaMemsetAsync(total_dev, 0, 8, s));
        return;
    }
    // Level sizes: level 1 holds the tile sums of the input, level k+1 the
    // tile sums of level k, up to a single element (the total).
    size_t sizes[8];
    size_t offs[8];
    int levels = 0;
    size_t m = n, total_elems = 0;
    do {
        m = (m + kTile - 1) / kTile;
        sizes[levels] = m;
        offs[levels] = total_elems;
        total_elems += m;
        ++levels;
    } while (m > 1 && levels < 8);
    unsigned long long* buf = static_cast<unsigned long long*>(
        ws.d.reserve((total_elems + 1) * sizeof(unsigned long long)));
    k_tile_sums<uint32_t><<<unsigned(sizes[0]), kThreads, 0, s>>>(in, n, buf + offs[0]);
    FCU_LAUNCH("k_tile_sums");
    for (int l = 1; l < levels; ++l) {
        k_tile_sums<unsigned long long><<<unsigned(sizes[l]), kThreads, 0, s>>>(
            buf + offs[l - 1], sizes[l - 1], buf + offs[l]);
        FCU_LAUNCH("k_tile_sums");
    }
    unsigned long long* top = buf + offs[levels - 1];
    if (total_dev) FCU_CHECK(cudaMemcpyAsync(total_dev, top, 8, cudaMemcpyDeviceToDevice, s));
    FCU_CHECK(cudaMemsetAsync(top, 0, 8, s));
    for (int l = levels - 2; l >= 0; --l) {
        k_tile_scan<unsigned long long><<<unsigned(sizes[l + 1]), kThreads, 0, s>>>(
            buf + offs[l], buf + offs[l], sizes[l], buf + offs[l + 1]);
        FCU_LAUNCH("k_tile_scan");
    }
    k_tile_scan<uint32_t><<<unsigned(sizes[0]), kThreads, 0, s>>>(in, out, n, buf + offs[0]);
    FCU_LAUNCH("k_tile_scan");
}

void radix_sort_u64(uint64_t*& keys, uint64_t*& keys_alt, uint32_t*& values,
                    uint32_t*& values_alt, size_t n, int key_bits, Workspace& ws,
                    cudaStream_t s)
{
    if (n <= 1 || key_bits <= 0) return;
    const uint32_t blocks = uint32_t((n + kTile - 1) / kTile);
    uint32_t* hist = static_cast<uint32_t*>(ws.c.reserve(size_t(blocks) * 256 * 4 + 16));
    for (int shift = 0; shift < key_bits; shift += 8) {
        k_digit_histogram<<<blocks, kThreads, 0, s>>>(keys, n, shift, hist, blocks);
        FCU_LAUNCH("k_digit_histogram");
        exclusive_scan_u32(hist, hist, size_t(blocks) * 256, nullptr, ws, s);
        k_digit_scatter<<<blocks, kThreads, 0, s>>>(keys, values, keys_alt, values_alt, n, shift,
                                                    hist, blocks);
        FCU_LAUNCH("k_digit_scatter");
        std::swap(keys, keys_alt);
        if (values) std::swap(values, values_alt);
    }
}

}  // namespace facetcu
