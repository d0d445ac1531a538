// graph.cu — symmetric count-form CSR from undirected (side, side) pair keys.
//
// The reference counts pairs in a std::unordered_map (buildCpuGraph,
// facetrtcore.cpp:1390) or a GPU open-addressing hash compacted on the host
// (visibility_resolve.comp:52-72, facetrt_vulkan.cpp:1006-1037).  Here the
// pair keys are radix-sorted on the device, run-length counted, mirrored to
// directed entries and sorted again, so each CSR row comes out ordered by
// neighbour and the build is deterministic and needs no capacity guess.
#include "internal.h"

namespace facetcu {
namespace {

__global__ void k_mark_heads(const uint64_t* keys, size_t n, uint32_t* heads)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    heads[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

__global__ void k_compact_heads(const uint64_t* keys, size_t n, const uint32_t* heads,
                                const uint32_t* index, uint64_t* ukeys, uint32_t* upos)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (heads[i]) {
        ukeys[index[i]] = keys[i];
        upos[index[i]] = uint32_t(i);
    }
}

// Directed entries 2u, 2u+1 of undirected edge u: (lo -> hi) and (hi -> lo)
// with the run length as value.
__global__ void k_mirror(const uint64_t* ukeys, const uint32_t* upos, size_t u, size_t n,
                         int side_bits, uint64_t* dkeys, uint32_t* dvals)
{
    const size_t j = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= u) return;
    const uint64_t mask = (1ull << side_bits) - 1ull;
    const uint64_t lo = ukeys[j] >> side_bits, hi = ukeys[j] & mask;
    const uint32_t count = (j + 1 < u ? upos[j + 1] : uint32_t(n)) - upos[j];
    dkeys[2 * j] = (lo << side_bits) | hi;
    dkeys[2 * j + 1] = (hi << side_bits) | lo;
    dvals[2 * j] = count;
    dvals[2 * j + 1] = count;
}

__global__ void k_csr_fill(const uint64_t* dkeys, const uint32_t* dvals, size_t n, int side_bits,
                           uint32_t surfaces, uint32_t* row_offsets, facetcu_csr_edge* edges)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i > n) return;
    const uint64_t mask = (1ull << side_bits) - 1ull;
    // row boundaries: rows (prev, cur] start at i
    const int64_t prev = i == 0 ? -1 : int64_t(dkeys[i - 1] >> side_bits);
    const int64_t cur = i == n ? int64_t(surfaces) : int64_t(dkeys[i] >> side_bits);
    for (int64_t r = prev + 1; r <= cur; ++r) row_offsets[r] = uint32_t(i);
    if (i < n) {
        edges[i].neighbor = uint32_t(dkeys[i] & mask);
        edges[i].count = dvals[i];
    }
}

// Closure diagnostic of buildCpuGraph / buildVisibilityGraph
// (facetrtcore.cpp:1414-1426, facetrt_vulkan.cpp:1042-1056).
__global__ void k_closure(const uint32_t* row_offsets, const facetcu_csr_edge* edges,
                          const uint32_t* denom, const uint32_t* sky, uint32_t surfaces,
                          uint32_t* closure_bits, uint32_t* sampled, uint32_t* max_count)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= surfaces) return;
    unsigned long long visible = sky[s];
    uint32_t mc = 0;
    for (uint32_t e = row_offsets[s]; e < row_offsets[s + 1]; ++e) {
        visible += edges[e].count;
        mc = max(mc, edges[e].count);
    }
    if (mc) atomicMax(max_count, mc);
    if (denom[s] == 0u) return;
    atomicAdd(sampled, 1u);
    const float c = __ull2float_rn(visible) / __uint2float_rn(denom[s]);
    atomicMax(closure_bits, __float_as_uint(fabsf(c - 1.0f)));
}

__global__ void k_pack(const facetcu_csr_edge* edges, size_t n, uint32_t nb_bits,
                       uint32_t* packed)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    packed[i] = edges[i].neighbor | (edges[i].count << nb_bits);
}

inline unsigned grid(size_t n, unsigned b) { return unsigned((n + b - 1) / b); }

// One scene's rows and edges into a block-diagonal union graph.
__global__ void k_append_rows(const uint32_t* rows, uint32_t S, uint64_t edge_offset,
                              uint32_t* dst)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < S) dst[i] = uint32_t(rows[i] + edge_offset);
}
__global__ void k_append_edges(const facetcu_csr_edge* edges, size_t n, uint32_t side_offset,
                               facetcu_csr_edge* dst)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = {edges[i].neighbor + side_offset, edges[i].count};
}

}  // namespace

void graph_append(DeviceGraph& dst, const DeviceGraph& src, uint32_t side_offset,
                  uint64_t edge_offset, cudaStream_t s)
{
    const uint32_t S = src.surfaces;
    if (!S) return;
    k_append_rows<<<grid(S, 256), 256, 0, s>>>(src.row_offsets.as<uint32_t>(), S, edge_offset,
                                                dst.row_offsets.as<uint32_t>() + side_offset);
    FCU_LAUNCH("k_append_rows");
    if (src.nnz) {
        k_append_edges<<<grid(src.nnz, 256), 256, 0, s>>>(
            src.edges.as<facetcu_csr_edge>(), src.nnz, side_offset,
            dst.edges.as<facetcu_csr_edge>() + edge_offset);
        FCU_LAUNCH("k_append_edges");
    }
    FCU_CHECK(cudaMemcpyAsync(dst.denominators.as<uint32_t>() + side_offset,
                              src.denominators.ptr, size_t(S) * 4, cudaMemcpyDeviceToDevice, s));
    FCU_CHECK(cudaMemcpyAsync(dst.sky.as<uint32_t>() + side_offset, src.sky.ptr, size_t(S) * 4,
                              cudaMemcpyDeviceToDevice, s));
}

void graph_from_pairs(uint64_t* d_pairs, size_t n, int side_bits, DeviceGraph& g, Workspace& ws,
                      cudaStream_t s)
{
    const uint32_t S = g.surfaces;
    uint64_t* keys = d_pairs;
    uint64_t* alt = static_cast<uint64_t*>(ws.a.reserve((n + 1) * 8));
    uint32_t* nov = nullptr;
    uint32_t* nov2 = nullptr;
    radix_sort_u64(keys, alt, nov, nov2, n, 2 * side_bits, ws, s);
    // keys now holds the sorted pairs (either d_pairs or ws.a); use the other
    // buffer for the unique keys.
    uint64_t* other = keys == d_pairs ? alt : d_pairs;
    uint32_t* heads = static_cast<uint32_t*>(ws.b.reserve((n + 1) * 4 * 2));
    uint32_t* index = heads + (n + 1);
    size_t u = 0;
    if (n) {
        k_mark_heads<<<grid(n, 256), 256, 0, s>>>(keys, n, heads);
        FCU_LAUNCH("k_mark_heads");
        unsigned long long* dtotal = static_cast<unsigned long long*>(ws.e.reserve(64));
        exclusive_scan_u32(heads, index, n, dtotal, ws, s);
        unsigned long long total = 0;
        FCU_CHECK(cudaMemcpyAsync(&total, dtotal, 8, cudaMemcpyDeviceToHost, s));
        FCU_CHECK(cudaStreamSynchronize(s));
        u = size_t(total);
    }
    // unique keys go to `other`, their run starts reuse `heads` storage after compaction
    DeviceBuffer upos_buf;
    uint32_t* upos = static_cast<uint32_t*>(upos_buf.reserve((u + 1) * 4));
    if (n) {
        k_compact_heads<<<grid(n, 256), 256, 0, s>>>(keys, n, heads, index, other, upos);
        FCU_LAUNCH("k_compact_heads");
    }
    const size_t m = 2 * u;
    if (m >= (1ull << 32)) throw Error(FACETCU_OVERFLOW_ERROR, "visibility graph exceeds 2^32 edges");
    DeviceBuffer dk, dk2, dv, dv2;
    uint64_t* dkeys = static_cast<uint64_t*>(dk.reserve((m + 1) * 8));
    uint64_t* dkeys2 = static_cast<uint64_t*>(dk2.reserve((m + 1) * 8));
    uint32_t* dvals = static_cast<uint32_t*>(dv.reserve((m + 1) * 4));
    uint32_t* dvals2 = static_cast<uint32_t*>(dv2.reserve((m + 1) * 4));
    if (u) {
        k_mirror<<<grid(u, 256), 256, 0, s>>>(other, upos, u, n, side_bits, dkeys, dvals);
        FCU_LAUNCH("k_mirror");
        radix_sort_u64(dkeys, dkeys2, dvals, dvals2, m, 2 * side_bits, ws, s);
    }
    g.nnz = m;
    uint32_t* rows = static_cast<uint32_t*>(g.row_offsets.reserve((size_t(S) + 1) * 4));
    facetcu_csr_edge* edges = static_cast<facetcu_csr_edge*>(g.edges.reserve((m + 1) * 8));
    k_csr_fill<<<grid(m + 1, 256), 256, 0, s>>>(dkeys, dvals, m, side_bits, S, rows, edges);
    FCU_LAUNCH("k_csr_fill");
    FCU_CHECK(cudaStreamSynchronize(s));
    g.packed_valid = false;
    g.perm_valid = false;
    g.scene_facets.clear();
}

void graph_closure(const DeviceGraph& g, float* closure, uint32_t* sampled, Workspace& ws,
                   cudaStream_t s)
{
    uint32_t* d = static_cast<uint32_t*>(ws.e.reserve(64));
    FCU_CHECK(cudaMemsetAsync(d, 0, 16, s));
    if (g.surfaces) {
        k_closure<<<grid(g.surfaces, 256), 256, 0, s>>>(
            g.row_offsets.as<uint32_t>(), g.edges.as<facetcu_csr_edge>(),
            g.denominators.as<uint32_t>(), g.sky.as<uint32_t>(), g.surfaces, d, d + 1, d + 2);
        FCU_LAUNCH("k_closure");
    }
    uint32_t h[3];
    FCU_CHECK(cudaMemcpyAsync(h, d, 12, cudaMemcpyDeviceToHost, s));
    FCU_CHECK(cudaStreamSynchronize(s));
    std::memcpy(closure, &h[0], 4);
    *sampled = h[1];
    const_cast<DeviceGraph&>(g).max_count = h[2];
}

bool graph_pack(DeviceGraph& g, Workspace& ws, cudaStream_t s)
{
    (void)ws;
    if (g.packed_valid) return true;
    g.perm_valid = false;
    // neighbour in the low nb_bits (at least 22), count above: exact while the
    // largest count fits the remaining bits (1023 up to 2^22 sides, 511 up
    // to 2^23, 255 up to 2^24); otherwise the 8-byte edges are used
    uint32_t bits = 22;
    while (bits < 25 && (1u << bits) < g.surfaces) ++bits;
    if ((1u << bits) < g.surfaces || bits > 24 || g.max_count >= (1u << (32 - bits))) return false;
    g.nb_bits = bits;
    uint32_t* p = static_cast<uint32_t*>(g.packed.reserve((g.nnz + 1) * 4));
    if (g.nnz) {
        k_pack<<<grid(g.nnz, 256), 256, 0, s>>>(g.edges.as<facetcu_csr_edge>(), g.nnz, bits, p);
        FCU_LAUNCH("k_pack");
    }
    g.packed_valid = true;
    return true;
}

}  // namespace facetcu
