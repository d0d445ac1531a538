// raster.cu — global-line visibility: orthographic A-buffer raster of every
// facet along each direction, per-pixel depth chains, pair emission.
//
// Semantics are those of the reference's CPU backend (CpuRasterizer,
// buildCpuGraph, computeCpuSunlit: facetrtcore.cpp:1212-1474) so that the
// integer counts are identical:
//   * the projection, edge functions and interpolated depth use the same
//     float expressions in the same order; this file is compiled with
//     -fmad=false so no multiply-add is fused, as in the reference build;
//   * coverage is the inclusive edge test at pixel centres (:1315-1318);
//   * fragments of a pixel are ordered as std::sort (GCC's introsort)
//     orders them when given the reference's append order (tile-major,
//     then facet index): chains of <= 16 are stably sorted by depth, longer
//     chains replay the introsort step for step.
//
// GB300 layout: instead of a fixed W x H x L A-buffer (512 MB per direction
// at 1024^2 x 64) the raster runs twice — count, exclusive scan, fill — into
// exact-size per-pixel lists for a whole chunk of directions at once, so a
// single launch covers all 40 directions and HBM holds only real fragments.
#include "internal.h"

namespace facetcu {
namespace {

constexpr uint32_t kBigPixels = 1024;  // bbox area above which a CTA takes the triangle
constexpr uint32_t kFastChain = 64;    // per-thread chain capacity of the main resolve
constexpr uint32_t kDeepChain = 1024;  // capacity of the deep-chain resolve
constexpr uint32_t kKeyMask = 0x7fffffffu;

__constant__ RasterView c_views[64];
__constant__ RasterFrame c_frame;

struct Projected {
    float x[3], y[3], d[3];
};

__device__ __forceinline__ float dot3(const float a[3], float b0, float b1, float b2)
{
    return a[0] * b0 + a[1] * b1 + a[2] * b2;
}

// facetrtcore.cpp:1259-1275
__device__ __forceinline__ void project(const facetcu_vertex* V, uint32_t f, uint32_t tile,
                                        const RasterView& v, Projected& p, uint32_t& flip)
{
    const float ox = c_frame.tile_dx[tile], oz = c_frame.tile_dz[tile];
    const float r = c_frame.radius;
    const float w = float(c_frame.width), h = float(c_frame.height);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const facetcu_vertex& vx = V[3 * f + c];
        const float rx = (vx.position[0] + ox) - c_frame.center[0];
        const float ry = vx.position[1] - c_frame.center[1];
        const float rz = (vx.position[2] + oz) - c_frame.center[2];
        p.x[c] = (0.5f + 0.5f * dot3(v.right, rx, ry, rz) / r) * w;
        p.y[c] = (0.5f + 0.5f * dot3(v.up, rx, ry, rz) / r) * h;
        p.d[c] = 0.5f - dot3(v.view, rx, ry, rz) / (2.0f * r);
    }
    const facetcu_vertex& v0 = V[3 * f];
    flip = dot3(v.view, v0.normal[0], v0.normal[1], v0.normal[2]) >= 0.0f ? 0u : 1u;
}

// edge() of facetrtcore.cpp:1287-1290, argument order kept.
__device__ __forceinline__ float edgef(float ax, float ay, float bx, float by, float px, float py)
{
    return (px - ax) * (by - ay) - (py - ay) * (bx - ax);
}

__device__ __forceinline__ float min3(float a, float b, float c)
{
    float m = a;
    if (b < m) m = b;
    if (c < m) m = c;
    return m;
}
__device__ __forceinline__ float max3(float a, float b, float c)
{
    float m = a;
    if (m < b) m = b;
    if (m < c) m = c;
    return m;
}

struct Bbox {
    int x0, x1, y0, y1;
    float area;
    bool valid;
};

// facetrtcore.cpp:1292-1308
__device__ __forceinline__ Bbox triangle_bbox(const Projected& p)
{
    Bbox b;
    b.area = edgef(p.x[0], p.y[0], p.x[1], p.y[1], p.x[2], p.y[2]);
    b.valid = !(fabsf(b.area) < 1.0e-8f);
    b.x0 = max(0, int(floorf(min3(p.x[0], p.x[1], p.x[2]))));
    b.x1 = min(int(c_frame.width) - 1, int(ceilf(max3(p.x[0], p.x[1], p.x[2]))));
    b.y0 = max(0, int(floorf(min3(p.y[0], p.y[1], p.y[2]))));
    b.y1 = min(int(c_frame.height) - 1, int(ceilf(max3(p.y[0], p.y[1], p.y[2]))));
    if (b.x1 < b.x0 || b.y1 < b.y0) b.valid = false;
    return b;
}

// Inclusive coverage and depth at one pixel centre (facetrtcore.cpp:1309-1332).
__device__ __forceinline__ bool cover(const Projected& p, float area, int x, int y, float& depth)
{
    const float px = float(x) + 0.5f;
    const float py = float(y) + 0.5f;
    const float w0 = edgef(p.x[1], p.y[1], p.x[2], p.y[2], px, py);
    const float w1 = edgef(p.x[2], p.y[2], p.x[0], p.y[0], px, py);
    const float w2 = edgef(p.x[0], p.y[0], p.x[1], p.y[1], px, py);
    const bool inside = area > 0.0f ? (w0 >= 0.0f && w1 >= 0.0f && w2 >= 0.0f)
                                    : (w0 <= 0.0f && w1 <= 0.0f && w2 <= 0.0f);
    if (!inside) return false;
    const float inv = 1.0f / area;
    depth = (w0 * p.d[0] + w1 * p.d[1] + w2 * p.d[2]) * inv;
    return true;
}

struct ItemRef {
    uint32_t dir, tile, facet;
};

__device__ __forceinline__ ItemRef decode_item(uint64_t w)
{
    const uint64_t per_dir = uint64_t(c_frame.tiles) * c_frame.facets;
    ItemRef r;
    r.dir = uint32_t(w / per_dir);
    const uint64_t rem = w - uint64_t(r.dir) * per_dir;
    r.tile = uint32_t(rem / c_frame.facets);
    r.facet = uint32_t(rem - uint64_t(r.tile) * c_frame.facets);
    return r;
}

// Count (kFill = false) or fill (kFill = true) the fragments of one
// triangle; big triangles are queued for the CTA kernel in the count pass.
template <bool kFill>
__global__ void __launch_bounds__(256) k_raster_small(const facetcu_vertex* V, uint64_t items,
                                                      uint32_t* counts, const uint32_t* offsets,
                                                      uint64_t* records, uint32_t* big_list,
                                                      uint32_t* big_count)
{
    const uint64_t w = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (w >= items) return;
    const ItemRef it = decode_item(w);
    Projected p;
    uint32_t flip;
    project(V, it.facet, it.tile, c_views[it.dir], p, flip);
    const Bbox b = triangle_bbox(p);
    if (!b.valid) return;
    const uint32_t area_px = uint32_t(b.x1 - b.x0 + 1) * uint32_t(b.y1 - b.y0 + 1);
    if (area_px > kBigPixels) {
        if (!kFill) big_list[atomicAdd(big_count, 1u)] = uint32_t(w);
        return;
    }
    const size_t plane = size_t(it.dir) * c_frame.width * c_frame.height;
    const uint32_t key = (it.tile * c_frame.facets + it.facet) | (flip << 31);
    for (int y = b.y0; y <= b.y1; ++y) {
        for (int x = b.x0; x <= b.x1; ++x) {
            float depth;
            if (!cover(p, b.area, x, y, depth)) continue;
            const size_t pix = plane + size_t(y) * c_frame.width + size_t(x);
            if (!kFill) {
                atomicAdd(&counts[pix], 1u);
            } else {
                const uint32_t slot = offsets[pix] + atomicAdd(&counts[pix], 1u);
                records[slot] = (uint64_t(__float_as_uint(depth)) << 32) | key;
            }
        }
    }
}

template <bool kFill>
__global__ void __launch_bounds__(256) k_raster_big(const facetcu_vertex* V,
                                                    const uint32_t* big_list, uint32_t* counts,
                                                    const uint32_t* offsets, uint64_t* records)
{
    const uint64_t w = big_list[blockIdx.x];
    const ItemRef it = decode_item(w);
    Projected p;
    uint32_t flip;
    project(V, it.facet, it.tile, c_views[it.dir], p, flip);
    const Bbox b = triangle_bbox(p);
    const uint32_t bw = uint32_t(b.x1 - b.x0 + 1), bh = uint32_t(b.y1 - b.y0 + 1);
    const size_t plane = size_t(it.dir) * c_frame.width * c_frame.height;
    const uint32_t key = (it.tile * c_frame.facets + it.facet) | (flip << 31);
    for (uint32_t i = threadIdx.x; i < bw * bh; i += blockDim.x) {
        const int x = b.x0 + int(i % bw), y = b.y0 + int(i / bw);
        float depth;
        if (!cover(p, b.area, x, y, depth)) continue;
        const size_t pix = plane + size_t(y) * c_frame.width + size_t(x);
        if (!kFill) {
            atomicAdd(&counts[pix], 1u);
        } else {
            const uint32_t slot = offsets[pix] + atomicAdd(&counts[pix], 1u);
            records[slot] = (uint64_t(__float_as_uint(depth)) << 32) | key;
        }
    }
}

// ---- per-pixel ordering ------------------------------------------------------
struct Frag {
    float depth;
    uint32_t key;  // append order | flip << 31
};

__device__ __forceinline__ bool frag_less(const Frag& a, const Frag& b) { return a.depth < b.depth; }

__device__ __forceinline__ bool frag_less_stable(const Frag& a, const Frag& b)
{
    return a.depth < b.depth || (a.depth == b.depth && (a.key & kKeyMask) < (b.key & kKeyMask));
}

__device__ void sort_by_append_order(Frag* f, int n)
{
    for (int i = 1; i < n; ++i) {
        const Frag v = f[i];
        int j = i;
        while (j > 0 && (f[j - 1].key & kKeyMask) > (v.key & kKeyMask)) {
            f[j] = f[j - 1];
            --j;
        }
        f[j] = v;
    }
}

// GCC libstdc++ std::sort, restated (see the oracle for the same steps):
// introsort with median-of-three, unguarded partition, heap-sort fallback at
// depth 2*floor(log2 n), final insertion sort with threshold 16.
// The bounds checks below never trigger when the introsort invariants hold
// (a smaller-or-equal element precedes every unguarded insertion, the
// partition scans stop inside the range); they only keep a wrong input from
// walking out of the local array.
__device__ void unguarded_linear_insert(Frag* f, int last)
{
    const Frag v = f[last];
    int next = last - 1;
    while (next >= 0 && frag_less(v, f[next])) {
        f[last] = f[next];
        last = next;
        --next;
    }
    f[last] = v;
}

__device__ void insertion_sort(Frag* f, int first, int last)
{
    if (first == last) return;
    for (int i = first + 1; i != last; ++i) {
        if (frag_less(f[i], f[first])) {
            const Frag v = f[i];
            for (int k = i; k > first; --k) f[k] = f[k - 1];
            f[first] = v;
        } else {
            unguarded_linear_insert(f, i);
        }
    }
}

__device__ void adjust_heap(Frag* first, int hole, int len, Frag value)
{
    const int top = hole;
    int child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (frag_less(first[child], first[child - 1])) child--;
        first[hole] = first[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        first[hole] = first[child - 1];
        hole = child - 1;
    }
    int parent = (hole - 1) / 2;
    while (hole > top && frag_less(first[parent], value)) {
        first[hole] = first[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    first[hole] = value;
}

__device__ void heap_sort(Frag* first, int len)
{
    if (len >= 2) {
        int parent = (len - 2) / 2;
        for (;;) {
            adjust_heap(first, parent, len, first[parent]);
            if (parent == 0) break;
            parent--;
        }
    }
    while (len > 1) {
        --len;
        const Frag v = first[len];
        first[len] = first[0];
        adjust_heap(first, 0, len, v);
    }
}

__device__ __forceinline__ void fswap(Frag& a, Frag& b)
{
    const Frag t = a;
    a = b;
    b = t;
}

__device__ void median_to_first(Frag* f, int result, int a, int b, int c)
{
    if (frag_less(f[a], f[b])) {
        if (frag_less(f[b], f[c])) fswap(f[result], f[b]);
        else if (frag_less(f[a], f[c])) fswap(f[result], f[c]);
        else fswap(f[result], f[a]);
    } else if (frag_less(f[a], f[c])) fswap(f[result], f[a]);
    else if (frag_less(f[b], f[c])) fswap(f[result], f[c]);
    else fswap(f[result], f[b]);
}

__device__ int unguarded_partition(Frag* f, int first, int last, int pivot)
{
    const int lo = first, hi = last;
    for (;;) {
        while (first < hi - 1 && frag_less(f[first], f[pivot])) ++first;
        --last;
        while (last > lo && frag_less(f[pivot], f[last])) --last;
        if (!(first < last)) return first;
        fswap(f[first], f[last]);
        ++first;
    }
}

__device__ void std_sort_by_depth(Frag* f, int n)
{
    if (n <= 1) return;
    if (n <= 16) {
        insertion_sort(f, 0, n);
        return;
    }
    int lg = 0;
    while ((1 << (lg + 1)) <= n) ++lg;
    // introsort loop with an explicit stack of pending right-hand ranges
    int stack_first[64], stack_last[64], stack_depth[64];
    int sp = 0;
    stack_first[sp] = 0;
    stack_last[sp] = n;
    stack_depth[sp] = 2 * lg;
    ++sp;
    while (sp > 0) {
        --sp;
        const int first = stack_first[sp];
        int last = stack_last[sp];
        int depth = stack_depth[sp];
        // The recursion of the reference handles (cut, last) before the
        // left part; ranges are disjoint, so order between them does not
        // change the result.
        while (last - first > 16) {
            if (depth == 0) {
                heap_sort(f + first, last - first);
                break;
            }
            --depth;
            const int mid = first + (last - first) / 2;
            median_to_first(f, first, first + 1, mid, last - 1);
            const int cut = unguarded_partition(f, first + 1, last, first);
            if (sp < 64) {
                stack_first[sp] = cut;
                stack_last[sp] = last;
                stack_depth[sp] = depth;
                ++sp;
            }
            last = cut;
        }
    }
    insertion_sort(f, 0, 16);
    for (int i = 16; i < n; ++i) unguarded_linear_insert(f, i);
}

__device__ __forceinline__ void order_chain(Frag* f, int n)
{
    if (n <= 16) {
        // libstdc++ sorts <= 16 elements by insertion sort, which is stable:
        // the result is sorted by (depth, append order) whatever the load order.
        for (int i = 1; i < n; ++i) {
            const Frag v = f[i];
            int j = i;
            while (j > 0 && frag_less_stable(v, f[j - 1])) {
                f[j] = f[j - 1];
                --j;
            }
            f[j] = v;
        }
    } else {
        sort_by_append_order(f, n);
        std_sort_by_depth(f, n);
    }
}

__device__ __forceinline__ uint32_t frag_side(uint32_t key, uint32_t facets)
{
    const uint32_t order = key & kKeyMask;
    return 2u * (order % facets) + (key >> 31);
}

// Emit denominators, sky counts and adjacent pairs of an ordered chain
// (facetrtcore.cpp:1374-1392; visibility_resolve.comp:102-116).
__device__ void emit_chain(const Frag* f, int n, uint32_t facets, uint32_t* denom, uint32_t* sky,
                           uint64_t* pairs, unsigned long long* pair_count, int side_bits,
                           bool warp_aggregate)
{
    for (int i = 0; i < n; ++i) {
        const uint32_t s = frag_side(f[i].key, facets);
        atomicAdd(&denom[s], 1u);
        atomicAdd(&denom[s ^ 1u], 1u);
    }
    if (n > 0) {
        atomicAdd(&sky[frag_side(f[0].key, facets)], 1u);
        atomicAdd(&sky[frag_side(f[n - 1].key, facets) ^ 1u], 1u);
    }
    uint32_t np = 0;
    for (int i = 0; i + 1 < n; ++i) {
        const uint32_t a = frag_side(f[i].key, facets) ^ 1u;
        const uint32_t b = frag_side(f[i + 1].key, facets);
        if ((a >> 1) != (b >> 1)) ++np;
    }
    unsigned long long base = 0;
    if (warp_aggregate) {
        // called by all 32 lanes of the warp (threads without a chain pass n = 0)
        __syncwarp();
        const unsigned lane = threadIdx.x & 31u;
        unsigned incl = np;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= unsigned(o)) incl += y;
        }
        const unsigned total = __shfl_sync(0xffffffffu, incl, 31);
        unsigned long long b0 = 0;
        if (lane == 31u && total) b0 = atomicAdd(pair_count, (unsigned long long)total);
        b0 = __shfl_sync(0xffffffffu, b0, 31);
        base = b0 + (incl - np);
    } else if (np) {
        base = atomicAdd(pair_count, (unsigned long long)np);
    }
    uint32_t k = 0;
    for (int i = 0; i + 1 < n; ++i) {
        const uint32_t a = frag_side(f[i].key, facets) ^ 1u;
        const uint32_t b = frag_side(f[i + 1].key, facets);
        if ((a >> 1) == (b >> 1)) continue;
        const uint64_t lo = a < b ? a : b, hi = a < b ? b : a;
        pairs[base + k] = (lo << side_bits) | hi;
        ++k;
    }
}

__device__ __forceinline__ Frag unpack(uint64_t r)
{
    Frag f;
    f.depth = __uint_as_float(uint32_t(r >> 32));
    f.key = uint32_t(r);
    return f;
}

__global__ void __launch_bounds__(128) k_resolve_graph(
    const uint32_t* offsets, const uint64_t* records, uint64_t npix, uint32_t cap,
    uint32_t* denom, uint32_t* sky, uint64_t* pairs, unsigned long long* pair_count,
    int side_bits, uint32_t* deep_list, uint32_t* deep_count, RasterStats* stats)
{
    const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool valid = i < npix;
    uint32_t n = 0, start = 0;
    if (valid) {
        start = offsets[i];
        n = offsets[i + 1] - start;
    }
    if (valid && n > cap) atomicAdd(&stats->overflow, (unsigned long long)(n - cap));
    if (valid && n > 0) atomicMax(&stats->max_chain, n);
    if (valid && n > kFastChain) {
        deep_list[atomicAdd(deep_count, 1u)] = uint32_t(i);
        n = 0;
    }
    Frag f[kFastChain];
    for (uint32_t k = 0; k < n; ++k) f[k] = unpack(records[start + k]);
    order_chain(f, int(n));
    // every thread of the warp reaches the aggregated allocation
    emit_chain(f, int(n), c_frame.facets, denom, sky, pairs, pair_count, side_bits, true);
}

__global__ void __launch_bounds__(32) k_resolve_graph_deep(
    const uint32_t* offsets, const uint64_t* records, const uint32_t* deep_list,
    const uint32_t* deep_count, uint32_t* denom, uint32_t* sky, uint64_t* pairs,
    unsigned long long* pair_count, int side_bits, RasterStats* stats)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= *deep_count) return;
    const uint32_t i = deep_list[j];
    const uint32_t start = offsets[i];
    const uint32_t n = offsets[i + 1] - start;
    if (n > kDeepChain) {
        atomicAdd(&stats->capacity_error, 1u);
        return;
    }
    Frag f[kDeepChain];
    for (uint32_t k = 0; k < n; ++k) f[k] = unpack(records[start + k]);
    order_chain(f, int(n));
    emit_chain(f, int(n), c_frame.facets, denom, sky, pairs, pair_count, side_bits, false);
}

// computeCpuSunlit per pixel (facetrtcore.cpp:1448-1466): every fragment
// counts towards its side's total; the nearest (first in append order among
// equal depths) is visible.
__global__ void __launch_bounds__(256) k_resolve_sunlit(const uint32_t* offsets,
                                                        const uint64_t* records, uint64_t npix,
                                                        uint32_t cap, uint32_t* total,
                                                        uint32_t* visible, RasterStats* stats)
{
    const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    const uint32_t start = offsets[i];
    const uint32_t n = offsets[i + 1] - start;
    if (n == 0) return;
    if (n > cap) atomicAdd(&stats->overflow, (unsigned long long)(n - cap));
    atomicMax(&stats->max_chain, n);
    Frag best = unpack(records[start]);
    atomicAdd(&total[frag_side(best.key, c_frame.facets)], 1u);
    for (uint32_t k = 1; k < n; ++k) {
        const Frag f = unpack(records[start + k]);
        atomicAdd(&total[frag_side(f.key, c_frame.facets)], 1u);
        if (frag_less_stable(f, best)) best = f;
    }
    atomicAdd(&visible[frag_side(best.key, c_frame.facets)], 1u);
}

__global__ void k_set_last_offset(uint32_t* offsets, uint64_t n, const unsigned long long* total)
{
    offsets[n] = uint32_t(*total);
}

}  // namespace

void raster_fragments(const facetcu_vertex* d_vertices, const RasterFrame& frame,
                      const RasterView* views, uint32_t dir_count, RasterBuffers& rb,
                      Workspace& ws, RasterStats& stats, cudaStream_t s)
{
    if (dir_count > 64) throw Error(FACETCU_INVALID_ARGUMENT, "raster chunk exceeds 64 directions");
    FCU_CHECK(cudaMemcpyToSymbolAsync(c_views, views, sizeof(RasterView) * dir_count, 0,
                                      cudaMemcpyHostToDevice, s));
    FCU_CHECK(cudaMemcpyToSymbolAsync(c_frame, &frame, sizeof(RasterFrame), 0,
                                      cudaMemcpyHostToDevice, s));
    const uint64_t npix = uint64_t(dir_count) * frame.width * frame.height;
    const uint64_t items = uint64_t(dir_count) * frame.tiles * frame.facets;
    if (items >= (1ull << 32)) throw Error(FACETCU_OVERFLOW_ERROR, "raster work exceeds 2^32 triangles");
    uint32_t* counts = static_cast<uint32_t*>(rb.counts.reserve(npix * 4));
    uint32_t* offsets = static_cast<uint32_t*>(rb.offsets.reserve((npix + 1) * 4));
    uint32_t* big = static_cast<uint32_t*>(rb.big_list.reserve(items * 4));
    RasterStats* dstats = static_cast<RasterStats*>(rb.stats.reserve(sizeof(RasterStats) + 64));
    unsigned long long* dtotal = reinterpret_cast<unsigned long long*>(
        static_cast<char*>(rb.stats.ptr) + sizeof(RasterStats));
    FCU_CHECK(cudaMemsetAsync(counts, 0, npix * 4, s));
    FCU_CHECK(cudaMemsetAsync(dstats, 0, sizeof(RasterStats), s));
    const unsigned blocks = unsigned((items + 255) / 256);
    k_raster_small<false><<<blocks, 256, 0, s>>>(d_vertices, items, counts, nullptr, nullptr,
                                                 big, &dstats->big);
    FCU_LAUNCH("k_raster_small<count>");
    RasterStats host{};
    FCU_CHECK(cudaMemcpyAsync(&host, dstats, sizeof(RasterStats), cudaMemcpyDeviceToHost, s));
    FCU_CHECK(cudaStreamSynchronize(s));
    if (host.big) {
        k_raster_big<false><<<host.big, 256, 0, s>>>(d_vertices, big, counts, nullptr, nullptr);
        FCU_LAUNCH("k_raster_big<count>");
    }
    exclusive_scan_u32(counts, offsets, npix, dtotal, ws, s);
    unsigned long long total = 0;
    FCU_CHECK(cudaMemcpyAsync(&total, dtotal, 8, cudaMemcpyDeviceToHost, s));
    FCU_CHECK(cudaStreamSynchronize(s));
    if (total >= (1ull << 32))
        throw Error(FACETCU_OVERFLOW_ERROR, "more than 2^32 fragments in one raster chunk");
    k_set_last_offset<<<1, 1, 0, s>>>(offsets, npix, dtotal);
    FCU_LAUNCH("k_set_last_offset");
    uint64_t* records = static_cast<uint64_t*>(rb.records.reserve((total + 1) * 8));
    FCU_CHECK(cudaMemsetAsync(counts, 0, npix * 4, s));
    k_raster_small<true><<<blocks, 256, 0, s>>>(d_vertices, items, counts, offsets, records,
                                                nullptr, nullptr);
    FCU_LAUNCH("k_raster_small<fill>");
    if (host.big) {
        k_raster_big<true><<<host.big, 256, 0, s>>>(d_vertices, big, counts, offsets, records);
        FCU_LAUNCH("k_raster_big<fill>");
    }
    stats.fragments = total;
    stats.big = host.big;
}

void raster_resolve_graph(const RasterFrame& frame, uint32_t dir_count, uint32_t chain_cap,
                          RasterBuffers& rb, uint32_t* d_denominators, uint32_t* d_sky,
                          uint64_t* d_pairs, unsigned long long* d_pair_count, int side_bits,
                          RasterStats& stats, cudaStream_t s)
{
    const uint64_t npix = uint64_t(dir_count) * frame.width * frame.height;
    RasterStats* dstats = rb.stats.as<RasterStats>();
    uint32_t* deep = static_cast<uint32_t*>(rb.deep_list.reserve(npix * 4));
    FCU_CHECK(cudaMemsetAsync(&dstats->deep, 0, 4, s));
    k_resolve_graph<<<unsigned((npix + 127) / 128), 128, 0, s>>>(
        rb.offsets.as<uint32_t>(), rb.records.as<uint64_t>(), npix, chain_cap,
        d_denominators, d_sky, d_pairs, d_pair_count, side_bits, deep, &dstats->deep, dstats);
    FCU_LAUNCH("k_resolve_graph");
    RasterStats host{};
    FCU_CHECK(cudaMemcpyAsync(&host, dstats, sizeof(RasterStats), cudaMemcpyDeviceToHost, s));
    FCU_CHECK(cudaStreamSynchronize(s));
    if (host.deep) {
        k_resolve_graph_deep<<<(host.deep + 31) / 32, 32, 0, s>>>(
            rb.offsets.as<uint32_t>(), rb.records.as<uint64_t>(), deep, &dstats->deep,
            d_denominators, d_sky, d_pairs, d_pair_count, side_bits, dstats);
        FCU_LAUNCH("k_resolve_graph_deep");
        FCU_CHECK(cudaMemcpyAsync(&host, dstats, sizeof(RasterStats), cudaMemcpyDeviceToHost, s));
        FCU_CHECK(cudaStreamSynchronize(s));
    }
    stats.overflow = host.overflow;
    stats.deep = host.deep;
    stats.max_chain = host.max_chain;
    stats.capacity_error = host.capacity_error;
}

void raster_resolve_sunlit(const RasterFrame& frame, uint32_t chain_cap, RasterBuffers& rb,
                           uint32_t* d_total, uint32_t* d_visible, RasterStats& stats,
                           cudaStream_t s)
{
    const uint64_t npix = uint64_t(frame.width) * frame.height;
    RasterStats* dstats = rb.stats.as<RasterStats>();
    k_resolve_sunlit<<<unsigned((npix + 255) / 256), 256, 0, s>>>(
        rb.offsets.as<uint32_t>(), rb.records.as<uint64_t>(), npix, chain_cap,
        d_total, d_visible, dstats);
    FCU_LAUNCH("k_resolve_sunlit");
    RasterStats host{};
    FCU_CHECK(cudaMemcpyAsync(&host, dstats, sizeof(RasterStats), cudaMemcpyDeviceToHost, s));
    FCU_CHECK(cudaStreamSynchronize(s));
    stats.overflow = host.overflow;
    stats.max_chain = host.max_chain;
}

}  // namespace facetcu
