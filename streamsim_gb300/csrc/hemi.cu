// hemi.cu — hemisphere ray-cast view factors and sun visibility over the LBVH.
//
// For every oriented side s (facet f = s / 2, normal N = +/- n_f) a warp
// casts `rays` rays: ray j of sample set (s mod sets) starts at
// a + u (b - a) + v (c - a) and leaves along T dx + Bt dy + N dz in the side's
// frame (T = normalize(helper x N), Bt = N x T).  A facet is hit when the
// Moller-Trumbore test accepts the ray at t > 0 and o + t d lies in the
// facet's box widened by the hit margin (the test's distance to a long thin
// facet met at a grazing angle can lie millimetres outside the facet; the
// BVH's leaf boxes are widened by twice the margin, so the traversal never
// culls a hit).  The nearest hit (smallest t, ties to the lower facet
// index, the origin facet skipped) gives the side seen: 2g if the ray
// meets g's normal side, 2g + 1 otherwise.  The warp
// sorts the 32 x (rays/32) hit ids in shared memory, counts runs, keeps the
// top_k most-hit sides (ties: lower side index) and writes the row sorted
// by neighbour with denominator = kept + sky rays.  With periodic tiles the
// nearest hit is taken over the scene and its copies (see Tiles).  Exactly
// the rules of the C oracle (orc_hemisphere_graph_periodic), so counts are
// comparable bit for bit.
// This file is compiled with -fmad=false: the origin, direction and
// Moller-Trumbore arithmetic round like the oracle's.
#include <cfloat>

#include "internal.h"

namespace facetcu {
namespace {

constexpr int kWarps = 8;
constexpr uint32_t kSky = 0xFFFFFFFFu;
constexpr int kStack = 64;

struct Vec {
    float x, y, z;
};

__device__ __forceinline__ Vec vsub(Vec a, Vec b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ float vdot(Vec a, Vec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ Vec vcross(Vec a, Vec b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ Vec pos(const facetcu_vertex& v)
{
    return {v.position[0], v.position[1], v.position[2]};
}

// Moller-Trumbore, the oracle's ray_triangle: t, or -1.
__device__ __forceinline__ float ray_triangle(Vec o, Vec d, Vec a, Vec e1, Vec e2)
{
    const Vec p = vcross(d, e2);
    const float det = vdot(e1, p);
    if (det == 0.0f) return -1.0f;
    const float inv = 1.0f / det;
    const Vec t0 = vsub(o, a);
    const float u = vdot(t0, p) * inv;
    if (u < 0.0f || u > 1.0f) return -1.0f;
    const Vec q = vcross(t0, e1);
    const float v = vdot(d, q) * inv;
    if (v < 0.0f || u + v > 1.0f) return -1.0f;
    const float t = vdot(e2, q) * inv;
    return t > 0.0f ? t : -1.0f;
}

__device__ __forceinline__ bool slab(const float4& lo, const float4& hi, Vec o, Vec inv, float tmax,
                                     float& tnear)
{
    const float tx0 = (lo.x - o.x) * inv.x, tx1 = (hi.x - o.x) * inv.x;
    const float ty0 = (lo.y - o.y) * inv.y, ty1 = (hi.y - o.y) * inv.y;
    const float tz0 = (lo.z - o.z) * inv.z, tz1 = (hi.z - o.z) * inv.z;
    const float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
    const float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
    tnear = tn;
    return tn <= tf && tn <= tmax;
}

// 1/d with |d| raised to at least 1e-30: the slab distances stay finite (no
// infinity, so no 0 * inf), and fminf/fmaxf order them.
__device__ __forceinline__ float safe_inv(float d)
{
    return 1.0f / (fabsf(d) < 1.0e-30f ? copysignf(1.0e-30f, d) : d);
}

// o + t d inside facet g's box widened by m (the hit rule's second half).
__device__ __forceinline__ bool in_hit_box(const facetcu_vertex* __restrict__ V, uint32_t g,
                                           Vec o, Vec d, float t, float m)
{
    const float p[3] = {o.x + t * d.x, o.y + t * d.y, o.z + t * d.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float v0 = V[3 * g].position[a], v1 = V[3 * g + 1].position[a],
                    v2 = V[3 * g + 2].position[a];
        const float lo = fminf(v0, fminf(v1, v2)) - m, hi = fmaxf(v0, fmaxf(v1, v2)) + m;
        if (!(p[a] >= lo && p[a] <= hi)) return false;
    }
    return true;
}

struct Hit {
    float t;
    uint32_t facet;
};

// Nearest hit (any_hit = false) or occlusion (any_hit = true) over the LBVH,
// improving on `best` (callers start it at {FLT_MAX, kSky}; periodic tiles
// carry it from tile to tile).  Returns false when the traversal stack
// overflowed.
template <bool kAny>
__device__ bool trace(const float4* __restrict__ nodes, const float4* __restrict__ tri,
                      const facetcu_vertex* __restrict__ V, float m, uint32_t leaves, Vec o,
                      Vec d, uint32_t skip, Hit& best)
{
    const Vec inv = {safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
    auto test_leaf = [&](uint32_t k) {
        const float4 A = __ldg(tri + 3 * size_t(k));
        const uint32_t g = __float_as_uint(A.w);
        if (g == skip) return;
        const float4 E1 = __ldg(tri + 3 * size_t(k) + 1);
        const float4 E2 = __ldg(tri + 3 * size_t(k) + 2);
        const float t = ray_triangle(o, d, {A.x, A.y, A.z}, {E1.x, E1.y, E1.z}, {E2.x, E2.y, E2.z});
        if (t > 0.0f && (t < best.t || (t == best.t && g < best.facet)) &&
            in_hit_box(V, g, o, d, t, m)) {
            best.t = t;
            best.facet = g;
        }
    };
    if (leaves == 1) {
        test_leaf(0);
        return true;
    }
    int stack[kStack];
    int sp = 0;
    int node = 0;
    while (true) {
        const float4 lo0 = __ldg(nodes + 4 * size_t(node));
        const float4 hi0 = __ldg(nodes + 4 * size_t(node) + 1);
        const float4 lo1 = __ldg(nodes + 4 * size_t(node) + 2);
        const float4 hi1 = __ldg(nodes + 4 * size_t(node) + 3);
        const int c0 = __float_as_int(lo0.w), c1 = __float_as_int(lo1.w);
        float n0, n1;
        bool h0 = slab(lo0, hi0, o, inv, best.t, n0);
        bool h1 = slab(lo1, hi1, o, inv, best.t, n1);
        if (h0 && c0 < 0) {
            test_leaf(uint32_t(~c0));
            h0 = false;
            if (kAny && best.facet != kSky) return true;
        }
        if (h1 && c1 < 0) {
            test_leaf(uint32_t(~c1));
            h1 = false;
            if (kAny && best.facet != kSky) return true;
        }
        if (h0 && h1) {
            const int first = n0 <= n1 ? c0 : c1, second = n0 <= n1 ? c1 : c0;
            if (sp >= kStack) return false;
            stack[sp++] = second;
            node = first;
            continue;
        }
        if (h0) { node = c0; continue; }
        if (h1) { node = c1; continue; }
        if (sp == 0) break;
        node = stack[--sp];
    }
    return true;
}

struct Frame {
    Vec N, T, B;
};

// Periodic tiles (the raster mode's: the scene plus up to 20 copies offset by
// periodicTileOffset(t) x (periodicSizeX, periodicSizeZ)).  A copy is met by
// shifting the ray origin back by the tile's offset; the hit names the
// original facet; the origin facet is skipped in the scene's own tile only.
struct Tiles {
    float x[21], z[21];
    uint32_t n;
};

template <bool kAny>
__device__ bool trace_tiles(const float4* __restrict__ nodes, const float4* __restrict__ tri,
                            const facetcu_vertex* __restrict__ V, float m, uint32_t leaves,
                            const Tiles& tiles, Vec o, Vec d, uint32_t skip, Hit& best)
{
    best.t = FLT_MAX;
    best.facet = kSky;
    if (tiles.n <= 1) return trace<kAny>(nodes, tri, V, m, leaves, o, d, skip, best);  // no copies
    bool ok = true;
    for (uint32_t t = 0; t < tiles.n; ++t) {
        const Vec ot = {o.x - tiles.x[t], o.y, o.z - tiles.z[t]};
        ok &= trace<kAny>(nodes, tri, V, m, leaves, ot, d, t == 0 ? skip : kSky, best);
        if (kAny && best.facet != kSky) break;
    }
    return ok;
}

// The oracle's side_frame: helper = |N.y| < 0.9 ? +Y : +X.
__device__ __forceinline__ Frame side_frame(const facetcu_vertex* V, uint32_t s)
{
    const uint32_t f = s >> 1;
    Vec N = {V[3 * f].normal[0], V[3 * f].normal[1], V[3 * f].normal[2]};
    if (s & 1u) N = {-N.x, -N.y, -N.z};
    const Vec helper = fabsf(N.y) < 0.9f ? Vec{0.0f, 1.0f, 0.0f} : Vec{1.0f, 0.0f, 0.0f};
    const Vec t = vcross(helper, N);
    const float len = sqrtf(vdot(t, t));
    const float il = 1.0f / len;
    Frame fr;
    fr.N = N;
    fr.T = {t.x * il, t.y * il, t.z * il};
    fr.B = vcross(N, fr.T);
    return fr;
}

__device__ __forceinline__ Vec sample_origin(const facetcu_vertex* V, uint32_t f, float u, float v)
{
    const Vec a = pos(V[3 * f]);
    const Vec e1 = vsub(pos(V[3 * f + 1]), a);
    const Vec e2 = vsub(pos(V[3 * f + 2]), a);
    return {(a.x + e1.x * u) + e2.x * v, (a.y + e1.y * u) + e2.y * v, (a.z + e1.z * u) + e2.z * v};
}

__device__ void warp_bitonic(uint32_t* a, int n, int lane)
{
    for (int k = 2; k <= n; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < n; i += 32) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const uint32_t x = a[i], y = a[ixj];
                    const bool up = (i & k) == 0;
                    if ((x > y) == up) {
                        a[i] = y;
                        a[ixj] = x;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// Warp-wide exclusive prefix sum of per-lane values.
__device__ __forceinline__ uint32_t warp_exclusive(uint32_t v, int lane, uint32_t& total)
{
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    total = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
}

__global__ void __launch_bounds__(kWarps * 32) k_hemi_rows(
    const facetcu_vertex* __restrict__ V, const float4* __restrict__ nodes,
    const float4* __restrict__ tri, uint32_t leaves, uint32_t surfaces, const float* __restrict__ uv,
    const float* __restrict__ dirs, uint32_t rays, uint32_t sets, uint32_t npow, uint32_t top_k,
    Tiles tiles, float hit_m, uint32_t* tmp_edges, uint32_t* nnz, uint32_t* denom,
    uint32_t* skyc, unsigned long long* dropped, uint32_t* error)
{
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t* hits = smem + size_t(warp) * npow * 3;
    uint32_t* uniq = hits + npow;
    uint32_t* start = uniq + npow;
    const uint32_t total_warps = gridDim.x * kWarps;
    for (uint32_t s = blockIdx.x * kWarps + warp; s < surfaces; s += total_warps) {
        const uint32_t f = s >> 1;
        const uint32_t set = s % sets;
        const Frame fr = side_frame(V, s);
        for (uint32_t j = lane; j < npow; j += 32) {
            uint32_t id = kSky;
            if (j < rays) {
                const size_t k = size_t(set) * rays + j;
                const Vec o = sample_origin(V, f, uv[2 * k], uv[2 * k + 1]);
                const float dx = dirs[3 * k], dy = dirs[3 * k + 1], dz = dirs[3 * k + 2];
                const Vec d = {fr.T.x * dx + fr.B.x * dy + fr.N.x * dz,
                               fr.T.y * dx + fr.B.y * dy + fr.N.y * dz,
                               fr.T.z * dx + fr.B.z * dy + fr.N.z * dz};
                Hit h;
                if (!trace_tiles<false>(nodes, tri, V, hit_m, leaves, tiles, o, d, f, h))
                    atomicExch(error, 1u);
                if (h.facet != kSky) {
                    const Vec ng = {V[3 * h.facet].normal[0], V[3 * h.facet].normal[1],
                                    V[3 * h.facet].normal[2]};
                    id = 2u * h.facet + (vdot(ng, d) < 0.0f ? 0u : 1u);
                }
            }
            hits[j] = id;
        }
        __syncwarp();
        warp_bitonic(hits, int(npow), lane);
        // run heads over the sorted ids; each lane owns a contiguous chunk
        const uint32_t chunk = npow / 32;
        const uint32_t b0 = lane * chunk;
        uint32_t heads = 0;
        for (uint32_t i = b0; i < b0 + chunk; ++i)
            if (hits[i] != kSky && (i == 0 || hits[i] != hits[i - 1])) ++heads;
        uint32_t unique;
        uint32_t at = warp_exclusive(heads, lane, unique);
        for (uint32_t i = b0; i < b0 + chunk; ++i)
            if (hits[i] != kSky && (i == 0 || hits[i] != hits[i - 1])) {
                uniq[at] = hits[i];
                start[at] = i;
                ++at;
            }
        __syncwarp();
        // first sky index = number of non-sky hits
        uint32_t nonsky_local = 0;
        for (uint32_t i = b0; i < b0 + chunk; ++i)
            if (hits[i] != kSky) ++nonsky_local;
        uint32_t nonsky;
        warp_exclusive(nonsky_local, lane, nonsky);
        const uint32_t sky = rays - nonsky;
        // counts: start[i + 1] - start[i]; pack (1023 - count) << 22 | side
        for (uint32_t i = lane; i < unique; i += 32) {
            const uint32_t end = i + 1 < unique ? start[i + 1] : nonsky;
            const uint32_t c = end - start[i];
            hits[i] = ((1023u - c) << 22) | uniq[i];
        }
        __syncwarp();
        uint32_t kept_local = 0, drop_local = 0;
        uint32_t keep = unique;
        if (unique <= top_k) {
            // already sorted by side in uniq; write directly
            for (uint32_t i = lane; i < unique; i += 32) {
                const uint32_t c = 1023u - (hits[i] >> 22);
                tmp_edges[2 * (size_t(s) * top_k + i)] = uniq[i];
                tmp_edges[2 * (size_t(s) * top_k + i) + 1] = c;
                kept_local += c;
            }
        } else {
            keep = top_k;
            uint32_t n2 = 1;
            while (n2 < unique) n2 <<= 1;
            for (uint32_t i = unique + lane; i < n2; i += 32) hits[i] = 0xFFFFFFFFu;
            __syncwarp();
            warp_bitonic(hits, int(n2), lane);  // count desc, side asc
            for (uint32_t i = top_k + lane; i < unique; i += 32) drop_local += 1023u - (hits[i] >> 22);
            // re-key the kept entries by side: side << 10 | count
            for (uint32_t i = lane; i < n2; i += 32) {
                if (i < top_k) {
                    const uint32_t c = 1023u - (hits[i] >> 22);
                    uniq[i] = ((hits[i] & 0x3FFFFFu) << 10) | c;
                } else {
                    uniq[i] = 0xFFFFFFFFu;
                }
            }
            __syncwarp();
            uint32_t k2 = 1;
            while (k2 < top_k) k2 <<= 1;
            warp_bitonic(uniq, int(k2), lane);
            for (uint32_t i = lane; i < top_k; i += 32) {
                const uint32_t c = uniq[i] & 0x3FFu;
                tmp_edges[2 * (size_t(s) * top_k + i)] = uniq[i] >> 10;
                tmp_edges[2 * (size_t(s) * top_k + i) + 1] = c;
                kept_local += c;
            }
        }
        uint32_t kept, dropped_warp;
        warp_exclusive(kept_local, lane, kept);
        warp_exclusive(drop_local, lane, dropped_warp);
        if (lane == 0) {
            nnz[s] = keep;
            skyc[s] = sky;
            denom[s] = kept + sky;
            if (dropped_warp) atomicAdd(dropped, (unsigned long long)dropped_warp);
        }
        __syncwarp();
    }
}

__global__ void k_hemi_compact(const uint32_t* tmp_edges, const uint32_t* rows, uint32_t surfaces,
                               uint32_t top_k, facetcu_csr_edge* edges)
{
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= surfaces) return;
    const uint32_t b = rows[warp], n = rows[warp + 1] - b;
    for (uint32_t i = lane; i < n; i += 32) {
        edges[b + i].neighbor = tmp_edges[2 * (size_t(warp) * top_k + i)];
        edges[b + i].count = tmp_edges[2 * (size_t(warp) * top_k + i) + 1];
    }
}

__global__ void k_set_total(uint32_t* rows, uint32_t n, const unsigned long long* total)
{
    rows[n] = uint32_t(*total);
}

// Occlusion toward the sun from `samples` points per side facing it.
__global__ void __launch_bounds__(256) k_hemi_sunlit(const facetcu_vertex* __restrict__ V,
                                                     const float4* __restrict__ nodes,
                                                     const float4* __restrict__ tri, uint32_t leaves,
                                                     uint32_t surfaces, const float* __restrict__ uv,
                                                     uint32_t samples, uint32_t sets, Vec sun,
                                                     Tiles tiles, float hit_m, float* fraction,
                                                     uint32_t* error)
{
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= surfaces) return;
    const uint32_t s = warp, f = s >> 1, set = s % sets;
    Vec N = {V[3 * f].normal[0], V[3 * f].normal[1], V[3 * f].normal[2]};
    if (s & 1u) N = {-N.x, -N.y, -N.z};
    if (!(vdot(N, sun) > 0.0f)) {
        if (lane == 0) fraction[s] = 0.0f;
        return;
    }
    uint32_t lit = 0;
    for (uint32_t j = lane; j < samples; j += 32) {
        const size_t k = size_t(set) * samples + j;
        const Vec o = sample_origin(V, f, uv[2 * k], uv[2 * k + 1]);
        Hit h;
        if (!trace_tiles<true>(nodes, tri, V, hit_m, leaves, tiles, o, sun, f, h))
            atomicExch(error, 1u);
        if (h.facet == kSky) ++lit;
    }
    for (int o = 16; o > 0; o >>= 1) lit += __shfl_xor_sync(0xffffffffu, lit, o);
    if (lane == 0) fraction[s] = float(lit) / float(samples);
}

Tiles make_tiles(const PeriodicTiles& p)
{
    Tiles t{};
    t.n = std::min<uint32_t>(p.count, 20u) + 1u;
    for (uint32_t i = 0; i < t.n; ++i) {
        t.x[i] = p.dx[i];
        t.z[i] = p.dz[i];
    }
    return t;
}

}  // namespace

void hemisphere_graph(const facetcu_vertex* d_vertices, uint32_t facets, const Lbvh& bvh,
                      const float* d_uv, const float* d_dir, uint32_t rays, uint32_t sets,
                      uint32_t top_k, const PeriodicTiles& periodic, DeviceGraph& g,
                      unsigned long long* dropped, Workspace& ws, cudaStream_t s)
{
    const uint32_t S = 2u * facets;
    top_k = std::min(top_k, rays);
    uint32_t npow = 32;
    while (npow < rays) npow <<= 1;
    g.surfaces = S;
    DeviceBuffer tmp, counters;
    uint32_t* tmp_edges = static_cast<uint32_t*>(tmp.reserve(size_t(S) * top_k * 8 + 8));
    uint32_t* rows = static_cast<uint32_t*>(g.row_offsets.reserve((size_t(S) + 1) * 4));
    uint32_t* den = static_cast<uint32_t*>(g.denominators.reserve(size_t(S) * 4));
    uint32_t* sky = static_cast<uint32_t*>(g.sky.reserve(size_t(S) * 4));
    char* cnt = static_cast<char*>(counters.reserve(64));
    unsigned long long* d_dropped = reinterpret_cast<unsigned long long*>(cnt);
    unsigned long long* d_total = reinterpret_cast<unsigned long long*>(cnt + 8);
    uint32_t* d_error = reinterpret_cast<uint32_t*>(cnt + 16);
    FCU_CHECK(cudaMemsetAsync(cnt, 0, 64, s));
    const size_t smem = size_t(kWarps) * npow * 3 * 4;
    FCU_CHECK(cudaFuncSetAttribute(k_hemi_rows, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   int(smem)));
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int per_sm = 0;
    FCU_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hemi_rows, kWarps * 32, smem));
    const unsigned grid_blocks = unsigned(std::max(1, sms * std::max(per_sm, 1)));
    k_hemi_rows<<<grid_blocks, kWarps * 32, smem, s>>>(
        d_vertices, bvh.nodes.as<float4>(), bvh.tri.as<float4>(), bvh.leaves, S, d_uv, d_dir, rays,
        sets, npow, top_k, make_tiles(periodic), bvh.hit_margin, tmp_edges, rows, den, sky,
        d_dropped, d_error);
    FCU_LAUNCH("k_hemi_rows");
    // rows currently holds per-side nnz; scan in place into offsets
    exclusive_scan_u32(rows, rows, S, d_total, ws, s);
    k_set_total<<<1, 1, 0, s>>>(rows, S, d_total);
    FCU_LAUNCH("k_set_total");
    unsigned long long host[3] = {0, 0, 0};
    FCU_CHECK(cudaMemcpyAsync(host, cnt, 24, cudaMemcpyDeviceToHost, s));
    FCU_CHECK(cudaStreamSynchronize(s));
    if (uint32_t(host[2])) throw Error(FACETCU_DEVICE_CAPACITY, "BVH traversal stack exceeded 64 entries");
    g.nnz = host[1];
    facetcu_csr_edge* edges = static_cast<facetcu_csr_edge*>(g.edges.reserve((g.nnz + 1) * 8));
    k_hemi_compact<<<(S * 32 + 255) / 256, 256, 0, s>>>(tmp_edges, rows, S, top_k, edges);
    FCU_LAUNCH("k_hemi_compact");
    FCU_CHECK(cudaStreamSynchronize(s));
    g.packed_valid = false;
    g.perm_valid = false;
    if (dropped) *dropped = host[0];
}

void hemisphere_sunlit(const facetcu_vertex* d_vertices, uint32_t facets, const Lbvh& bvh,
                       const float* d_uv, uint32_t samples, uint32_t sets, float3 sun,
                       const PeriodicTiles& periodic, float* d_fraction, cudaStream_t s)
{
    const uint32_t S = 2u * facets;
    DeviceBuffer err;
    uint32_t* d_error = static_cast<uint32_t*>(err.reserve(16));
    FCU_CHECK(cudaMemsetAsync(d_error, 0, 16, s));
    k_hemi_sunlit<<<(S * 32 + 255) / 256, 256, 0, s>>>(d_vertices, bvh.nodes.as<float4>(),
                                                       bvh.tri.as<float4>(), bvh.leaves, S, d_uv,
                                                       samples, sets, {sun.x, sun.y, sun.z},
                                                       make_tiles(periodic), bvh.hit_margin,
                                                       d_fraction, d_error);
    FCU_LAUNCH("k_hemi_sunlit");
    uint32_t e = 0;
    FCU_CHECK(cudaMemcpyAsync(&e, d_error, 4, cudaMemcpyDeviceToHost, s));
    FCU_CHECK(cudaStreamSynchronize(s));
    if (e) throw Error(FACETCU_DEVICE_CAPACITY, "BVH traversal stack exceeded 64 entries");
}

}  // namespace facetcu
