// lbvh.cu — linear BVH over the facets for the hemisphere ray caster.
//
// Morton codes (10 bits per axis) of facet centroids, a stable radix sort,
// the radix-tree construction of Karras (2012) with index-augmented keys for
// duplicate codes, and a bottom-up refit with one atomic per internal node.
// Each internal node stores both children's boxes (64 bytes), so a traversal
// step is one node fetch and two slab tests; each leaf stores the triangle
// as (a, e1 = b - a, e2 = c - a) and the facet index (48 bytes), the exact
// operands of the intersection test.  A hit counts only when its point lies
// in the facet's box widened by the hit margin (hemi.cu), and leaf boxes are
// widened by twice that margin, so no float slab test rejects a hit: nearest
// hits are the same as a brute-force search over all facets.
#include <cmath>

#include "internal.h"

namespace facetcu {
namespace {

__device__ __forceinline__ uint32_t expand_bits(uint32_t v)
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

struct Bounds {
    float lo[3], hi[3];
};

__global__ void k_morton(const facetcu_vertex* V, uint32_t n, Bounds scene, uint64_t* keys,
                         uint32_t* ids, float* leaf_box, float margin)
{
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n) return;
    float lo[3], hi[3], c[3];
    for (int a = 0; a < 3; ++a) {
        const float p0 = V[3 * f].position[a], p1 = V[3 * f + 1].position[a],
                    p2 = V[3 * f + 2].position[a];
        lo[a] = fminf(p0, fminf(p1, p2));
        hi[a] = fmaxf(p0, fmaxf(p1, p2));
        c[a] = (lo[a] + hi[a]) * 0.5f;
    }
    uint32_t q[3];
    for (int a = 0; a < 3; ++a) {
        const float ext = scene.hi[a] - scene.lo[a];
        float u = ext > 0.0f ? (c[a] - scene.lo[a]) / ext : 0.5f;
        u = fminf(fmaxf(u, 0.0f), 1.0f);
        q[a] = min(uint32_t(u * 1024.0f), 1023u);
    }
    keys[f] = (expand_bits(q[0]) << 2) | (expand_bits(q[1]) << 1) | expand_bits(q[2]);
    ids[f] = f;
    for (int a = 0; a < 3; ++a) {
        leaf_box[6 * f + a] = lo[a] - margin;
        leaf_box[6 * f + 3 + a] = hi[a] + margin;
    }
}

__device__ __forceinline__ int delta(const uint64_t* m, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    const uint32_t a = uint32_t(m[i]), b = uint32_t(m[j]);
    if (a == b) return 32 + __clz(uint32_t(i) ^ uint32_t(j));
    return __clz(a ^ b);
}

// Karras 2012, Figure 4.  Children: >= 0 internal index, < 0 leaf ~index.
__global__ void k_build_internal(const uint64_t* m, int n, int* child, int* parent_int,
                                 int* parent_leaf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(m, n, i, i + 1) - delta(m, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(m, n, i, i - d);
    int lmax = 2;
    while (delta(m, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(m, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(m, n, i, j);
    int s = 0;
    int div = 2;
    int t = (l + div - 1) / div;
    while (true) {
        if (delta(m, n, i, i + (s + t) * d) > dnode) s += t;
        if (t == 1) break;
        div <<= 1;
        t = (l + div - 1) / div;
    }
    const int gamma = i + s * d + min(d, 0);
    const int left = min(i, j) == gamma ? ~gamma : gamma;
    const int right = max(i, j) == gamma + 1 ? ~(gamma + 1) : gamma + 1;
    child[2 * i] = left;
    child[2 * i + 1] = right;
    if (left < 0) parent_leaf[~left] = i; else parent_int[left] = i;
    if (right < 0) parent_leaf[~right] = i; else parent_int[right] = i;
    if (i == 0) parent_int[0] = -1;
}

__device__ __forceinline__ void child_box(int c, const float* leaf_box_sorted, const float* int_box,
                                          float lo[3], float hi[3])
{
    const float* b = c < 0 ? leaf_box_sorted + 6 * size_t(~c) : int_box + 6 * size_t(c);
    for (int a = 0; a < 3; ++a) {
        lo[a] = b[a];
        hi[a] = b[3 + a];
    }
}

// A child's box as the refit must read it: an internal child's box was
// written by another thread, possibly on another SM, so it is read from L2
// (ld.global.cg); a plain load may return a line this SM's L1 cached before
// the write.
__device__ __forceinline__ void child_box_l2(int c, const float* leaf_box_sorted,
                                             const float* int_box, float lo[3], float hi[3])
{
    const float* b = c < 0 ? leaf_box_sorted + 6 * size_t(~c) : int_box + 6 * size_t(c);
    for (int a = 0; a < 3; ++a) {
        lo[a] = __ldcg(b + a);
        hi[a] = __ldcg(b + 3 + a);
    }
}

__global__ void k_refit(int n, const int* child, const int* parent_int, const int* parent_leaf,
                        const float* leaf_box_sorted, float* int_box, unsigned* flags)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int node = parent_leaf[k];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(&flags[node], 1u) == 0u) return;  // the sibling finishes this node
        __threadfence();
        float l0[3], h0[3], l1[3], h1[3];
        child_box_l2(child[2 * node], leaf_box_sorted, int_box, l0, h0);
        child_box_l2(child[2 * node + 1], leaf_box_sorted, int_box, l1, h1);
        for (int a = 0; a < 3; ++a) {
            __stcg(int_box + 6 * size_t(node) + a, fminf(l0[a], l1[a]));
            __stcg(int_box + 6 * size_t(node) + 3 + a, fmaxf(h0[a], h1[a]));
        }
        node = parent_int[node];
    }
}

// Gather leaf boxes and triangles into sorted order.
__global__ void k_leaves(const facetcu_vertex* V, const uint32_t* ids, uint32_t n,
                         const float* leaf_box, float* leaf_box_sorted, float4* tri)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t f = ids[k];
    for (int a = 0; a < 6; ++a) leaf_box_sorted[6 * size_t(k) + a] = leaf_box[6 * size_t(f) + a];
    const facetcu_vertex& A = V[3 * f];
    const facetcu_vertex& B = V[3 * f + 1];
    const facetcu_vertex& C = V[3 * f + 2];
    tri[3 * size_t(k)] = make_float4(A.position[0], A.position[1], A.position[2], __uint_as_float(f));
    tri[3 * size_t(k) + 1] = make_float4(B.position[0] - A.position[0], B.position[1] - A.position[1],
                                         B.position[2] - A.position[2], 0.0f);
    tri[3 * size_t(k) + 2] = make_float4(C.position[0] - A.position[0], C.position[1] - A.position[1],
                                         C.position[2] - A.position[2], 0.0f);
}

// Node record: float4 {lo0.xyz, child0}, {hi0.xyz, 0}, {lo1.xyz, child1}, {hi1.xyz, 0}.
__global__ void k_nodes(int n, const int* child, const float* leaf_box_sorted, const float* int_box,
                        float4* nodes)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    float l[3], h[3];
    for (int k = 0; k < 2; ++k) {
        const int c = child[2 * i + k];
        child_box(c, leaf_box_sorted, int_box, l, h);
        nodes[4 * size_t(i) + 2 * k] = make_float4(l[0], l[1], l[2], __int_as_float(c));
        nodes[4 * size_t(i) + 2 * k + 1] = make_float4(h[0], h[1], h[2], 0.0f);
    }
}

inline unsigned grid(size_t n, unsigned b) { return unsigned((n + b - 1) / b); }

}  // namespace

float hit_margin(const float lo[3], const float hi[3], uint32_t periodic_count, float size_x,
                 float size_z)
{
    float extent = 0.0f, reach = 0.0f;
    for (int a = 0; a < 3; ++a) {
        extent = std::max(extent, hi[a] - lo[a]);
        reach = std::max(reach, std::max(std::fabs(lo[a]), std::fabs(hi[a])));
    }
    if (periodic_count > 0u) reach = reach + 2.0f * std::max(std::fabs(size_x), std::fabs(size_z));
    return 1.0e-5f * (reach + extent) + 1.0e-7f;
}

void lbvh_build(const facetcu_vertex* d_vertices, uint32_t n, Lbvh& bvh, Workspace& ws,
                cudaStream_t s)
{
    if (n == 0) throw Error(FACETCU_LOGIC_ERROR, "setGeometry() must be called before building the BVH");
    bvh.leaves = n;
    Bounds sb;
    for (int a = 0; a < 3; ++a) {
        sb.lo[a] = bvh.scene_min[a];
        sb.hi[a] = bvh.scene_max[a];
    }
    const float margin = 2.0f * bvh.hit_margin;
    DeviceBuffer keys_a, keys_b, ids_a, ids_b, leaf_box, int_box, child, parent_int, parent_leaf;
    uint64_t* ka = static_cast<uint64_t*>(keys_a.reserve(size_t(n) * 8));
    uint64_t* kb = static_cast<uint64_t*>(keys_b.reserve(size_t(n) * 8));
    uint32_t* ia = static_cast<uint32_t*>(ids_a.reserve(size_t(n) * 4));
    uint32_t* ib = static_cast<uint32_t*>(ids_b.reserve(size_t(n) * 4));
    float* lb = static_cast<float*>(leaf_box.reserve(size_t(n) * 24));
    k_morton<<<grid(n, 256), 256, 0, s>>>(d_vertices, n, sb, ka, ia, lb, margin);
    FCU_LAUNCH("k_morton");
    radix_sort_u64(ka, kb, ia, ib, n, 30, ws, s);
    float* lbs = static_cast<float*>(bvh.parent.reserve(size_t(n) * 24));  // sorted leaf boxes
    float4* tri = static_cast<float4*>(bvh.tri.reserve(size_t(n) * 48));
    k_leaves<<<grid(n, 256), 256, 0, s>>>(d_vertices, ia, n, lb, lbs, tri);
    FCU_LAUNCH("k_leaves");
    if (n == 1) {
        FCU_CHECK(cudaStreamSynchronize(s));
        return;
    }
    int* ch = static_cast<int*>(child.reserve(size_t(n) * 8));
    int* pi = static_cast<int*>(parent_int.reserve(size_t(n) * 4));
    int* pl = static_cast<int*>(parent_leaf.reserve(size_t(n) * 4));
    float* ib2 = static_cast<float*>(int_box.reserve(size_t(n) * 24));
    unsigned* fl = static_cast<unsigned*>(bvh.flags.reserve(size_t(n) * 4));
    FCU_CHECK(cudaMemsetAsync(fl, 0, size_t(n) * 4, s));
    k_build_internal<<<grid(n - 1, 256), 256, 0, s>>>(ka, int(n), ch, pi, pl);
    FCU_LAUNCH("k_build_internal");
    k_refit<<<grid(n, 256), 256, 0, s>>>(int(n), ch, pi, pl, lbs, ib2, fl);
    FCU_LAUNCH("k_refit");
    float4* nodes = static_cast<float4*>(bvh.nodes.reserve(size_t(n) * 64));
    k_nodes<<<grid(n - 1, 256), 256, 0, s>>>(int(n), ch, lbs, ib2, nodes);
    FCU_LAUNCH("k_nodes");
    FCU_CHECK(cudaStreamSynchronize(s));
}

void morton_order(const facetcu_vertex* d_vertices, uint32_t n, const float lo[3],
                  const float hi[3], uint32_t* d_order, Workspace& ws, cudaStream_t s)
{
    Bounds sb;
    for (int a = 0; a < 3; ++a) {
        sb.lo[a] = lo[a];
        sb.hi[a] = hi[a];
    }
    DeviceBuffer keys_a, keys_b, ids_b, boxes;
    uint64_t* ka = static_cast<uint64_t*>(keys_a.reserve(size_t(n) * 8));
    uint64_t* kb = static_cast<uint64_t*>(keys_b.reserve(size_t(n) * 8));
    uint32_t* ia = d_order;
    uint32_t* ib = static_cast<uint32_t*>(ids_b.reserve(size_t(n) * 4));
    float* lb = static_cast<float*>(boxes.reserve(size_t(n) * 24));
    k_morton<<<grid(n, 256), 256, 0, s>>>(d_vertices, n, sb, ka, ia, lb, 0.0f);
    FCU_LAUNCH("k_morton");
    radix_sort_u64(ka, kb, ia, ib, n, 30, ws, s);
    if (ia != d_order)
        FCU_CHECK(cudaMemcpyAsync(d_order, ia, size_t(n) * 4, cudaMemcpyDeviceToDevice, s));
    FCU_CHECK(cudaStreamSynchronize(s));
}

}  // namespace facetcu
