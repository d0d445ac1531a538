// batched.cu — many right-hand sides (bands x suns) against one graph.
//
// The sweep is the reference's two-sided Jacobi update (radiosity.comp:63-106,
// solveCpu facetrtcore.cpp:1476-1529) applied to a panel of P RHS columns at
// once:
//   H_s,c  = (sky_s * L_c + sum_e count_e * B_{n_e,c}) / denom_s + D_s,c
//   B'_s,c = e_s,c + rho_s,c * H_s,c + tau_s,c * H_{s^1},c
// (denom_s = 0: H = L_c + D_s,c).
//
// GB300 mapping.  The panel is stored side-major ([S][P]), so the gather of
// neighbour n reads one contiguous row of P values shared by every column.
// Wide panels (P = 32, 64, 128) give each lane P/32 adjacent columns: one
// vector load per lane per edge (float / float2 / float4 in FP32, 1/2/4
// packed BF16 in the defect sweep), one warp shuffle per packed 4-byte edge
// (22-bit neighbour, 10-bit count), full 32-edge chunks without predication.
// Narrow panels (P < 32, few RHS) split the warp into 32/P edge groups.
// The graph is renumbered once along a Morton curve of facet centroids and
// every warp sweeps a contiguous run of facets, so the neighbour rows a CTA
// touches stay hot in L1/L2.  The grid is persistent (a multiple of the SM
// count); each warp keeps per-column max|dB| and max|B| in registers and one
// atomicMax per CTA and column publishes them.  A one-block check kernel
// after every sweep sets a device-side done flag, so sweeps run in batches
// without host round trips and stop at the exact sweep that converged.
//
// Precision modes:
//   FP32  — panel and gather in FP32;
//   FP64  — the same sweep in double (the truth the 1e-4 bar is checked on);
//   MIXED — FP32 state with low-precision corrections.  Panels of 32 or
//           more columns: an FP32 sweep, then residual-tracked int8 steps
//           (per-column scale, exact int32 gather sums, FP32 residual; see
//           k_step_i8), then a verifying FP32 sweep.  Narrower panels:
//           defect cycles, d <- K d with d stored in BF16 and accumulated in
//           FP32, each cycle restarted from a fresh FP32 sweep.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "internal.h"

namespace facetcu {
namespace {

constexpr int kWarps = 8;  // warps per CTA
constexpr int kMaxP = 128;
#ifndef FCU_NARROW_U
// loads in flight per lane for 1-4 column panels (the 32-scene batch of
// 4.7 M facets, whose thermal band is a 1-column panel: 172.0 ms at 8, 172.6
// at 4, 192 at 12 or 16)
#define FCU_NARROW_U 8
#endif

struct PanelParams {
    // per side and column, [S][P]
    const float* rho;
    const float* tau;
    const float* emis;
    const float* direct;
    const float* skyL;    // [P]
    const float* colmax;  // [P] max|B| of the previous sweep (floor of the per-side test)
    const float* omega;   // [P] Chebyshev weight of the int8 step being formed (or null)
};

// The per-side stop test: |dB_s| / max(|B_s|, kSideFloor * max|B|) <= tol
// per column, the form of the accuracy bar (relative error per side, with
// sides below 1e-6 of the column's maximum measured against that floor).
constexpr float kSideFloor = 1e-6f;
__device__ __forceinline__ float rel_change(float d, float b, float floor_abs)
{
    d = fabsf(d);
    if (d == 0.0f) return 0.0f;
    const float den = fmaxf(fabsf(b), floor_abs);
    return den > 0.0f ? d / den : INFINITY;
}

struct GraphView {
    const uint32_t* rows;
    const uint32_t* packed;            // when non-null
    const facetcu_csr_edge* edges;     // otherwise
    const uint32_t* denom;
    const uint32_t* skyc;
    uint32_t facets;
    uint32_t nb_bits;                  // neighbour field of a packed word (count above it)
    // scene batches (block-diagonal graphs): the scene of each facet, and per
    // scene the int8 steps' worst per-side ratio per column and a done flag
    const uint16_t* scene;             // null when the graph is one scene
    uint32_t scenes;
    uint32_t* scene_stats;             // [scenes][kMaxP] worst per-side ratio (float bits)
    uint32_t* scene_md;                // [scenes][kMaxP] max |R| (float bits)
    float* scene_sig;                  // two slots of [scenes][kMaxP] int8 step scales
    float* scene_cheb;                 // [scenes][4 kMaxP] Chebyshev state (weights at 2 kMaxP)
    uint32_t* scene_done;              // [scenes]
    uint32_t legacy_step;              // 1: 64-column int8 steps on the register-gather kernel
    uint32_t counts8;                  // 1: every count is at most 255 (the solver's copy)
    uint32_t step_ctas;                // pipelined step: CTAs per SM (0: as many as fit)
};

__device__ __forceinline__ void edge_at(const GraphView& g, uint32_t e, uint32_t& nb, float& c)
{
    if (g.packed) {
        const uint32_t p = __ldg(g.packed + e);
        nb = p & ((1u << g.nb_bits) - 1u);
        c = float(p >> g.nb_bits);
    } else {
        const facetcu_csr_edge ed = g.edges[e];
        nb = ed.neighbor;
        c = float(ed.count);
    }
}

template <typename T> __device__ __forceinline__ float load_as_float(const T* p);
template <> __device__ __forceinline__ float load_as_float<float>(const float* p) { return __ldg(p); }
template <> __device__ __forceinline__ float load_as_float<__nv_bfloat16>(const __nv_bfloat16* p)
{
    return __bfloat162float(*p);
}

template <typename T> __device__ __forceinline__ float absf(T x) { return float(x < T(0) ? -x : x); }

// The facet range of one warp: contiguous runs keep neighbour rows local.
__device__ __forceinline__ void warp_range(uint32_t facets, uint32_t& begin, uint32_t& end)
{
    const uint32_t warps = gridDim.x * kWarps;
    const uint32_t w = blockIdx.x * kWarps + (threadIdx.x >> 5);
    const uint32_t chunk = (facets + warps - 1) / warps;
    begin = min(facets, w * chunk);
    end = min(facets, begin + chunk);
}

// ---- narrow panels (P < 32): 32/P edge groups per warp -------------------
template <int P, typename T, typename Acc>
__device__ __forceinline__ Acc gather_narrow(const GraphView& g, uint32_t s, const T* X, int lane)
{
    constexpr int G = 32 / P;
    const int grp = lane / P, col = lane % P;
    const uint32_t start = g.rows[s], end = g.rows[s + 1];
    Acc acc = 0;
    if constexpr (P <= 4) {
        // 8+ edge groups: each lane walks its group's edges itself, U loads
        // in flight (a broadcast of one 32-edge chunk would leave most of
        // the unrolled loads empty)
        constexpr int U = FCU_NARROW_U;
        for (uint32_t e = start + uint32_t(grp); e < end; e += uint32_t(G * U)) {
            Acc v[U];
            float c[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t idx = e + uint32_t(u * G);
                v[u] = 0;
                c[u] = 0.0f;
                if (idx < end) {
                    uint32_t nb;
                    edge_at(g, idx, nb, c[u]);
                    if constexpr (sizeof(Acc) == 8)
                        v[u] = Acc(X[size_t(nb) * P + col]);
                    else
                        v[u] = Acc(load_as_float<T>(X + size_t(nb) * P + col));
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) acc += Acc(c[u]) * v[u];
        }
    } else {
    for (uint32_t base = start; base < end; base += 32) {
        const uint32_t n = min(32u, end - base);
        uint32_t pk = 0;
        float pc = 0.0f;
        if (uint32_t(lane) < n) {
            uint32_t nb;
            edge_at(g, base + lane, nb, pc);
            pk = nb;
        }
        constexpr int U = 8;
        for (uint32_t j = 0; j < n; j += G * U) {
            Acc v[U];
            float c[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t idx = j + u * G + grp;
                const uint32_t nb = __shfl_sync(0xffffffffu, pk, int(idx & 31u));
                c[u] = __shfl_sync(0xffffffffu, pc, int(idx & 31u));
                if (idx < n) {
                    if constexpr (sizeof(Acc) == 8)
                        v[u] = Acc(X[size_t(nb) * P + col]);
                    else
                        v[u] = Acc(load_as_float<T>(X + size_t(nb) * P + col));
                } else {
                    v[u] = 0;
                    c[u] = 0.0f;
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) acc += Acc(c[u]) * v[u];
        }
    }
    }
#pragma unroll
    for (int o = P; o < 32; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}

// ---- 1- and 2-column panels: a group of 8P lanes per side -----------------
// 8 edge lanes x P columns per side, so a warp holds 4/P sides (2/P facets)
// at once: a row of 100-200 edges keeps each lane's U loads busy, and the
// chain of dependent loads of a side (row offsets, edge words, neighbour
// values, parameters) is paid once for several sides.  (One side per warp
// left most of the 32 x U load slots empty and took ~7 dependent round
// trips per facet.)
// Warps take facet pairs round robin (pair w, w + W, ...): every warp sees
// every part of the graph, so scenes with longer rows in a batch do not
// load single warps (a contiguous range per warp did), and no counter.
template <int P> struct NarrowGroup {
    static_assert(P == 1 || P == 2, "1 or 2 columns");
    static constexpr int kLanes = 8 * P;        // lanes per side
    static constexpr int kFacets = 16 / kLanes;  // facets per warp pass
};
__device__ __forceinline__ void warp_pairs(uint32_t& first, uint32_t& stride)
{
    first = blockIdx.x * kWarps + (threadIdx.x >> 5);
    stride = gridDim.x * kWarps;
}

// An edge read once per sweep: a streaming load, so that the graph passing
// through L2 does not evict the neighbour values the gathers hit there.
__device__ __forceinline__ void edge_stream(const GraphView& g, uint32_t e, uint32_t& nb, float& c)
{
    if (g.packed) {
        const uint32_t p = __ldcs(g.packed + e);
        nb = p & ((1u << g.nb_bits) - 1u);
        c = float(p >> g.nb_bits);
    } else {
        edge_at(g, e, nb, c);
    }
}

template <int P, typename T, typename Acc>
__device__ __forceinline__ Acc gather_group(const GraphView& g, uint32_t s, bool valid, const T* X,
                                            int eg, int col)
{
    constexpr int U = FCU_NARROW_U;
    Acc acc = 0;
    if (valid) {
        const uint32_t start = __ldg(g.rows + s), end = __ldg(g.rows + s + 1);
        for (uint32_t e = start + uint32_t(eg); e < end; e += uint32_t(8 * U)) {
            Acc v[U];
            float c[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t idx = e + uint32_t(u * 8);
                v[u] = 0;
                c[u] = 0.0f;
                if (idx < end) {
                    uint32_t nb;
                    edge_stream(g, idx, nb, c[u]);
                    if constexpr (sizeof(Acc) == 8)
                        v[u] = Acc(X[size_t(nb) * P + col]);
                    else
                        v[u] = Acc(load_as_float<T>(X + size_t(nb) * P + col));
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) acc += Acc(c[u]) * v[u];
        }
    }
    // the sum over the side's 8 edge lanes (lanes eg * P + col of the group)
#pragma unroll
    for (int o = P; o < 8 * P; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}

// Fold the statistics of every lane of column c into lane c.
__device__ __forceinline__ void fold_narrow_stats(float* md, float* mb, float* mr, int P)
{
    for (int o = P; o < 32; o <<= 1) {
        md[0] = fmaxf(md[0], __shfl_xor_sync(0xffffffffu, md[0], o));
        mb[0] = fmaxf(mb[0], __shfl_xor_sync(0xffffffffu, mb[0], o));
        mr[0] = fmaxf(mr[0], __shfl_xor_sync(0xffffffffu, mr[0], o));
    }
}

// ---- wide panels (P = 32, 64, 128) ---------------------------------------
// Each lane moves 16 bytes of a neighbour row per load: CPL = 4 FP32 or 8
// BF16 columns.  L = P / CPL lanes cover one row, so a warp gathers
// G = 32 / L edges per load instruction (e.g. P = 64 BF16: 8 lanes per
// 128-byte row, 4 edges at once); the G partial sums are folded with
// shuffles at the end of the row and the first L lanes own the result.
// Columns per 16-byte vector: 4 FP32 or 8 BF16.
template <bool kBF16> constexpr int kVecCols = kBF16 ? 8 : 4;

// acc[k] += sum over edges e of side s of count_e * X[n_e][col0 + k], where
// col0 = (lane % L) * CPL; valid in every lane after the fold (lanes of the
// same sub-index hold the same sums).  kGatherU vector loads per lane are in
// flight at once (raw 16-byte words, unpacked at the multiply-add), and with
// kPrefetch the next 32-edge chunk's packed edges are loaded while the
// current chunk is gathered.
#ifndef FCU_GATHER_U
#define FCU_GATHER_U 8
#endif
#ifndef FCU_PREFETCH
#define FCU_PREFETCH 1
#endif
#ifndef FCU_MIN_BLOCKS
#define FCU_MIN_BLOCKS 3
#endif
#ifndef FCU_STEP64_MIN_BLOCKS
#define FCU_STEP64_MIN_BLOCKS 4
#endif
// Resident CTAs per SM of the FP32 wide sweep (64 registers at 4): the
// config-2 forest's 64-column sweep 1.096 ms at 4 against 1.146 at 3 and
// 1.458 at 2 (latency hidden by warps, not by registers); at 128 columns
// the spills at 64 registers cost more (the batched FP32 solve of 479,600
// facets x 16,384 columns: 11.5 s at 3, 12.3 s at 4), so that width keeps 3.
#ifndef FCU_SWEEP_MIN_BLOCKS
#define FCU_SWEEP_MIN_BLOCKS 4
#endif
template <int P> struct SweepBlocks {
    static constexpr int value = P == 128 ? 3 : FCU_SWEEP_MIN_BLOCKS;
};
#ifndef FCU_SCENE_SKIP
#define FCU_SCENE_SKIP 1
#endif
constexpr int kGatherU = FCU_GATHER_U;
constexpr bool kPrefetch = FCU_PREFETCH != 0;
constexpr int kMinBlocks = FCU_MIN_BLOCKS;
// Resident CTAs per SM of the int8 step: the 64-column step is bound by L2
// latency and runs 6 % faster with 4 CTAs (64 registers, a few spills to
// L1) than with 3; at 128 columns the spills grow and 3 CTAs are faster.
template <int P>
struct StepBlocks {
    static constexpr int value = P == 64 ? FCU_STEP64_MIN_BLOCKS : kMinBlocks;
};

__device__ __forceinline__ void edge_word(const uint32_t* __restrict__ packed,
                                          const facetcu_csr_edge* __restrict__ edges, uint32_t e,
                                          uint32_t nb_bits, uint32_t& nb, float& c)
{
    if (packed) {
        const uint32_t p = __ldcs(packed + e);  // read once per sweep: evict first
        nb = p & ((1u << nb_bits) - 1u);
        c = float(p >> nb_bits);
    } else {
        const uint2 w = __ldcs(reinterpret_cast<const uint2*>(edges) + e);
        nb = w.x;
        c = float(w.y);
    }
}

template <bool kBF16>
__device__ __forceinline__ void unpack16(const uint4& q, float* v)
{
    if constexpr (kBF16) {
        const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            v[2 * i] = __uint_as_float(w[i] << 16);
            v[2 * i + 1] = __uint_as_float(w[i] & 0xFFFF0000u);
        }
    } else {
        v[0] = __uint_as_float(q.x);
        v[1] = __uint_as_float(q.y);
        v[2] = __uint_as_float(q.z);
        v[3] = __uint_as_float(q.w);
    }
}

template <int P, bool kBF16>
__device__ __forceinline__ void gather_split(const uint32_t* __restrict__ rows,
                                             const uint32_t* __restrict__ packed,
                                             const facetcu_csr_edge* __restrict__ edges,
                                             uint32_t nb_bits, uint32_t s, const void* X,
                                             int lane, float* acc)
{
    constexpr int CPL = kVecCols<kBF16>;
    constexpr int L = P / CPL;  // lanes per row = 16-byte vectors per row
    constexpr int G = 32 / L;   // edges per load instruction
    constexpr int U = kGatherU;
    const int grp = lane / L, sub = lane % L;
    const uint4* __restrict__ X16 = reinterpret_cast<const uint4*>(X);
    const uint32_t start = __ldg(rows + s), end = __ldg(rows + s + 1);
    uint32_t nbn = 0;
    float cn = 0.0f;
    if (kPrefetch && start + uint32_t(lane) < end)
        edge_word(packed, edges, start + lane, nb_bits, nbn, cn);
    for (uint32_t base = start; base < end; base += 32) {
        const uint32_t n = min(32u, end - base);
        uint32_t nbv = 0;
        float cv = 0.0f;
        if constexpr (kPrefetch) {
            nbv = nbn;
            cv = cn;
            const uint32_t next = base + 32u + uint32_t(lane);
            if (next < end) edge_word(packed, edges, next, nb_bits, nbn, cn);
        } else if (uint32_t(lane) < n) {
            edge_word(packed, edges, base + lane, nb_bits, nbv, cv);
        }
        for (uint32_t j = 0; j < n; j += G * U) {
            uint4 q[U];
            float c[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t idx = j + u * G + grp;
                const int src = int(idx & 31u);
                const uint32_t nb = __shfl_sync(0xffffffffu, nbv, src);
                c[u] = __shfl_sync(0xffffffffu, cv, src);
                if (idx < n) {
                    q[u] = __ldg(X16 + size_t(nb) * L + sub);
                } else {
                    c[u] = 0.0f;
                    q[u] = make_uint4(0u, 0u, 0u, 0u);
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                float v[CPL];
                unpack16<kBF16>(q[u], v);
#pragma unroll
                for (int k = 0; k < CPL; ++k) acc[k] += c[u] * v[k];
            }
        }
    }
#pragma unroll
    for (int o = L; o < 32; o <<= 1)
#pragma unroll
        for (int k = 0; k < CPL; ++k) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
}

// The same product for 8 or 16 FP32 columns: L = P / 4 lanes per row, so one
// load instruction covers G = 32 / L = 16 or 8 edges, and a round of
// 32 * G / 4 edges (128 or 64, G / 4 packed words per lane) gives every lane
// eight 16-byte loads in flight (a 32-edge chunk would fill only two or four
// of them).  Afterwards every lane holds the sums of its 4 columns
// (col0 = (lane % L) * 4).
template <int P>
__device__ __forceinline__ void gather_rounds(const uint32_t* __restrict__ rows,
                                              const uint32_t* __restrict__ packed,
                                              const facetcu_csr_edge* __restrict__ edges,
                                              uint32_t nb_bits, uint32_t s, const float* X,
                                              int lane, float* acc)
{
    constexpr int L = P / 4;
    constexpr int G = 32 / L;
    constexpr int W = G / 4;   // packed words per lane per round
    constexpr int E = 32 * W;  // edges per round
    constexpr int U = E / G;   // loads per lane per round (8)
    static_assert(P == 8 || P == 16, "rounds of 8 loads for 8 or 16 columns");
    const int grp = lane / L, sub = lane % L;
    const float4* __restrict__ X4 = reinterpret_cast<const float4*>(X);
    const uint32_t start = __ldg(rows + s), end = __ldg(rows + s + 1);
    for (uint32_t base = start; base < end; base += E) {
        uint32_t nbv[W];
        float cv[W];
#pragma unroll
        for (int w = 0; w < W; ++w) {
            nbv[w] = 0u;
            cv[w] = 0.0f;
            const uint32_t e = base + uint32_t(w * 32 + lane);
            if (e < end) edge_word(packed, edges, e, nb_bits, nbv[w], cv[w]);
        }
        float4 q[U];
        float c[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int idx = u * G + grp;
            const uint32_t nb = __shfl_sync(0xffffffffu, nbv[idx >> 5], idx & 31);
            c[u] = __shfl_sync(0xffffffffu, cv[idx >> 5], idx & 31);
            if (base + uint32_t(idx) < end) {
                q[u] = __ldg(X4 + size_t(nb) * L + sub);
            } else {
                q[u] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                c[u] = 0.0f;
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            acc[0] += c[u] * q[u].x;
            acc[1] += c[u] * q[u].y;
            acc[2] += c[u] * q[u].z;
            acc[3] += c[u] * q[u].w;
        }
    }
#pragma unroll
    for (int o = L; o < 32; o <<= 1)
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
}

// Dynamic hand-out of facet chunks (contiguous in Morton order); the counter
// is reset by k_check after every sweep.
// Facets per hand-out: 2 measured best on the config-2 forest (64-column
// step 0.648 ms at 8 facets, 0.626 at 4, 0.623 at 2, 0.632 at 1; whole
// solve 11.80 -> 11.35 ms), finer chunks evening out the warps' rows.
// Scene batches hand out 8: a warp that moves into another scene publishes
// its per-scene statistics (atomics per column), and small chunks scatter a
// warp over many scenes (the 32-scene batch of 4.7 M facets: 235 ms at 8
// facets, 252 at 2, 236 at 32 with the register-gather step; 172.8 ms at 8,
// 176.8 at 4, 174.1 at 6, 172.7 at 12 with the pipelined one).
#ifndef FCU_CHUNK
#define FCU_CHUNK 2
#endif
#ifndef FCU_SCENE_CHUNK
#define FCU_SCENE_CHUNK 8
#endif
constexpr uint32_t kChunk = FCU_CHUNK;
constexpr uint32_t kSceneChunk = FCU_SCENE_CHUNK;
__device__ __forceinline__ uint32_t next_chunk(uint32_t* counter, int lane)
{
    uint32_t c = 0;
    if (lane == 0) c = atomicAdd(counter, 1u);
    return __shfl_sync(0xffffffffu, c, 0);
}

// Every warp takes chunks of kChunk consecutive facets until none are left.
// (Handing a CTA a larger run for its warps to share, for L1 reuse of
// neighbour rows, measured slower at 64-256 facets per CTA.)
template <uint32_t C = kChunk, typename F>
__device__ __forceinline__ void for_each_facet(uint32_t facets, uint32_t* counter, int lane,
                                               F&& body)
{
    const uint32_t chunks = (facets + C - 1) / C;
    for (uint32_t ch = next_chunk(counter, lane); ch < chunks; ch = next_chunk(counter, lane)) {
        const uint32_t fe = min(facets, (ch + 1) * C);
        for (uint32_t f = ch * C; f < fe; ++f) body(f);
    }
}

__device__ __forceinline__ void load4(const float* p, float* v)
{
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
    v[3] = q.w;
}
__device__ __forceinline__ void store4(float* p, const float* v)
{
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}

// CTA-level max over warps, then one atomic per column; columns [col0,
// col0 + n) of the lane hold md (max |dB|), mb (max |B|) and mr (max
// per-side relative change); lanes with own = false contribute nothing.
template <int NC>
__device__ __forceinline__ void publish_cols(const float* md, const float* mb, const float* mr,
                                             int col0, bool own, int P, uint32_t* stats)
{
    __shared__ float s_md[kWarps][kMaxP], s_mb[kWarps][kMaxP], s_mr[kWarps][kMaxP];
    const int warp = threadIdx.x >> 5;
    for (int c = (threadIdx.x & 31); c < kMaxP; c += 32) {
        s_md[warp][c] = 0.0f;
        s_mb[warp][c] = 0.0f;
        s_mr[warp][c] = 0.0f;
    }
    __syncwarp();
    if (own) {
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            s_md[warp][col0 + k] = md[k];
            s_mb[warp][col0 + k] = mb[k];
            s_mr[warp][col0 + k] = mr[k];
        }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < P; c += blockDim.x) {
        float a = 0.0f, b = 0.0f, r = 0.0f;
        for (int w = 0; w < kWarps; ++w) {
            a = fmaxf(a, s_md[w][c]);
            b = fmaxf(b, s_mb[w][c]);
            r = fmaxf(r, s_mr[w][c]);
        }
        atomicMax(stats + c, __float_as_uint(a));
        atomicMax(stats + kMaxP + c, __float_as_uint(b));
        atomicMax(stats + 2 * kMaxP + c, __float_as_uint(r));
    }
}

// Narrow-kernel statistics: lane c < P holds column c.
template <int NC>
__device__ __forceinline__ void publish_stats(const float* md, const float* mb, const float* mr,
                                              int lane, int P, uint32_t* stats)
{
    publish_cols<NC>(md, mb, mr, lane * NC, lane < P, P, stats);
}

// One full FP32 sweep B_out = Q + K B_in over a wide panel.  Bin == nullptr
// stands for B_in = 0 (the first sweep of a solve that starts from zero):
// the gather is skipped, which gives the same bits as gathering zeros.
template <int P>
__global__ void __launch_bounds__(kWarps * 32, SweepBlocks<P>::value) k_sweep_wide(GraphView g, PanelParams pp,
                                                            const float* __restrict__ Bin,
                                                            float* __restrict__ Bout,
                                                            uint32_t* stats, uint32_t* counter,
                                                            const uint32_t* done)
{
    if (*done) return;
    constexpr int CPL = 4;
    constexpr int L = P / CPL;
    const int lane = threadIdx.x & 31;
    const bool owner = lane < L;
    const int col0 = (lane % L) * CPL;
    float md[CPL], mb[CPL], mr[CPL], Lsky[CPL], fl[CPL];
#pragma unroll
    for (int k = 0; k < CPL; ++k) {
        md[k] = 0.0f;
        mb[k] = 0.0f;
        mr[k] = 0.0f;
        Lsky[k] = pp.skyL[col0 + k];
        fl[k] = kSideFloor * pp.colmax[col0 + k];
    }
    for_each_facet(g.facets, counter, lane, [&](uint32_t f) {
        {
            float h[2][CPL];
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                const uint32_t s = 2u * f + side;
                float acc[CPL];
#pragma unroll
                for (int k = 0; k < CPL; ++k) acc[k] = 0.0f;
                if (Bin) {
                    if constexpr (P < 32)
                        gather_rounds<P>(g.rows, g.packed, g.edges, g.nb_bits, s, Bin, lane, acc);
                    else
                        gather_split<P, false>(g.rows, g.packed, g.edges, g.nb_bits, s, Bin, lane,
                                               acc);
                }
                const uint32_t d = __ldg(g.denom + s);
                const float skyc = float(__ldg(g.skyc + s));
                float dir[CPL];
                load4(pp.direct + size_t(s) * P + col0, dir);
#pragma unroll
                for (int k = 0; k < CPL; ++k)
                    h[side][k] = (d != 0u ? (skyc * Lsky[k] + acc[k]) / float(d) : Lsky[k]) + dir[k];
            }
            if (owner) {
                const size_t i0 = size_t(2u * f) * P + col0, i1 = i0 + P;
                float e0[CPL], e1[CPL], r0[CPL], r1[CPL], t0[CPL], t1[CPL], o0[CPL], o1[CPL];
                float b0[CPL], b1[CPL];
                load4(pp.emis + i0, e0);
                load4(pp.emis + i1, e1);
                load4(pp.rho + i0, r0);
                load4(pp.rho + i1, r1);
                load4(pp.tau + i0, t0);
                load4(pp.tau + i1, t1);
                if (Bin) {
                    load4(Bin + i0, o0);
                    load4(Bin + i1, o1);
                } else {
#pragma unroll
                    for (int k = 0; k < CPL; ++k) o0[k] = o1[k] = 0.0f;
                }
#pragma unroll
                for (int k = 0; k < CPL; ++k) {
                    b0[k] = e0[k] + r0[k] * h[0][k] + t0[k] * h[1][k];
                    b1[k] = e1[k] + r1[k] * h[1][k] + t1[k] * h[0][k];
                    md[k] = fmaxf(md[k], fmaxf(fabsf(b0[k] - o0[k]), fabsf(b1[k] - o1[k])));
                    mb[k] = fmaxf(mb[k], fmaxf(fabsf(b0[k]), fabsf(b1[k])));
                    mr[k] = fmaxf(mr[k], fmaxf(rel_change(b0[k] - o0[k], b0[k], fl[k]),
                                               rel_change(b1[k] - o1[k], b1[k], fl[k])));
                }
                store4(Bout + i0, b0);
                store4(Bout + i1, b1);
            }
        }
    });
    publish_cols<CPL>(md, mb, mr, col0, owner, P, stats);
}

// The first sweep of a solve from zero, B = T(0): no gather, so one thread
// per facet and column, facets round robin over the grid (a thread keeps
// its column, its statistics stay in registers), the same arithmetic as
// k_sweep_wide with a zero gather.  (Run through k_sweep_wide's warp-per-
// facet loop it took 0.35 ms at the bench's 64 columns.)
template <int P>
__global__ void __launch_bounds__(256) k_sweep_zero(GraphView g, PanelParams pp,
                                                    float* __restrict__ Bout, uint32_t* stats,
                                                    const uint32_t* done)
{
    static_assert(256 % P == 0, "whole facets per block");
    constexpr int FPB = 256 / P;  // facets per block pass
    if (*done) return;
    const int c = threadIdx.x % P;
    const float L = pp.skyL[c], fl = kSideFloor * pp.colmax[c];
    float md = 0.0f, mb = 0.0f, mr = 0.0f;
    const uint32_t stride = gridDim.x * FPB;
    for (uint32_t f = blockIdx.x * FPB + threadIdx.x / P; f < g.facets; f += stride) {
        const uint32_t s0 = 2u * f, s1 = s0 + 1u;
        const uint32_t d0 = __ldg(g.denom + s0), d1 = __ldg(g.denom + s1);
        const float k0 = float(__ldg(g.skyc + s0)), k1 = float(__ldg(g.skyc + s1));
        const size_t i0 = size_t(s0) * P + c, i1 = i0 + P;
        const float h0 = (d0 != 0u ? (k0 * L) / float(d0) : L) + __ldcs(pp.direct + i0);
        const float h1 = (d1 != 0u ? (k1 * L) / float(d1) : L) + __ldcs(pp.direct + i1);
        const float b0 = __ldcs(pp.emis + i0) + __ldcs(pp.rho + i0) * h0 + __ldcs(pp.tau + i0) * h1;
        const float b1 = __ldcs(pp.emis + i1) + __ldcs(pp.rho + i1) * h1 + __ldcs(pp.tau + i1) * h0;
        Bout[i0] = b0;
        Bout[i1] = b1;
        md = fmaxf(md, fmaxf(fabsf(b0), fabsf(b1)));
        mr = fmaxf(mr, fmaxf(rel_change(b0, b0, fl), rel_change(b1, b1, fl)));
    }
    mb = md;  // the change from zero is the value
    __shared__ float s_st[3][256];
    s_st[0][threadIdx.x] = md;
    s_st[1][threadIdx.x] = mb;
    s_st[2][threadIdx.x] = mr;
    __syncthreads();
    for (int col = threadIdx.x; col < P; col += blockDim.x) {
        float a = 0.0f, b = 0.0f, r = 0.0f;
        for (int t = col; t < 256; t += P) {
            a = fmaxf(a, s_st[0][t]);
            b = fmaxf(b, s_st[1][t]);
            r = fmaxf(r, s_st[2][t]);
        }
        atomicMax(stats + col, __float_as_uint(a));
        atomicMax(stats + kMaxP + col, __float_as_uint(b));
        atomicMax(stats + 2 * kMaxP + col, __float_as_uint(r));
    }
}

// ---- residual-tracked int8 steps (MIXED, wide panels) --------------------
// State per cell: X (FP32 iterate), R = T(X) - X (FP32, its Jacobi
// residual) and Q = round(R / sigma) (int8, one scale sigma per column, not
// yet applied).  One step applies the quantized residual and updates the
// residual by exactly what was applied:
//   delta = sigma_in * Q_in,  X += delta,  R += K delta - delta,
//   Q_out = round(R / sigma_out),  sigma_out = max|R_in| / 127,
// where K delta comes from gathering the int8 neighbour rows (count * q
// summed exactly in int32).  R stays the true residual of X up to FP32
// rounding, so the int8 rounding only perturbs the step: max|R| contracts by
// about c + (1 + c) / 254 per step (c the spectral radius of K), as with a
// BF16 defect, while each gathered neighbour row is half as wide and no
// periodic FP32 correction sweep is needed.  |R_out| < max|R_in| because
// c < 1, so Q_out fits in [-127, 127] (clamped all the same).
//
// Chebyshev acceleration (Golub and Varga's semi-iterative method on
// [-c, c]): the step formed is delta' = omega R + (omega - 1) delta instead
// of R, with the weights omega_1 = 1, omega_2 = 1 / (1 - c^2 / 2),
// omega_{k+1} = 1 / (1 - c^2 omega_k / 4).  K is non-negative, so every
// eigenvalue lies in |lambda| <= c, its Perron root; c is estimated per
// column from the residual ratio after kChebWarm plain steps and Chebyshev
// is used only for c <= kChebMax, where the convergence ellipse of [-c, c]
// holds that whole disk.  R is updated by exactly the applied step, so the
// weights change the path, never the fixed point.

__device__ __forceinline__ void edge_word_i(const uint32_t* __restrict__ packed,
                                            const facetcu_csr_edge* __restrict__ edges,
                                            uint32_t e, uint32_t nb_bits, uint32_t& nb, int& c)
{
    if (packed) {
        const uint32_t w = __ldcs(packed + e);  // read once per step: evict first
        nb = w & ((1u << nb_bits) - 1u);
        c = int(w >> nb_bits);
    } else {
        const uint2 w = __ldg(reinterpret_cast<const uint2*>(edges) + e);
        nb = w.x;
        c = int(w.y);
    }
}

// sum over 4 of signed byte a_i x unsigned byte b_i, plus c (PTX dp4a).
__device__ __forceinline__ int dp4a_su(uint32_t a, uint32_t b, int c)
{
    int d;
    asm("dp4a.s32.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel)
{
    uint32_t d;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(sel));
    return d;
}

// Bytes (shift .. shift+7) of four counts as one word, edge i in byte i.
__device__ __forceinline__ uint32_t pack_bytes(int c0, int c1, int c2, int c3, int shift)
{
    return (uint32_t(c0 >> shift) & 255u) | ((uint32_t(c1 >> shift) & 255u) << 8) |
           ((uint32_t(c2 >> shift) & 255u) << 16) | ((uint32_t(c3 >> shift) & 255u) << 24);
}

// 4 x 4 byte transpose: a, b, c, d are four edges' words (byte k = column
// k); t[k] gets column k of the four edges (byte i = edge i).
__device__ __forceinline__ void transpose4(uint32_t a, uint32_t b, uint32_t c, uint32_t d,
                                           uint32_t* t)
{
    const uint32_t ab_lo = prmt(a, b, 0x5140u), ab_hi = prmt(a, b, 0x7362u);
    const uint32_t cd_lo = prmt(c, d, 0x5140u), cd_hi = prmt(c, d, 0x7362u);
    t[0] = prmt(ab_lo, cd_lo, 0x5410u);
    t[1] = prmt(ab_lo, cd_lo, 0x7632u);
    t[2] = prmt(ab_hi, cd_hi, 0x5410u);
    t[3] = prmt(ab_hi, cd_hi, 0x7632u);
}

// acc[0..16) += sum over edges of side s of count * Q[n][sub * 16 + k]; the
// G lane groups each take every G-th edge (partial sums).  Eight 16-byte
// loads per lane are in flight per round; the next round's packed edges are
// prefetched.
template <int P>
__device__ __forceinline__ void gather_i8(const uint32_t* __restrict__ rows,
                                          const uint32_t* __restrict__ packed,
                                          const facetcu_csr_edge* __restrict__ edges,
                                          uint32_t nb_bits, uint32_t s,
                                          const int8_t* __restrict__ Q, int lane, int* acc)
{
    constexpr int L = P / 16;              // lanes per row, 16 bytes each
    constexpr int G = 32 / L;              // edges per load instruction
    constexpr int W = G >= 4 ? G / 4 : 1;  // packed words per lane per round
    constexpr int E = 32 * W;              // edges per round
    constexpr int U = E / G;               // loads per lane per round
    static_assert(U % 4 == 0, "edges are accumulated four at a time");
    const int grp = lane / L, sub = lane % L;
    const uint4* __restrict__ Q16 = reinterpret_cast<const uint4*>(Q);
    const uint32_t start = __ldg(rows + s), end = __ldg(rows + s + 1);
    uint32_t nbn[W];
    int cn[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
        nbn[w] = 0u;
        cn[w] = 0;
        const uint32_t e = start + uint32_t(w * 32 + lane);
        if (e < end) edge_word_i(packed, edges, e, nb_bits, nbn[w], cn[w]);
    }
    for (uint32_t base = start; base < end; base += E) {
        uint32_t nbv[W];
        int cv[W];
#pragma unroll
        for (int w = 0; w < W; ++w) {
            nbv[w] = nbn[w];
            cv[w] = cn[w];
            nbn[w] = 0u;
            cn[w] = 0;
            const uint32_t e = base + uint32_t(E + w * 32 + lane);
            if (e < end) edge_word_i(packed, edges, e, nb_bits, nbn[w], cn[w]);
        }
        uint4 q[U];
        int c[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int src = (u * G + grp) & 31;
            const uint32_t nb = __shfl_sync(0xffffffffu, nbv[(u * G) >> 5], src);
            c[u] = __shfl_sync(0xffffffffu, cv[(u * G) >> 5], src);
            if (base + uint32_t(u * G + grp) < end) {
                q[u] = __ldcg(Q16 + size_t(nb) * L + sub);  // L2 only: rows rarely repeat in L1
            } else {
                q[u] = make_uint4(0u, 0u, 0u, 0u);
                c[u] = 0;
            }
        }
        // Four edges at a time: transpose their 4 x 4 byte blocks so that
        // one register holds one column's four values, then one dp4a adds
        // value x count for all four (counts packed as unsigned bytes).  A
        // packed word's count is below 2^(32 - nb_bits) <= 2^10; the rare
        // counts above 255 (and any 32-bit count of an unpacked graph) add
        // their higher bytes in further warp-uniform passes, which keeps the
        // sums equal to the 32-bit products.
        uint32_t cor = 0u;
#pragma unroll
        for (int u = 0; u < U; ++u) cor |= uint32_t(c[u]);
        const uint32_t call = __reduce_or_sync(0xffffffffu, cor);
#pragma unroll
        for (int h = 0; h < U; h += 4) {
            const uint32_t lo = pack_bytes(c[h], c[h + 1], c[h + 2], c[h + 3], 0);
            const uint32_t e0[4] = {q[h].x, q[h].y, q[h].z, q[h].w};
            const uint32_t e1[4] = {q[h + 1].x, q[h + 1].y, q[h + 1].z, q[h + 1].w};
            const uint32_t e2[4] = {q[h + 2].x, q[h + 2].y, q[h + 2].z, q[h + 2].w};
            const uint32_t e3[4] = {q[h + 3].x, q[h + 3].y, q[h + 3].z, q[h + 3].w};
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                uint32_t t[4];
                transpose4(e0[i], e1[i], e2[i], e3[i], t);
#pragma unroll
                for (int k = 0; k < 4; ++k) acc[4 * i + k] = dp4a_su(t[k], lo, acc[4 * i + k]);
                for (int sh = 8; sh < 32 && (call >> sh) != 0u; sh += 8) {
                    const uint32_t cb = pack_bytes(c[h], c[h + 1], c[h + 2], c[h + 3], sh);
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        acc[4 * i + k] += int(uint32_t(dp4a_su(t[k], cb, 0)) << sh);
                }
            }
        }
    }
}

// Sum the G groups' partial sums and scatter: afterwards a[0 .. 16 / G) of
// lane (grp, sub) are the totals of columns sub * 16 + i8_offset<G>(grp) + i.
template <int G, int L>
__device__ __forceinline__ void reduce_scatter_i8(int* a, int lane)
{
    const int grp = lane / L;
#pragma unroll
    for (int lvl = 0; (1 << lvl) < G; ++lvl) {
        const bool hi = ((grp >> lvl) & 1) != 0;
        const int half = 16 >> (lvl + 1);
#pragma unroll
        for (int i = 0; i < half; ++i) {
            const int send = hi ? a[i] : a[i + half];
            const int keep = hi ? a[i + half] : a[i];
            a[i] = keep + __shfl_xor_sync(0xffffffffu, send, L << lvl);
        }
    }
}

template <int G>
__device__ __forceinline__ int i8_offset(int grp)
{
    int off = 0;
#pragma unroll
    for (int lvl = 0; (1 << lvl) < G; ++lvl) off += ((grp >> lvl) & 1) * (16 >> (lvl + 1));
    return off;
}

// Per-cell planes of the int8 step (rho, tau, X, R) are read and written
// once per step: streaming loads and stores (evict first), so that L2 keeps
// the gathered int8 rows.  The gather itself loads through L2 only (__ldcg)
// and the packed edge words stream (__ldcs): 4 % faster at 64 columns on
// the config-2 forest than plain loads.
template <int N> struct VecN;
template <> struct VecN<1> {
    static __device__ __forceinline__ void ld(const float* p, float* v) { v[0] = __ldcs(p); }
    static __device__ __forceinline__ void st(float* p, const float* v) { __stcs(p, v[0]); }
    static __device__ __forceinline__ void ldq(const int8_t* p, int* v) { v[0] = *p; }
    static __device__ __forceinline__ void stq(int8_t* p, const int* v) { *p = int8_t(v[0]); }
};
template <> struct VecN<2> {
    static __device__ __forceinline__ void ld(const float* p, float* v)
    {
        const float2 q = __ldcs(reinterpret_cast<const float2*>(p));
        v[0] = q.x;
        v[1] = q.y;
    }
    static __device__ __forceinline__ void st(float* p, const float* v)
    {
        __stcs(reinterpret_cast<float2*>(p), make_float2(v[0], v[1]));
    }
    static __device__ __forceinline__ void ldq(const int8_t* p, int* v)
    {
        const char2 q = *reinterpret_cast<const char2*>(p);
        v[0] = q.x;
        v[1] = q.y;
    }
    static __device__ __forceinline__ void stq(int8_t* p, const int* v)
    {
        *reinterpret_cast<char2*>(p) = make_char2(char(v[0]), char(v[1]));
    }
};
template <> struct VecN<4> {
    static __device__ __forceinline__ void ld(const float* p, float* v)
    {
        const float4 q = __ldcs(reinterpret_cast<const float4*>(p));
        v[0] = q.x;
        v[1] = q.y;
        v[2] = q.z;
        v[3] = q.w;
    }
    static __device__ __forceinline__ void st(float* p, const float* v)
    {
        __stcs(reinterpret_cast<float4*>(p), make_float4(v[0], v[1], v[2], v[3]));
    }
    static __device__ __forceinline__ void ldq(const int8_t* p, int* v)
    {
        const char4 q = *reinterpret_cast<const char4*>(p);
        v[0] = q.x;
        v[1] = q.y;
        v[2] = q.z;
        v[3] = q.w;
    }
    static __device__ __forceinline__ void stq(int8_t* p, const int* v)
    {
        *reinterpret_cast<char4*>(p) = make_char4(char(v[0]), char(v[1]), char(v[2]), char(v[3]));
    }
};

template <int P, bool Scenes>
__global__ void __launch_bounds__(kWarps * 32, StepBlocks<P>::value) k_step_i8(
    GraphView g, PanelParams pp, const int8_t* __restrict__ Qin, int8_t* __restrict__ Qout,
    float* __restrict__ X, float* __restrict__ R, const float* __restrict__ sig_in,
    const float* __restrict__ sig_out, uint32_t* stats, uint32_t* counter, const uint32_t* done,
    const float* __restrict__ scene_sig_in, const float* __restrict__ scene_sig_out)
{
    if (*done) return;
    constexpr int L = P / 16, G = 32 / L, NC = P / 32;
    const int lane = threadIdx.x & 31;
    const int col0 = (lane % L) * 16 + i8_offset<G>(lane / L);
    float si[NC], inv_so[NC], md[NC], mb[NC], mr[NC], om[NC], fl[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        si[k] = sig_in[col0 + k];
        const float so = sig_out[col0 + k];
        inv_so[k] = so > 0.0f ? 1.0f / so : 0.0f;
        om[k] = pp.omega ? pp.omega[col0 + k] : 1.0f;
        fl[k] = kSideFloor * pp.colmax[col0 + k];
        md[k] = 0.0f;
        mb[k] = 0.0f;
        mr[k] = 0.0f;
    }
    // Scene batches: each scene steps with its own int8 scales (a scale set
    // by another scene's larger residual would round this scene's steps to
    // zero), its worst per-side ratio and max |R| are gathered while the
    // warp stays in that scene, and the facets of a converged scene are
    // skipped.
    uint32_t cur = 0xffffffffu;
    float ms[NC], mq[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        ms[k] = 0.0f;
        mq[k] = 0.0f;
    }
    auto flush = [&]() {
        if (Scenes && cur != 0xffffffffu) {
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                atomicMax(g.scene_stats + size_t(cur) * kMaxP + col0 + k, __float_as_uint(ms[k]));
                atomicMax(g.scene_md + size_t(cur) * kMaxP + col0 + k, __float_as_uint(mq[k]));
            }
        }
    };
    for_each_facet<Scenes ? kSceneChunk : kChunk>(g.facets, counter, lane, [&](uint32_t f) {
        if (Scenes) {
            const uint32_t sc = __ldg(g.scene + f);
            if (g.scene_done[sc]) return;
            if (sc != cur) {
                flush();
                cur = sc;
#pragma unroll
                for (int k = 0; k < NC; ++k) {
                    ms[k] = 0.0f;
                    mq[k] = 0.0f;
                    si[k] = scene_sig_in[size_t(sc) * kMaxP + col0 + k];
                    const float so = scene_sig_out[size_t(sc) * kMaxP + col0 + k];
                    inv_so[k] = so > 0.0f ? 1.0f / so : 0.0f;
                    om[k] = g.scene_cheb[size_t(sc) * 4 * kMaxP + 2 * kMaxP + col0 + k];
                }
            }
        }
        {
            float h[2][NC];
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                const uint32_t s = 2u * f + side;
                int acc[16];
#pragma unroll
                for (int k = 0; k < 16; ++k) acc[k] = 0;
                gather_i8<P>(g.rows, g.packed, g.edges, g.nb_bits, s, Qin, lane, acc);
                reduce_scatter_i8<G, L>(acc, lane);
                const uint32_t d = __ldg(g.denom + s);
                const float inv = d ? 1.0f / float(d) : 0.0f;
#pragma unroll
                for (int k = 0; k < NC; ++k) h[side][k] = float(acc[k]) * si[k] * inv;
            }
            const size_t i0 = size_t(2u * f) * P + col0, i1 = i0 + P;
            float r0[NC], r1[NC], t0[NC], t1[NC], x0[NC], x1[NC], e0[NC], e1[NC];
            int q0[NC], q1[NC];
            VecN<NC>::ld(pp.rho + i0, r0);
            VecN<NC>::ld(pp.rho + i1, r1);
            VecN<NC>::ld(pp.tau + i0, t0);
            VecN<NC>::ld(pp.tau + i1, t1);
            VecN<NC>::ld(X + i0, x0);
            VecN<NC>::ld(X + i1, x1);
            VecN<NC>::ld(R + i0, e0);
            VecN<NC>::ld(R + i1, e1);
            VecN<NC>::ldq(Qin + i0, q0);
            VecN<NC>::ldq(Qin + i1, q1);
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                const float kd0 = r0[k] * h[0][k] + t0[k] * h[1][k];
                const float kd1 = r1[k] * h[1][k] + t1[k] * h[0][k];
                const float dl0 = si[k] * float(q0[k]), dl1 = si[k] * float(q1[k]);
                x0[k] += dl0;
                x1[k] += dl1;
                e0[k] = e0[k] - dl0 + kd0;
                e1[k] = e1[k] - dl1 + kd1;
                // next step: omega R + (omega - 1) delta (omega = 1: the residual)
                const float n0 = om[k] * e0[k] + (om[k] - 1.0f) * dl0;
                const float n1 = om[k] * e1[k] + (om[k] - 1.0f) * dl1;
                q0[k] = max(-127, min(127, __float2int_rn(n0 * inv_so[k])));
                q1[k] = max(-127, min(127, __float2int_rn(n1 * inv_so[k])));
                md[k] = fmaxf(md[k], fmaxf(fabsf(e0[k]), fabsf(e1[k])));
                mb[k] = fmaxf(mb[k], fmaxf(fabsf(x0[k]), fabsf(x1[k])));
                // per-side test on the exact residual: R is the change the
                // next Jacobi sweep would make
                mr[k] = fmaxf(mr[k], fmaxf(__fdividef(fabsf(e0[k]), fmaxf(fabsf(x0[k]), fl[k])),
                                           __fdividef(fabsf(e1[k]), fmaxf(fabsf(x1[k]), fl[k]))));
                if (Scenes) {
                    // a zero residual passes (the column test's md == 0 case)
                    const float a0 = fabsf(e0[k]) > 0.0f
                                         ? __fdividef(fabsf(e0[k]), fmaxf(fabsf(x0[k]), fl[k]))
                                         : 0.0f;
                    const float a1 = fabsf(e1[k]) > 0.0f
                                         ? __fdividef(fabsf(e1[k]), fmaxf(fabsf(x1[k]), fl[k]))
                                         : 0.0f;
                    ms[k] = fmaxf(ms[k], fmaxf(a0, a1));
                    mq[k] = fmaxf(mq[k], fmaxf(fabsf(e0[k]), fabsf(e1[k])));
                }
            }
            VecN<NC>::st(X + i0, x0);
            VecN<NC>::st(X + i1, x1);
            VecN<NC>::st(R + i0, e0);
            VecN<NC>::st(R + i1, e1);
            VecN<NC>::stq(Qout + i0, q0);
            VecN<NC>::stq(Qout + i1, q1);
        }
    });
    flush();
    publish_cols<NC>(md, mb, mr, col0, true, P, stats);
}

// ---- the 64-column int8 step as an asynchronous-copy pipeline --------------
// The same step as k_step_i8<64, false> (bit-identical X, R, Q and
// statistics: the gathered sums are exact int32), restructured so that each
// warp keeps neighbour rows in flight while it computes.  A warp walks the
// rows of its facets as a sequence of 64-edge stages (a side's last stage
// may be partial; an empty side is one empty stage) with three cursors:
//   request — kLookahead stages ahead of issue: writes the stage's
//             descriptor (side, last-stage flag, denominator, edges) to
//             shared memory and loads its 32 packed edge words into a
//             register queue;
//   issue   — kAsyncStages - 1 stages ahead of consume: 16-byte cp.async
//             copies (LDGSTS, L2 only) of the stage's neighbour rows into a
//             ring of kAsyncStages stages in shared memory, and its counts
//             (one byte each, packed per dp4a word: the kernel runs on the
//             solver's graph copy, whose counts are split at 255);
//   consume — 4 x 4 byte transposes and dp4a from shared memory; at a
//             side's last stage the reduction and (odd side) the facet's
//             epilogue.
// In-flight rows cost shared memory instead of registers, and the edge
// words are requested before their rows are, so neither the dp4a work nor
// the epilogue's loads stop the gather.  Facets come in chunks of kAsyncChunk
// from the step's counter; the request cursor takes its next chunk (and
// that chunk's row offsets and denominators) one chunk ahead, and asks L2
// for the next chunk's edge words and each chunk's per-cell planes
// (cp.async.bulk.prefetch) as it enters a chunk.  Measured on GB300 with a
// 64-byte row gather of the bench's size: tile::gather4 TMA loads peak at
// 0.52 ms (the TMA unit's rate for 256-byte requests), cp.async.bulk per
// row at 1.1 ms, LDGSTS rings at 0.30 ms, plain register loads at 0.31 ms.
#ifndef FCU_STEP_ASYNC
#define FCU_STEP_ASYNC 1
#endif
// Measured on the config-2 forest (203,840 facets, 64 columns; the register-gather
// kernel 0.619 ms): 64-edge stages, 2 ring stages, 1 stage of lookahead
// 0.527 ms; 2 of lookahead 0.608; 3 ring stages on 2 CTAs per SM 0.636;
// 32-edge stages with 4 ring stages 0.622 (their per-stage bookkeeping
// doubled the instructions per edge); 64-edge stages with 4 warps per CTA
// (6 CTAs per SM) 0.529; 128-edge stages with 4 or 2 warps 0.588-0.590
// (a 183-edge mean row fills 72 % of two 128-edge stages).  With three
// facets per chunk, CTA shapes (warps x CTAs per SM, registers per thread):
// 8 x 3 (80, spills) 0.488 ms; 8 x 2 (128) 0.474; 4 x 6 0.486; 12 x 2 0.496;
// 12 x 1 0.518; 16 x 1 (118) 0.466; 20 x 1 (96) 0.452; 22 x 1 (80, spills)
// 0.479; 24 x 1 0.494; 26 x 1 0.503; 16 x 1 with 3 ring stages 0.471, with 3
// stages and 2 of lookahead 0.478.  One CTA of 20 warps per SM: the most
// warps whose registers (96) hold the step without spills.
#ifndef FCU_ASYNC_STAGES
#define FCU_ASYNC_STAGES 2
#endif
#ifndef FCU_ASYNC_LOOKAHEAD
#define FCU_ASYNC_LOOKAHEAD 1
#endif
#ifndef FCU_ASYNC_BLOCKS
#define FCU_ASYNC_BLOCKS 1
#endif
#ifndef FCU_ASYNC_EDGES
#define FCU_ASYNC_EDGES 64
#endif
#ifndef FCU_ASYNC_WARPS
#define FCU_ASYNC_WARPS 20
#endif
constexpr int kAsyncWarps = FCU_ASYNC_WARPS;  // warps per CTA of the pipelined step (64 columns)
// At 128 columns a stage holds 8 KB of rows: 4 warps per CTA, 3 CTAs per SM
// (measured on the config-2 forest with two suns: 0.788 ms; 6 x 2 0.790,
// 12 x 1 0.793, 10 x 1 0.835, 8 x 1 0.901).
#ifndef FCU_ASYNC_WARPS_128
#define FCU_ASYNC_WARPS_128 4
#endif
#ifndef FCU_ASYNC_BLOCKS_128
#define FCU_ASYNC_BLOCKS_128 3
#endif
template <int P> struct AsyncWarps {
    static constexpr int value = P == 128 ? FCU_ASYNC_WARPS_128 : kAsyncWarps;
    static constexpr int blocks = P == 128 ? FCU_ASYNC_BLOCKS_128 : FCU_ASYNC_BLOCKS;  // min CTAs per SM
};
constexpr int kAsyncStages = FCU_ASYNC_STAGES;
constexpr int kLookahead = FCU_ASYNC_LOOKAHEAD;
constexpr int kStageEdges = FCU_ASYNC_EDGES;  // 32, 64 or 128 edges per stage
// Facets per hand-out of the pipelined step (single scenes): the request
// cursor takes chunks one ahead, so a chunk's row offsets and the L2
// prefetches of its planes serve its C facets.  Measured on the config-2
// forest: 1 facet 0.512 ms, 2 0.497, 3 0.488, 4 0.501, 5 0.497, 6 0.505,
// 8 0.535.
#ifndef FCU_ASYNC_CHUNK
#define FCU_ASYNC_CHUNK 3
#endif
constexpr uint32_t kAsyncChunk = FCU_ASYNC_CHUNK;

constexpr int pow2_at_least(int n) { return n <= 1 ? 1 : 2 * pow2_at_least((n + 1) / 2); }

template <int P>
struct AsyncLayout {
    static constexpr int kStageBytes = kStageEdges * P;  // int8 rows of one stage
    // a stage's counts, one byte per edge packed for the dp4a (the solver's
    // graph copy holds no count above 255)
    static constexpr int kCountBytes = kStageEdges;
    // descriptor slots (a power of two, at least stages + lookahead)
    static constexpr int kDesc = pow2_at_least(kAsyncStages + kLookahead);
    // per warp: the row ring, the counts of each ring stage, the descriptors
    static constexpr int kWarpBytes = kAsyncStages * (kStageBytes + kCountBytes) + kDesc * 16;
    static constexpr int kBlockBytes = AsyncWarps<P>::value * kWarpBytes;
};

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return uint32_t(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit()
{
    asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N> __device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
// Asynchronous prefetch of `bytes` (a multiple of 16, 16-byte aligned) into L2.
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

template <int P, bool Scenes>
__global__ void __launch_bounds__(AsyncWarps<P>::value * 32, AsyncWarps<P>::blocks) k_step_i8_async(
    GraphView g, PanelParams pp, const int8_t* __restrict__ Qin, int8_t* __restrict__ Qout,
    float* __restrict__ X, float* __restrict__ R, const float* __restrict__ sig_in,
    const float* __restrict__ sig_out, uint32_t* stats, uint32_t* counter, const uint32_t* done,
    const float* __restrict__ scene_sig_in, const float* __restrict__ scene_sig_out)
{
    static_assert(P == 64 || P == 128, "the pipelined step covers 64- and 128-column panels");
    constexpr int W = AsyncWarps<P>::value;
    using Lay = AsyncLayout<P>;
    constexpr int L = P / 16, G = 32 / L, NC = P / 32;
    constexpr int SE = kStageEdges;
    constexpr int WPL = SE / 32;       // packed edge words per lane per stage
    constexpr int EPL = SE / G;        // edges per lane per stage
    constexpr int CPL = SE * L / 32;   // 16-byte copies per lane per stage
    constexpr int NST = kAsyncStages, D = kLookahead, NQ = Lay::kDesc;
    constexpr uint32_t C = Scenes ? kSceneChunk : kAsyncChunk;
    static_assert(2 * C + 1 <= 32, "a chunk's row offsets fit one warp");
    constexpr unsigned kAll = 0xffffffffu;
    static_assert(SE == 32 || SE == 64 || SE == 128, "32, 64 or 128 edges per stage");
    static_assert(Lay::kBlockBytes >= 3 * W * P * 4, "the statistics reuse the rings");
    static_assert(EPL % 4 == 0 && (G == 8 || G == 4), "4 x 4 transpose blocks, 8 or 4 edge groups");
    static_assert(NST >= 2 && D >= 1, "pipeline depths");
    extern __shared__ __align__(16) unsigned char dyn[];
    if (*done) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int grp = lane / L, sub = lane % L;
    unsigned char* ring = dyn + size_t(warp) * Lay::kWarpBytes;
    unsigned char* cnt_s = ring + NST * Lay::kStageBytes;  // [NST][kCountBytes]
    uint4* meta = reinterpret_cast<uint4*>(cnt_s + NST * Lay::kCountBytes);

    const int col0 = sub * 16 + i8_offset<G>(grp);
    float si[NC], inv_so[NC], md[NC], mb[NC], mr[NC], om[NC], fl[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        si[k] = sig_in[col0 + k];
        const float so = sig_out[col0 + k];
        inv_so[k] = so > 0.0f ? 1.0f / so : 0.0f;
        om[k] = pp.omega ? pp.omega[col0 + k] : 1.0f;
        fl[k] = kSideFloor * pp.colmax[col0 + k];
        md[k] = 0.0f;
        mb[k] = 0.0f;
        mr[k] = 0.0f;
    }

    // Scene batches: each scene steps with its own int8 scales and Chebyshev
    // weight, the facets of a converged scene get no stages, and the
    // scene's worst per-side ratio and max |R| are gathered while the warp
    // stays in that scene (flushed with atomics when it moves on), as in
    // k_step_i8<P, true>.
    uint32_t cur = 0xffffffffu;
    float ms[NC], mq[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        ms[k] = 0.0f;
        mq[k] = 0.0f;
    }
    auto flush = [&]() {
        if (Scenes && cur != 0xffffffffu) {
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                atomicMax(g.scene_stats + size_t(cur) * kMaxP + col0 + k, __float_as_uint(ms[k]));
                atomicMax(g.scene_md + size_t(cur) * kMaxP + col0 + k, __float_as_uint(mq[k]));
            }
        }
    };

    // ---- request cursor: chunks, sides, stages ---------------------------
    const uint32_t F = g.facets;
    const uint32_t chunks = (F + C - 1) / C;
    const uint32_t nb_mask = (1u << g.nb_bits) - 1u;
    const size_t word_bytes = (size_t(__ldg(g.rows + 2u * F)) * 4u) & ~size_t(15);  // prefetch bound
    // a chunk: its id, and in lane i its side i's row start (lanes 0..sides)
    // and denominator (lanes 0..sides-1); with scenes, in lane i facet i's
    // scene and whether that scene is done
    auto grab = [&](uint32_t& id, uint32_t& rw, uint32_t& dn, uint32_t& sc, uint32_t& fd) {
        id = next_chunk(counter, lane);
        rw = 0u;
        dn = 0u;
        sc = 0u;
        fd = 0u;
        if (id < chunks) {
            const uint32_t s0 = 2u * id * C, ns = 2u * (min(F, (id + 1u) * C) - id * C);
            if (uint32_t(lane) <= ns) rw = __ldg(g.rows + s0 + lane);
            if (uint32_t(lane) < ns) dn = __ldg(g.denom + s0 + lane);
            if (Scenes && uint32_t(lane) < ns / 2u) {
                sc = __ldg(g.scene + id * C + lane);
                fd = g.scene_done[sc];
            }
        }
    };
    uint32_t r_id, r_rw, r_dn, r_sc, r_fd, n_id, n_rw, n_dn, n_sc, n_fd;
    grab(r_id, r_rw, r_dn, r_sc, r_fd);
    grab(n_id, n_rw, n_dn, n_sc, n_fd);
    bool rdone = r_id >= chunks;
    uint32_t r_side = 0, r_ns = 0, r_e = 0, r_end = 0;
    // Entering chunk r_id (its row offsets were loaded a chunk ago): its
    // first side, and L2 prefetches of its per-cell planes for its epilogues.
    auto start_chunk = [&]() {
        const uint32_t f0 = r_id * C;
        r_ns = 2u * (min(F, f0 + C) - f0);
        r_side = 0;
        r_e = __shfl_sync(kAll, r_rw, 0);
        r_end = __shfl_sync(kAll, r_rw, 1);
        if (lane == 0) {
            const size_t c0 = size_t(2u * f0) * P;
            const uint32_t bytes = r_ns * P * 4u;
            prefetch_l2(pp.rho + c0, bytes);
            prefetch_l2(pp.tau + c0, bytes);
            prefetch_l2(X + c0, bytes);
            prefetch_l2(R + c0, bytes);
            prefetch_l2(Qin + c0, r_ns * P);
        }
    };
    // L2 prefetch of the next chunk's edge words, once its row offsets have
    // arrived (at the current chunk's second side).
    bool words_pending = true;
    auto prefetch_words = [&]() {
        words_pending = false;
        if (n_id >= chunks) return;
        const uint32_t nns = 2u * (min(F, (n_id + 1u) * C) - n_id * C);
        const uint32_t nb0 = __shfl_sync(kAll, n_rw, 0);
        const uint32_t nb1 = __shfl_sync(kAll, n_rw, int(nns));
        const size_t b0 = (size_t(nb0) * 4u) & ~size_t(15);
        const size_t b1 = min(word_bytes, (size_t(nb1) * 4u + 15u) & ~size_t(15));
        if (lane == 0 && b1 > b0)
            prefetch_l2(reinterpret_cast<const unsigned char*>(g.packed) + b0, uint32_t(b1 - b0));
    };
    if (!rdone) start_chunk();

    uint32_t wf[D][WPL];  // packed edge words of the requested, not yet issued stages
    uint32_t nf[D];       // their edge counts
    uint32_t requested = 0, issued = 0, consumed = 0;
    // Request the next stage: its descriptor goes to meta[stage % NQ], its
    // words (0 past the stage's edges) to the back of the queue.
    // The cursor's next side (side r_side + 1, or the next chunk's first).
    auto next_side = [&]() {
        ++r_side;
        if (r_side == r_ns) {
            r_id = n_id;
            r_rw = n_rw;
            r_dn = n_dn;
            r_sc = n_sc;
            r_fd = n_fd;
            if (r_id >= chunks) {
                rdone = true;
            } else {
                start_chunk();
                grab(n_id, n_rw, n_dn, n_sc, n_fd);
                words_pending = true;
            }
        } else {
            r_e = __shfl_sync(kAll, r_rw, int(r_side));
            r_end = __shfl_sync(kAll, r_rw, int(r_side) + 1);
            if (words_pending) prefetch_words();
        }
    };
    auto request = [&]() {
        uint32_t w[WPL], n = 0u;
#pragma unroll
        for (int j = 0; j < WPL; ++j) w[j] = 0u;
        if constexpr (Scenes) {
            // a converged scene's facets get no stages
            while (!rdone && (r_side & 1u) == 0u &&
                   __shfl_sync(kAll, r_fd, int(r_side >> 1)) != 0u) {
                next_side();
                if (!rdone) next_side();
            }
        }
        if (!rdone) {
            n = min(uint32_t(kStageEdges), r_end - r_e);
            const bool last = r_e + n == r_end;
            const uint32_t dn = __shfl_sync(kAll, r_dn, int(r_side));
            const uint32_t sc = Scenes ? __shfl_sync(kAll, r_sc, int(r_side >> 1)) : 0u;
            if (lane == 0)
                meta[requested & (NQ - 1)] = make_uint4(2u * r_id * C + r_side, last ? 1u : 0u, dn, sc);
#pragma unroll
            for (int j = 0; j < WPL; ++j)
                if (uint32_t(j * 32 + lane) < n) w[j] = __ldcs(g.packed + r_e + j * 32 + lane);
            ++requested;
            r_e += n;
            if (last) next_side();
        }
#pragma unroll
        for (int k = 0; k < D - 1; ++k) {
#pragma unroll
            for (int j = 0; j < WPL; ++j) wf[k][j] = wf[k + 1][j];
            nf[k] = nf[k + 1];
        }
#pragma unroll
        for (int j = 0; j < WPL; ++j) wf[D - 1][j] = w[j];
        nf[D - 1] = n;
    };
    // Issue the oldest requested stage (front of the queue): its counts and
    // row copies into ring slot issued % NST, as one copy group.
    // Edge e = k * G + grp of a stage is the k-th edge of lane group grp:
    // its count goes to byte k % 4 of word (k / 4) * G + grp, the word one
    // dp4a of that group uses.  Lane l holds edges j * 32 + l, so
    // k = (32 / G) j + l / G and the byte is 32 j + cnt_byte (G = 8 or 4).
    const int cnt_byte = 4 * G * ((lane / G) / 4) + 4 * (lane % G) + (lane / G) % 4;
    const unsigned char* qsrc = reinterpret_cast<const unsigned char*>(Qin) + sub * 16;
    auto issue = [&]() {
        if (issued < requested) {
            const int slot = int(issued % NST);
            const uint32_t n = nf[0];
            uint32_t nb[WPL];
            unsigned char* cs = cnt_s + slot * Lay::kCountBytes;
#pragma unroll
            for (int j = 0; j < WPL; ++j) {
                nb[j] = wf[0][j] & nb_mask;
                cs[j * 32 + cnt_byte] = static_cast<unsigned char>(wf[0][j] >> g.nb_bits);
            }
            unsigned char* dst = ring + slot * Lay::kStageBytes + sub * 16;
#pragma unroll
            for (int k = 0; k < CPL; ++k) {
                const int row = k * G + grp;  // row / 32 == k G / 32
                const uint32_t rn = __shfl_sync(kAll, nb[(k * G) / 32], row & 31);
                if (uint32_t(row) < n) cp_async16(dst + row * P, qsrc + size_t(rn) * P);
            }
            ++issued;
        }
        cp_async_commit();
    };

    // ---- consumer ----------------------------------------------------------
    int acc[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) acc[k] = 0;
    float h0[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) h0[k] = 0.0f;

    auto consume = [&]() {
        const int slot = int(consumed % NST);
        const uint4 mt = meta[consumed & (NQ - 1)];
        const unsigned char* cs = cnt_s + slot * Lay::kCountBytes;
        const uint4* rows = reinterpret_cast<const uint4*>(ring + slot * Lay::kStageBytes);
#pragma unroll
        for (int blk = 0; blk < EPL / 4; ++blk) {
            uint4 q[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) q[k] = rows[((blk * 4 + k) * G + grp) * L + sub];
            const uint32_t lo = reinterpret_cast<const uint32_t*>(cs)[blk * G + grp];
            const uint32_t e0[4] = {q[0].x, q[0].y, q[0].z, q[0].w};
            const uint32_t e1[4] = {q[1].x, q[1].y, q[1].z, q[1].w};
            const uint32_t e2[4] = {q[2].x, q[2].y, q[2].z, q[2].w};
            const uint32_t e3[4] = {q[3].x, q[3].y, q[3].z, q[3].w};
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                uint32_t t[4];
                transpose4(e0[i], e1[i], e2[i], e3[i], t);
#pragma unroll
                for (int k = 0; k < 4; ++k) acc[4 * i + k] = dp4a_su(t[k], lo, acc[4 * i + k]);
            }
        }
        ++consumed;
        if (!mt.y) return;
        // the side's last stage: sums, then (odd side) the facet's update
        if constexpr (Scenes) {
            if (mt.w != cur) {
                flush();
                cur = mt.w;
#pragma unroll
                for (int k = 0; k < NC; ++k) {
                    ms[k] = 0.0f;
                    mq[k] = 0.0f;
                    si[k] = scene_sig_in[size_t(cur) * kMaxP + col0 + k];
                    const float so = scene_sig_out[size_t(cur) * kMaxP + col0 + k];
                    inv_so[k] = so > 0.0f ? 1.0f / so : 0.0f;
                    om[k] = g.scene_cheb[size_t(cur) * 4 * kMaxP + 2 * kMaxP + col0 + k];
                }
            }
        }
        reduce_scatter_i8<G, L>(acc, lane);
        const float inv = mt.z ? 1.0f / float(mt.z) : 0.0f;
        float h[NC];
#pragma unroll
        for (int k = 0; k < NC; ++k) h[k] = float(acc[k]) * si[k] * inv;
#pragma unroll
        for (int k = 0; k < 16; ++k) acc[k] = 0;
        if ((mt.x & 1u) == 0u) {
#pragma unroll
            for (int k = 0; k < NC; ++k) h0[k] = h[k];
            return;
        }
        const uint32_t f = mt.x >> 1;
        const size_t i0 = size_t(2u * f) * P + col0, i1 = i0 + P;
        float r0[NC], r1[NC], t0[NC], t1[NC], x0[NC], x1[NC], s0[NC], s1[NC];
        int q0[NC], q1[NC];
        VecN<NC>::ld(pp.rho + i0, r0);
        VecN<NC>::ld(pp.rho + i1, r1);
        VecN<NC>::ld(pp.tau + i0, t0);
        VecN<NC>::ld(pp.tau + i1, t1);
        VecN<NC>::ld(X + i0, x0);
        VecN<NC>::ld(X + i1, x1);
        VecN<NC>::ld(R + i0, s0);
        VecN<NC>::ld(R + i1, s1);
        VecN<NC>::ldq(Qin + i0, q0);
        VecN<NC>::ldq(Qin + i1, q1);
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            const float kd0 = r0[k] * h0[k] + t0[k] * h[k];
            const float kd1 = r1[k] * h[k] + t1[k] * h0[k];
            const float dl0 = si[k] * float(q0[k]), dl1 = si[k] * float(q1[k]);
            x0[k] += dl0;
            x1[k] += dl1;
            s0[k] = s0[k] - dl0 + kd0;
            s1[k] = s1[k] - dl1 + kd1;
            const float n0 = om[k] * s0[k] + (om[k] - 1.0f) * dl0;
            const float n1 = om[k] * s1[k] + (om[k] - 1.0f) * dl1;
            q0[k] = max(-127, min(127, __float2int_rn(n0 * inv_so[k])));
            q1[k] = max(-127, min(127, __float2int_rn(n1 * inv_so[k])));
            md[k] = fmaxf(md[k], fmaxf(fabsf(s0[k]), fabsf(s1[k])));
            mb[k] = fmaxf(mb[k], fmaxf(fabsf(x0[k]), fabsf(x1[k])));
            mr[k] = fmaxf(mr[k], fmaxf(__fdividef(fabsf(s0[k]), fmaxf(fabsf(x0[k]), fl[k])),
                                       __fdividef(fabsf(s1[k]), fmaxf(fabsf(x1[k]), fl[k]))));
            if (Scenes) {
                // a zero residual passes (the column test's md == 0 case)
                const float a0 = fabsf(s0[k]) > 0.0f
                                     ? __fdividef(fabsf(s0[k]), fmaxf(fabsf(x0[k]), fl[k]))
                                     : 0.0f;
                const float a1 = fabsf(s1[k]) > 0.0f
                                     ? __fdividef(fabsf(s1[k]), fmaxf(fabsf(x1[k]), fl[k]))
                                     : 0.0f;
                ms[k] = fmaxf(ms[k], fmaxf(a0, a1));
                mq[k] = fmaxf(mq[k], fmaxf(fabsf(s0[k]), fabsf(s1[k])));
            }
        }
        VecN<NC>::st(X + i0, x0);
        VecN<NC>::st(X + i1, x1);
        VecN<NC>::st(R + i0, s0);
        VecN<NC>::st(R + i1, s1);
        VecN<NC>::stq(Qout + i0, q0);
        VecN<NC>::stq(Qout + i1, q1);
    };

    // ---- the pipeline --------------------------------------------------------
    // Issue step j commits copy group j (empty once the facets run out), so
    // waiting until at most NST - 1 newer groups are pending completes the
    // stage about to be consumed.  Stage k's descriptor was written D issue
    // steps before it is issued and NST - 1 + D before it is consumed; its
    // slot (k % NQ) is rewritten only after stage k was consumed.
#pragma unroll
    for (int k = 0; k < D; ++k) request();
    __syncwarp();
#pragma unroll 1
    for (int k = 0; k < NST - 1; ++k) {
        issue();
        request();
        __syncwarp();
    }
#pragma unroll 1
    while (consumed < issued) {
        issue();
        request();
        cp_async_wait<NST - 1>();
        __syncwarp();
        consume();
        __syncwarp();
    }
    cp_async_wait<0>();
    flush();

    // ---- statistics: CTA max per column, one atomic per column -------------
    __syncthreads();  // every warp is done with its ring
    float* s_md = reinterpret_cast<float*>(dyn);
    float* s_mb = s_md + W * P;
    float* s_mr = s_mb + W * P;
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        s_md[warp * P + col0 + k] = md[k];
        s_mb[warp * P + col0 + k] = mb[k];
        s_mr[warp * P + col0 + k] = mr[k];
    }
    __syncthreads();
    for (int c = threadIdx.x; c < P; c += blockDim.x) {
        float a = 0.0f, b = 0.0f, r = 0.0f;
        for (int w = 0; w < W; ++w) {
            a = fmaxf(a, s_md[w * P + c]);
            b = fmaxf(b, s_mb[w * P + c]);
            r = fmaxf(r, s_mr[w * P + c]);
        }
        atomicMax(stats + c, __float_as_uint(a));
        atomicMax(stats + kMaxP + c, __float_as_uint(b));
        atomicMax(stats + 2 * kMaxP + c, __float_as_uint(r));
    }
}

__device__ __forceinline__ float cheb_advance(float* cheb, int c, int mode, float md);

// After an int8 step of a scene batch: a scene whose worst per-side ratio is
// within the tolerance in every column is done (its facets are skipped by
// the following steps); the others advance their own Chebyshev schedule
// (their own spectral-radius estimate, as if solved alone) and get the scale
// of their step after next from their own max |R|, as the column check forms
// them for the whole panel.  The step records are cleared for the next step.
__global__ void k_scene_check(uint32_t* ratio, uint32_t* mdr, float* sig_write,
                              const float* sig_prev, uint32_t* done, float* cheb, int P,
                              float tol)
{
    __shared__ int bad;
    const uint32_t sc = blockIdx.x;
    const uint32_t c = threadIdx.x;
    if (c == 0) bad = 0;
    __syncthreads();
    if (c < uint32_t(P)) {
        const size_t i = size_t(sc) * kMaxP + c;
        const float r = __uint_as_float(ratio[i]);
        const float md = __uint_as_float(mdr[i]);
        ratio[i] = 0u;
        mdr[i] = 0u;
        if (!(r <= tol)) bad = 1;
        if (!done[sc]) {
            const float w = cheb_advance(cheb + size_t(sc) * 4 * kMaxP, int(c), 2, md);
            float sigma = md / 127.0f;
            if (w != 1.0f) sigma = (w * md + (w - 1.0f) * 127.0f * sig_prev[i]) / 127.0f;
            sig_write[i] = sigma;
        }
    }
    __syncthreads();
    if (c == 0 && !bad) done[sc] = 1u;
}

// At the start of an int8 phase of a scene batch: max |Y - X| per scene and
// column (a block per run of sides, a thread per column), then the scenes'
// first scales.
__global__ void k_scene_init_md(const float* __restrict__ X, const float* __restrict__ Y,
                                const uint16_t* __restrict__ scene, uint32_t S, int P,
                                uint32_t* mdr)
{
    constexpr uint32_t kRun = 256;
    const uint32_t c = threadIdx.x;
    if (c >= uint32_t(P)) return;
    const uint32_t s0 = blockIdx.x * kRun, s1 = min(S, s0 + kRun);
    uint32_t cur = 0xffffffffu;
    float m = 0.0f;
    for (uint32_t sd = s0; sd < s1; ++sd) {
        const uint32_t sc = scene[sd >> 1];
        if (sc != cur) {
            if (cur != 0xffffffffu) atomicMax(mdr + size_t(cur) * kMaxP + c, __float_as_uint(m));
            cur = sc;
            m = 0.0f;
        }
        const size_t i = size_t(sd) * P + c;
        m = fmaxf(m, fabsf(Y[i] - X[i]));
    }
    if (cur != 0xffffffffu) atomicMax(mdr + size_t(cur) * kMaxP + c, __float_as_uint(m));
}

// both scale slots (step 0 reads slot 0 and writes with slot 1) and a fresh
// Chebyshev schedule per scene
__global__ void k_scene_init_sigma(uint32_t* mdr, float* sig, float* cheb, uint32_t scenes, int P)
{
    const size_t i = size_t(blockIdx.x) * kMaxP + threadIdx.x;
    if (threadIdx.x >= uint32_t(P)) return;
    const float md = __uint_as_float(mdr[i]);
    const float sigma = md / 127.0f;
    sig[i] = sigma;
    sig[size_t(scenes) * kMaxP + i] = sigma;
    cheb_advance(cheb + size_t(blockIdx.x) * 4 * kMaxP, int(threadIdx.x), 1, md);
    mdr[i] = 0u;
}

// R = Y - X and Q = round(R / sigma) for the first int8 step (X unchanged).
__global__ void k_init_i8(const float* __restrict__ X, const float* __restrict__ Y,
                          float* __restrict__ R, int8_t* __restrict__ Q,
                          const float* __restrict__ sig, size_t n, int P, uint32_t* it_dev,
                          uint32_t it, const uint16_t* __restrict__ scene = nullptr,
                          const float* __restrict__ scene_sig = nullptr)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i == 0) *it_dev = it;  // sweep index of the first step's check
    if (i >= n) return;
    const float r = Y[i] - X[i];
    const size_t c = i % size_t(P);
    const float sg = scene ? scene_sig[size_t(scene[(i / size_t(P)) >> 1]) * kMaxP + c] : sig[c];
    R[i] = r;
    Q[i] = int8_t(sg > 0.0f ? max(-127, min(127, __float2int_rn(r / sg))) : 0);
}

// Narrow-panel sweep (FP32 or FP64 state; also used for the FP64 truth);
// Bin == nullptr stands for B_in = 0, as in the wide sweep.
template <int P, typename T>
__global__ void __launch_bounds__(kWarps * 32) k_sweep(GraphView g, PanelParams pp, const T* Bin,
                                                       T* Bout, uint32_t* stats,
                                                       const uint32_t* done)
{
    if (*done) return;
    using Acc = T;
    const int lane = threadIdx.x & 31;
    const int col = lane % P;
    float md[1] = {0.0f}, mb[1] = {0.0f}, mr[1] = {0.0f};
    const Acc L = Acc(pp.skyL[col]);
    const float fl = kSideFloor * pp.colmax[col];
    uint32_t fb, fe;
    warp_range(g.facets, fb, fe);
    if constexpr (P <= 2) {
        using NG = NarrowGroup<P>;
        const int grp = lane / NG::kLanes, eg = (lane % NG::kLanes) / P;
        uint32_t pair, stride;
        warp_pairs(pair, stride);
        for (; 2u * pair < g.facets; pair += stride)
#pragma unroll
        for (int q = 0; q < 2 / NG::kFacets; ++q) {
            const uint32_t f = 2u * pair + uint32_t(q) + uint32_t(grp >> 1);
            const bool valid = f < g.facets;
            const uint32_t s = 2u * f + uint32_t(grp & 1);
            const size_t i = size_t(s) * P + col;
            // the side's own loads first, so that they overlap the gather
            uint32_t d = 0u, sk = 0u;
            Acc dir = 0, em = 0, rh = 0, ta = 0, o = 0;
            if (valid) {
                d = __ldcs(g.denom + s);
                sk = __ldcs(g.skyc + s);
                dir = Acc(__ldcs(pp.direct + i));
                if (eg == 0) {
                    em = Acc(__ldcs(pp.emis + i));
                    rh = Acc(__ldcs(pp.rho + i));
                    ta = Acc(__ldcs(pp.tau + i));
                    o = Bin ? Bin[i] : Acc(0);
                }
            }
            const Acc acc = Bin ? gather_group<P, T, Acc>(g, s, valid, Bin, eg, col) : Acc(0);
            const Acc h = valid ? (d == 0u ? L : (Acc(sk) * L + acc) / Acc(d)) + dir : Acc(0);
            const Acc ho = __shfl_xor_sync(0xffffffffu, h, NG::kLanes);  // the facet's other side
            if (valid && eg == 0) {
                const Acc b = em + rh * h + ta * ho;
                Bout[i] = b;
                md[0] = fmaxf(md[0], absf(b - o));
                mb[0] = fmaxf(mb[0], absf(b));
                mr[0] = fmaxf(mr[0], rel_change(float(b - o), float(b), fl));
            }
        }
        fold_narrow_stats(md, mb, mr, P);
        publish_stats<1>(md, mb, mr, lane, P, stats);
    } else {
    for (uint32_t f = fb; f < fe; ++f) {
        const uint32_t s0 = 2u * f, s1 = s0 + 1u;
        Acc h[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const uint32_t s = s0 + k;
            const Acc acc = Bin ? gather_narrow<P, T, Acc>(g, s, Bin, lane) : Acc(0);
            const uint32_t d = g.denom[s];
            const Acc dir = Acc(pp.direct[size_t(s) * P + col]);
            h[k] = (d == 0u ? L : (Acc(g.skyc[s]) * L + acc) / Acc(d)) + dir;
        }
        if (lane < P) {
            const size_t i0 = size_t(s0) * P + col, i1 = size_t(s1) * P + col;
            const Acc b0 = Acc(pp.emis[i0]) + Acc(pp.rho[i0]) * h[0] + Acc(pp.tau[i0]) * h[1];
            const Acc b1 = Acc(pp.emis[i1]) + Acc(pp.rho[i1]) * h[1] + Acc(pp.tau[i1]) * h[0];
            const Acc o0 = Bin ? Bin[i0] : Acc(0), o1 = Bin ? Bin[i1] : Acc(0);
            Bout[i0] = b0;
            Bout[i1] = b1;
            md[0] = fmaxf(md[0], fmaxf(absf(b0 - o0), absf(b1 - o1)));
            mb[0] = fmaxf(mb[0], fmaxf(absf(b0), absf(b1)));
            mr[0] = fmaxf(mr[0], fmaxf(rel_change(float(b0 - o0), float(b0), fl),
                                       rel_change(float(b1 - o1), float(b1), fl)));
        }
    }
    // lanes >= P hold zeros; column c of the stats is lane c (one column each)
    publish_stats<1>(md, mb, mr, lane, P, stats);
    }
}

template <int P>
__global__ void __launch_bounds__(kWarps * 32) k_sweep_defect(GraphView g, PanelParams pp,
                                                              const __nv_bfloat16* Din,
                                                              __nv_bfloat16* Dout, float* X,
                                                              uint32_t* stats,
                                                              const uint32_t* done)
{
    if (*done) return;
    const int lane = threadIdx.x & 31;
    const int col = lane % P;
    float md[1] = {0.0f}, mb[1] = {0.0f};
    uint32_t fb, fe;
    warp_range(g.facets, fb, fe);
    if constexpr (P <= 2) {
        using NG = NarrowGroup<P>;
        const int grp = lane / NG::kLanes, eg = (lane % NG::kLanes) / P;
        uint32_t pair, stride;
        warp_pairs(pair, stride);
        for (; 2u * pair < g.facets; pair += stride)
#pragma unroll
        for (int q = 0; q < 2 / NG::kFacets; ++q) {
            const uint32_t f = 2u * pair + uint32_t(q) + uint32_t(grp >> 1);
            const bool valid = f < g.facets;
            const uint32_t s = 2u * f + uint32_t(grp & 1);
            const size_t i = size_t(s) * P + col;
            // the side's own loads first, so that they overlap the gather
            uint32_t d = 0u;
            float rh = 0.0f, ta = 0.0f, xo = 0.0f;
            if (valid) {
                d = __ldg(g.denom + s);
                if (eg == 0) {
                    rh = pp.rho[i];
                    ta = pp.tau[i];
                    xo = X[i];
                }
            }
            const float acc = gather_group<P, __nv_bfloat16, float>(g, s, valid, Din, eg, col);
            const float h = valid && d != 0u ? acc / float(d) : 0.0f;
            const float ho = __shfl_xor_sync(0xffffffffu, h, NG::kLanes);
            if (valid && eg == 0) {
                const float dd = rh * h + ta * ho;
                Dout[i] = __float2bfloat16_rn(dd);
                const float x = xo + dd;
                X[i] = x;
                md[0] = fmaxf(md[0], fabsf(dd));
                mb[0] = fmaxf(mb[0], fabsf(x));
            }
        }
        float mr[1] = {0.0f};
        fold_narrow_stats(md, mb, mr, P);
        publish_stats<1>(md, mb, mr, lane, P, stats);
    } else {
    for (uint32_t f = fb; f < fe; ++f) {
        const uint32_t s0 = 2u * f, s1 = s0 + 1u;
        float h[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const uint32_t s = s0 + k;
            const float acc = gather_narrow<P, __nv_bfloat16, float>(g, s, Din, lane);
            const uint32_t d = g.denom[s];
            h[k] = d == 0u ? 0.0f : acc / float(d);
        }
        if (lane < P) {
            const size_t i0 = size_t(s0) * P + col, i1 = size_t(s1) * P + col;
            const float d0 = pp.rho[i0] * h[0] + pp.tau[i0] * h[1];
            const float d1 = pp.rho[i1] * h[1] + pp.tau[i1] * h[0];
            Dout[i0] = __float2bfloat16_rn(d0);
            Dout[i1] = __float2bfloat16_rn(d1);
            const float x0 = X[i0] + d0, x1 = X[i1] + d1;
            X[i0] = x0;
            X[i1] = x1;
            md[0] = fmaxf(md[0], fmaxf(fabsf(d0), fabsf(d1)));
            mb[0] = fmaxf(mb[0], fmaxf(fabsf(x0), fabsf(x1)));
        }
    }
    const float mr[1] = {0.0f};  // defect cycles stop on the absolute test
    publish_stats<1>(md, mb, mr, lane, P, stats);
    }
}

// d = Bnew - Bold (FP32) -> BF16.
__global__ void k_defect_init(const float* Bold, const float* Bnew, __nv_bfloat16* D, size_t n,
                              const uint32_t* done)
{
    if (*done) return;
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) D[i] = __float2bfloat16_rn(Bnew[i] - Bold[i]);
}

// Convergence check after sweep `it` (0-based).  Absolute test: max|dB|
// <= tol * max|B| per column; per-side test (per_side): the column's largest
// per-side relative change <= tol.  flag[0] = done (by the chosen test),
// flag[1] = sweeps run, flag[2] = worst change of the last sweep (by the
// chosen test), flag[6] = the absolute test held.  Stores max|B| per column
// in colmax (the next sweep's floor) and clears the stats.  With scale_a /
// scale_b, also stores max|dB| / 127 per column there (the int8 step
// scales).
// Plain int8 steps before c is estimated: on the config-2 forest 3, 4 and 5
// all end in 17 iterations (errors 6.4e-6, 5.2e-6, 8.3e-6 against FP64), 2
// in 18 (the estimate from the first steps is too low).
#ifndef FCU_CHEB_WARM
#define FCU_CHEB_WARM 4
#endif
constexpr float kChebWarm = float(FCU_CHEB_WARM);  // plain int8 steps before c is estimated
constexpr float kChebMax = 0.7f;   // largest c for which the weights are used

// Chebyshev state per column (cheb[0..4 kMaxP)): previous max|R|, c (-1 =
// off), the weight of the step being formed, steps done.  mode 1: reset
// after an FP32 sweep (max|R_0| = md); mode 2: after an int8 step, advance
// the schedule and size the next scale for omega R + (omega - 1) delta.
__device__ __forceinline__ float cheb_advance(float* cheb, int c, int mode, float md)
{
    float* prev = cheb;
    float* cc = cheb + kMaxP;
    float* om = cheb + 2 * kMaxP;
    float* nn = cheb + 3 * kMaxP;
    if (mode == 1) {
        prev[c] = md;
        cc[c] = 0.0f;
        om[c] = 1.0f;
        nn[c] = 0.0f;
        return 1.0f;
    }
    const float n = nn[c] + 1.0f;
    nn[c] = n;
    float w = 1.0f;
    if (n < kChebWarm) {
        prev[c] = md;
    } else if (n == kChebWarm) {
        const float est = prev[c] > 0.0f ? md / prev[c] : 0.0f;
        cc[c] = est > 0.0f && est <= kChebMax ? est : -1.0f;
    } else if (cc[c] > 0.0f) {
        const float c2 = cc[c] * cc[c];
        w = n == kChebWarm + 1.0f ? 1.0f / (1.0f - 0.5f * c2) : 1.0f / (1.0f - 0.25f * c2 * om[c]);
    }
    om[c] = w;
    return w;
}

__global__ void k_check(uint32_t* stats, uint32_t* flag, int P, float tol, uint32_t it,
                        uint32_t* counter, float* scale_a, float* scale_b, uint32_t* it_dev,
                        bool per_side, float* colmax, float* cheb = nullptr, int cheb_mode = 0,
                        const float* scale_prev = nullptr)
{
    __shared__ int all_ok, abs_ok;
    __shared__ float worst;
    if (it_dev) it = *it_dev;  // the sweep index kept on the device (graph replays)
    if (threadIdx.x == 0) {
        all_ok = 1;
        abs_ok = 1;
        worst = 0.0f;
    }
    __syncthreads();
    const bool already = flag[0] != 0u;
    if (threadIdx.x < uint32_t(P)) {
        const float md = __uint_as_float(stats[threadIdx.x]);
        const float mb = __uint_as_float(stats[kMaxP + threadIdx.x]);
        const float mr = __uint_as_float(stats[2 * kMaxP + threadIdx.x]);
        const float rel = mb > 0.0f ? md / mb : (md > 0.0f ? INFINITY : 0.0f);
        const bool a_ok = (md <= tol * mb) || md == 0.0f;
        const bool s_ok = (mr <= tol) || md == 0.0f;
        if (!a_ok) atomicExch(&abs_ok, 0);
        if (!(per_side ? s_ok : a_ok)) atomicExch(&all_ok, 0);
        atomicMax(reinterpret_cast<int*>(&worst), __float_as_int(per_side ? mr : rel));
        // int8 step scales: sigma = max|R| / 127 for the column, or with
        // Chebyshev weights a bound on omega R + (omega - 1) delta
        float w = 1.0f;
        if (cheb && !already) w = cheb_advance(cheb, int(threadIdx.x), cheb_mode, md);
        float sigma = md / 127.0f;
        if (w != 1.0f && scale_prev) sigma = (w * md + (w - 1.0f) * 127.0f * scale_prev[threadIdx.x]) / 127.0f;
        if (scale_a && !already) scale_a[threadIdx.x] = sigma;
        if (scale_b && !already) scale_b[threadIdx.x] = md / 127.0f;
        if (colmax && !already) colmax[threadIdx.x] = mb;
    }
    __syncthreads();
    if (threadIdx.x == 0 && !already) {
        flag[1] = it + 1;
        flag[2] = __float_as_uint(worst);
        flag[6] = abs_ok ? 1u : 0u;
        if (all_ok) flag[0] = 1;
    }
    for (int i = threadIdx.x; i < 3 * kMaxP; i += blockDim.x) stats[i] = 0;
    if (threadIdx.x == 0) {
        *counter = 0u;
        if (it_dev) *it_dev = it + 1;
    }
}

__device__ __forceinline__ uint32_t new_side(const uint32_t* rank, uint32_t so)
{
    return rank ? 2u * rank[so >> 1] + (so & 1u) : so;
}

// The panel kernels move [R][S] arrays (caller side order, band-major) to
// [S][P] panels (solver order) and back.  A block takes 32 consecutive
// caller sides and 32 columns at a time: the band-major side reads and
// writes are 128-byte rows, the panel side is one 128-byte row segment per
// side (rank maps caller facet -> solver facet), transposed through a
// shared tile.  Reading in solver order instead (one 4-byte element of a
// different band row per thread) moved 8x the bytes once the inputs
// outgrew L2.
constexpr int kPanelTile = 32;

// Panel parameters for columns [c0, c0 + P) (column c = sun * bands + band).
__global__ void __launch_bounds__(256) k_prepare_panel(
    uint32_t S, uint32_t bands, uint32_t R, uint32_t c0, int P, const uint32_t* rank,
    const float* __restrict__ rho, const float* __restrict__ tau, const float* __restrict__ emis,
    const float* __restrict__ beam, const float* __restrict__ dgeo, float* __restrict__ prho,
    float* __restrict__ ptau, float* __restrict__ pemis, float* __restrict__ pdir)
{
    __shared__ float tile[4][kPanelTile][kPanelTile + 1];
    __shared__ uint32_t dest[kPanelTile];
    const uint32_t so0 = blockIdx.x * kPanelTile;
    if (threadIdx.x < kPanelTile) {
        const uint32_t so = so0 + threadIdx.x;
        dest[threadIdx.x] = so < S ? new_side(rank, so) : 0u;
    }
    for (int j0 = 0; j0 < P; j0 += kPanelTile) {
        const int w = min(P - j0, kPanelTile);
        __syncthreads();
        for (int k = threadIdx.x; k < kPanelTile * w; k += blockDim.x) {
            const int j = k / kPanelTile, ls = k % kPanelTile;
            const uint32_t so = so0 + ls, c = c0 + j0 + j;
            float r = 0.0f, t = 0.0f, e = 0.0f, d = 0.0f;
            if (so < S && c < R) {
                const uint32_t b = c % bands, kk = c / bands;
                const size_t bi = size_t(b) * S + so;
                r = rho[bi];
                t = tau[bi];
                e = emis ? emis[bi] : 0.0f;
                d = dgeo ? beam[b] * dgeo[size_t(kk) * S + so] : 0.0f;
            }
            tile[0][ls][j] = r;
            tile[1][ls][j] = t;
            tile[2][ls][j] = e;
            tile[3][ls][j] = d;
        }
        __syncthreads();
        for (int k = threadIdx.x; k < kPanelTile * w; k += blockDim.x) {
            const int ls = k / w, j = k % w;
            if (so0 + ls >= S) continue;
            const size_t o = size_t(dest[ls]) * P + j0 + j;
            prho[o] = tile[0][ls][j];
            ptau[o] = tile[1][ls][j];
            pemis[o] = tile[2][ls][j];
            pdir[o] = tile[3][ls][j];
        }
    }
}

__global__ void k_panel_sky(uint32_t bands, uint32_t R, uint32_t c0, int P, const float* sky,
                            float* psky)
{
    for (int j = threadIdx.x; j < P; j += blockDim.x) {
        const uint32_t c = c0 + j;
        psky[j] = c < R ? sky[c % bands] : 0.0f;
    }
}

// [R][S] (caller order) -> [S][P] (solver order); src null: zeros
template <typename T>
__global__ void __launch_bounds__(256) k_panel_in(const float* __restrict__ src, uint32_t S,
                                                  uint32_t R, uint32_t c0, int P,
                                                  const uint32_t* rank, T* __restrict__ dst)
{
    __shared__ float tile[kPanelTile][kPanelTile + 1];
    __shared__ uint32_t dest[kPanelTile];
    const uint32_t so0 = blockIdx.x * kPanelTile;
    if (threadIdx.x < kPanelTile) {
        const uint32_t so = so0 + threadIdx.x;
        dest[threadIdx.x] = so < S ? new_side(rank, so) : 0u;
    }
    for (int j0 = 0; j0 < P; j0 += kPanelTile) {
        const int w = min(P - j0, kPanelTile);
        __syncthreads();
        for (int k = threadIdx.x; k < kPanelTile * w; k += blockDim.x) {
            const int j = k / kPanelTile, ls = k % kPanelTile;
            const uint32_t so = so0 + ls, c = c0 + j0 + j;
            tile[ls][j] = (src && so < S && c < R) ? src[size_t(c) * S + so] : 0.0f;
        }
        __syncthreads();
        for (int k = threadIdx.x; k < kPanelTile * w; k += blockDim.x) {
            const int ls = k / w, j = k % w;
            if (so0 + ls < S) dst[size_t(dest[ls]) * P + j0 + j] = T(tile[ls][j]);
        }
    }
}

// [S][P] (solver order) -> [R][S] (caller order)
template <typename T>
__global__ void __launch_bounds__(256) k_panel_out(const T* __restrict__ src, uint32_t S,
                                                   uint32_t R, uint32_t c0, int P,
                                                   const uint32_t* rank, float* __restrict__ dst)
{
    __shared__ float tile[kPanelTile][kPanelTile + 1];
    __shared__ uint32_t from[kPanelTile];
    const uint32_t so0 = blockIdx.x * kPanelTile;
    if (threadIdx.x < kPanelTile) {
        const uint32_t so = so0 + threadIdx.x;
        from[threadIdx.x] = so < S ? new_side(rank, so) : 0u;
    }
    for (int j0 = 0; j0 < P; j0 += kPanelTile) {
        const int w = min(P - j0, kPanelTile);
        __syncthreads();
        for (int k = threadIdx.x; k < kPanelTile * w; k += blockDim.x) {
            const int ls = k / w, j = k % w;
            tile[ls][j] = so0 + ls < S ? float(src[size_t(from[ls]) * P + j0 + j]) : 0.0f;
        }
        __syncthreads();
        for (int k = threadIdx.x; k < kPanelTile * w; k += blockDim.x) {
            const int j = k / kPanelTile, ls = k % kPanelTile;
            const uint32_t so = so0 + ls, c = c0 + j0 + j;
            if (so < S && c < R) dst[size_t(c) * S + so] = tile[ls][j];
        }
    }
}

// ---- Morton renumbering of the graph -----------------------------------------
__global__ void k_rank(const uint32_t* order, uint32_t facets, uint32_t* rank)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < facets) rank[order[i]] = i;
}

// The solver's copy of the graph splits every edge whose count is above 255
// into edges of at most 255 to the same neighbour (255, 255, ..., the rest),
// adjacent in the row: the int8 step's dp4a then takes every count as one
// byte.  Its integer sums are the same; the FP32 and FP64 sweeps add the
// pieces one by one.  (The forests hold about one such edge in 10^6.)
__device__ __forceinline__ uint32_t count_pieces(uint32_t c) { return c > 255u ? (c + 254u) / 255u : 1u; }

// One warp per renumbered side: its row length in pieces, denominator and
// sky count.
__global__ void k_perm_lengths(const uint32_t* order, uint32_t S, const uint32_t* rows,
                               const uint32_t* packed, uint32_t nb_bits, const uint32_t* denom,
                               const uint32_t* sky, uint32_t* len, uint32_t* pden, uint32_t* psky)
{
    const uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= S) return;
    const uint32_t so = 2u * order[s >> 1] + (s & 1u);
    const uint32_t b = rows[so], n = rows[so + 1] - b;
    uint32_t k = 0;
    for (uint32_t i = lane; i < n; i += 32) k += count_pieces(packed[b + i] >> nb_bits);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
    if (lane == 0) {
        len[s] = k;
        pden[s] = denom[so];
        psky[s] = sky[so];
    }
}

// The scene of each renumbered facet.
__global__ void k_perm_scene(const uint32_t* __restrict__ order, const uint16_t* __restrict__ scene,
                             uint32_t F, uint16_t* __restrict__ out)
{
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < F) out[f] = scene[order[f]];
}

// One warp per renumbered side: its edges with neighbours renumbered and
// counts above 255 split (the pieces' places from a scan over the lanes).
__global__ void k_perm_copy(const uint32_t* order, const uint32_t* rank, uint32_t S,
                            const uint32_t* rows, const uint32_t* packed, const uint32_t* prows,
                            uint32_t* ppacked, uint32_t nb_bits)
{
    const uint32_t mask = (1u << nb_bits) - 1u;
    const uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= S) return;
    const uint32_t so = 2u * order[s >> 1] + (s & 1u);
    const uint32_t b = rows[so], n = rows[so + 1] - b;
    uint32_t out = prows[s];
    for (uint32_t i0 = 0; i0 < n; i0 += 32) {
        const uint32_t i = i0 + uint32_t(lane);
        uint32_t nn = 0u, c = 0u, k = 0u;
        if (i < n) {
            const uint32_t p = packed[b + i];
            const uint32_t nb = p & mask;
            nn = 2u * rank[nb >> 1] + (nb & 1u);
            c = p >> nb_bits;
            k = count_pieces(c);
        }
        uint32_t incl = k;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const uint32_t first = out + incl - k;
        for (uint32_t j = 0; j < k; ++j) {
            const uint32_t cj = j + 1u < k ? 255u : c - 255u * (k - 1u);
            ppacked[first + j] = nn | (cj << nb_bits);
        }
        out += __shfl_sync(0xffffffffu, incl, 31);
    }
}

__global__ void k_set_last(uint32_t* rows, uint32_t n, const unsigned long long* total)
{
    rows[n] = uint32_t(*total);
}

inline unsigned blocks_for(size_t n, unsigned b) { return unsigned((n + b - 1) / b); }

template <typename K>
int grid_for(K kernel)
{
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kWarps * 32, 0);
    return std::max(1, sms) * std::max(1, per_sm);
}

template <typename T>
void launch_sweep(int P, const GraphView& g, const PanelParams& pp, const T* in, T* out,
                  uint32_t* stats, uint32_t* counter, const uint32_t* done, cudaStream_t s)
{
    if constexpr (sizeof(T) == 4) {
        if (in == nullptr && P >= 8) {
            // a solve from zero: its first sweep has nothing to gather
            static const int grid = [] {
                int dev = 0, sms = 0;
                cudaGetDevice(&dev);
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
                return std::max(1, sms) * 8;
            }();
            switch (P) {
            case 8: k_sweep_zero<8><<<grid, 256, 0, s>>>(g, pp, out, stats, done); break;
            case 16: k_sweep_zero<16><<<grid, 256, 0, s>>>(g, pp, out, stats, done); break;
            case 32: k_sweep_zero<32><<<grid, 256, 0, s>>>(g, pp, out, stats, done); break;
            case 64: k_sweep_zero<64><<<grid, 256, 0, s>>>(g, pp, out, stats, done); break;
            default: k_sweep_zero<128><<<grid, 256, 0, s>>>(g, pp, out, stats, done); break;
            }
            FCU_LAUNCH("k_sweep_zero");
            return;
        }
        if (P == 8 || P == 16) {
            // 16-byte row vectors in rounds of 8 loads per lane
            if (P == 8) {
                static const int grid = grid_for(k_sweep_wide<8>);
                k_sweep_wide<8><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, stats, counter, done);
            } else {
                static const int grid = grid_for(k_sweep_wide<16>);
                k_sweep_wide<16><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, stats, counter, done);
            }
            FCU_LAUNCH("k_sweep_wide");
            return;
        }
        if (P >= 32) {
            switch (P) {
            case 32: {
                static const int grid = grid_for(k_sweep_wide<32>);
                k_sweep_wide<32><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, stats, counter, done);
                break;
            }
            case 64: {
                static const int grid = grid_for(k_sweep_wide<64>);
                k_sweep_wide<64><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, stats, counter, done);
                break;
            }
            default: {
                static const int grid = grid_for(k_sweep_wide<128>);
                k_sweep_wide<128><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, stats, counter, done);
                break;
            }
            }
            FCU_LAUNCH("k_sweep_wide");
            return;
        }
    }
    static const int grid = grid_for(k_sweep<32, T>);
    switch (P) {
    case 1: k_sweep<1, T><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, stats, done); break;
    case 2: k_sweep<2, T><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, stats, done); break;
    case 4: k_sweep<4, T><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, stats, done); break;
    case 8: k_sweep<8, T><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, stats, done); break;
    case 16: k_sweep<16, T><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, stats, done); break;
    default: k_sweep<32, T><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, stats, done); break;
    }
    FCU_LAUNCH("k_sweep");
}

// BF16 defect sweep; only panels narrower than 32 columns take this path
// (wider MIXED panels run k_step_i8).
void launch_defect(int P, const GraphView& g, const PanelParams& pp, const __nv_bfloat16* in,
                   __nv_bfloat16* out, float* X, uint32_t* stats, uint32_t* counter,
                   const uint32_t* done, cudaStream_t s)
{
    (void)counter;
    static const int grid = grid_for(k_sweep_defect<32>);
    switch (P) {
    case 1: k_sweep_defect<1><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, X, stats, done); break;
    case 2: k_sweep_defect<2><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, X, stats, done); break;
    case 4: k_sweep_defect<4><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, X, stats, done); break;
    case 8: k_sweep_defect<8><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, X, stats, done); break;
    case 16: k_sweep_defect<16><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, X, stats, done); break;
    default: k_sweep_defect<32><<<grid, kWarps * 32, 0, s>>>(g, pp, in, out, X, stats, done); break;
    }
    FCU_LAUNCH("k_sweep_defect");
}

template <int P, bool Scenes>
int step_grid()
{
    static const int grid = grid_for(k_step_i8<P, Scenes>);
    return grid;
}

// The pipelined step: its dynamic shared memory is opted in once (before
// any graph capture); the grid is the SM count times the CTAs per SM that
// fit, or fewer when the autotuner asks for fewer (`ctas`).
template <int P, bool Scenes>
int async_step_grid(uint32_t ctas = 0)
{
    struct Fit {
        int sms, per_sm;
    };
    static const Fit fit = [] {
        constexpr int bytes = AsyncLayout<P>::kBlockBytes;
        FCU_CHECK(cudaFuncSetAttribute(k_step_i8_async<P, Scenes>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        FCU_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, k_step_i8_async<P, Scenes>, AsyncWarps<P>::value * 32, bytes));
        return Fit{std::max(1, sms), std::max(1, per_sm)};
    }();
    const int per_sm = ctas ? std::min(fit.per_sm, int(ctas)) : fit.per_sm;
    return fit.sms * per_sm;
}

template <int P, bool Scenes>
void launch_async_step(const GraphView& g, const PanelParams& pp, const int8_t* qin, int8_t* qout,
                       float* X, float* R, const float* sin, const float* sout, uint32_t* stats,
                       uint32_t* counter, const uint32_t* done, const float* ssin,
                       const float* ssout, cudaStream_t s)
{
    k_step_i8_async<P, Scenes><<<async_step_grid<P, Scenes>(g.step_ctas),
                                 AsyncWarps<P>::value * 32, AsyncLayout<P>::kBlockBytes, s>>>(
        g, pp, qin, qout, X, R, sin, sout, stats, counter, done, ssin, ssout);
}

#ifndef FCU_STEP_ASYNC_128
#define FCU_STEP_ASYNC_128 1
#endif
bool use_async_step(int P, const GraphView& g)
{
    return FCU_STEP_ASYNC && (P == 64 || (P == 128 && FCU_STEP_ASYNC_128)) &&
           g.packed != nullptr && g.counts8 != 0u && g.legacy_step == 0u;
}

// parity: the step's index modulo 2 (its input scales are slot `parity`,
// its output scales slot `parity ^ 1`)
void launch_step_i8(int P, const GraphView& g, const PanelParams& pp, const int8_t* qin,
                    int8_t* qout, float* X, float* R, const float* sin, const float* sout,
                    uint32_t* stats, uint32_t* counter, const uint32_t* done, uint32_t parity,
                    cudaStream_t s)
{
    const bool sc = g.scene != nullptr;
    const size_t slot = size_t(g.scenes) * kMaxP;
    const float* ssin = sc ? g.scene_sig + (parity & 1u) * slot : nullptr;
    const float* ssout = sc ? g.scene_sig + ((parity + 1u) & 1u) * slot : nullptr;
    switch (P) {
    case 32:
        if (sc)
            k_step_i8<32, true><<<step_grid<32, true>(), kWarps * 32, 0, s>>>(
                g, pp, qin, qout, X, R, sin, sout, stats, counter, done, ssin, ssout);
        else
            k_step_i8<32, false><<<step_grid<32, false>(), kWarps * 32, 0, s>>>(
                g, pp, qin, qout, X, R, sin, sout, stats, counter, done, ssin, ssout);
        break;
    case 64:
        if (use_async_step(P, g) && sc)
            launch_async_step<64, true>(g, pp, qin, qout, X, R, sin, sout, stats, counter, done,
                                        ssin, ssout, s);
        else if (use_async_step(P, g))
            launch_async_step<64, false>(g, pp, qin, qout, X, R, sin, sout, stats, counter, done,
                                         ssin, ssout, s);
        else if (sc)
            k_step_i8<64, true><<<step_grid<64, true>(), kWarps * 32, 0, s>>>(
                g, pp, qin, qout, X, R, sin, sout, stats, counter, done, ssin, ssout);
        else
            k_step_i8<64, false><<<step_grid<64, false>(), kWarps * 32, 0, s>>>(
                g, pp, qin, qout, X, R, sin, sout, stats, counter, done, ssin, ssout);
        break;
    default:
        if (use_async_step(128, g) && sc)
            launch_async_step<128, true>(g, pp, qin, qout, X, R, sin, sout, stats, counter, done,
                                         ssin, ssout, s);
        else if (use_async_step(128, g))
            launch_async_step<128, false>(g, pp, qin, qout, X, R, sin, sout, stats, counter,
                                          done, ssin, ssout, s);
        else if (sc)
            k_step_i8<128, true><<<step_grid<128, true>(), kWarps * 32, 0, s>>>(
                g, pp, qin, qout, X, R, sin, sout, stats, counter, done, ssin, ssout);
        else
            k_step_i8<128, false><<<step_grid<128, false>(), kWarps * 32, 0, s>>>(
                g, pp, qin, qout, X, R, sin, sout, stats, counter, done, ssin, ssout);
        break;
    }
    FCU_LAUNCH("k_step_i8");
}

// The scene check after step `parity` (after the column check): writes the
// scales of slot `parity`, reading slot `parity ^ 1`.
void launch_scene_check(const GraphView& g, int P, uint32_t parity, float tol, cudaStream_t s)
{
    if (!g.scene) return;
    const size_t slot = size_t(g.scenes) * kMaxP;
    k_scene_check<<<g.scenes, kMaxP, 0, s>>>(g.scene_stats, g.scene_md,
                                              g.scene_sig + (parity & 1u) * slot,
                                              g.scene_sig + ((parity + 1u) & 1u) * slot,
                                              g.scene_done, g.scene_cheb, P, tol);
    FCU_LAUNCH("k_scene_check");
}

// The int8 phase of a solve as one CUDA graph launch: a conditional WHILE
// node whose body is two steps (the q panels and scales alternate with the
// step's parity), each followed by its check (the sweep index comes from the
// device counter k_init_i8 seeds), and k_steps_continue, which keeps the loop
// going while the phase's done flag is clear and two more steps fit under
// the iteration limit.  The device decides when the phase ends; the host
// reads the flags once, after the launch.  The graph is captured once per
// panel configuration and replayed.
constexpr uint32_t kStepBatch = 2;  // steps per loop body

__global__ void k_steps_continue(cudaGraphConditionalHandle loop, const uint32_t* done,
                                 const uint32_t* it_dev, uint32_t limit)
{
    cudaGraphSetConditional(loop, (*done == 0u && *it_dev + kStepBatch <= limit) ? 1u : 0u);
}

struct StepGraphKey {
    int P;
    GraphView g;
    PanelParams pp;
    const int8_t* q0;
    const int8_t* q1;
    float* X;
    float* R;
    float* slot0;
    float* slot1;
    uint32_t* stats;
    uint32_t* flag;
    float tol;
    uint32_t limit;  // iteration limit of the solve
    cudaStream_t stream;
};

void record_steps(const StepGraphKey& k, cudaStream_t s)
{
    int8_t* qb[2] = {const_cast<int8_t*>(k.q0), const_cast<int8_t*>(k.q1)};
    float* slot[2] = {k.slot0, k.slot1};
    uint32_t* counter = k.flag + 8;
    for (uint32_t j = 0; j < kStepBatch; ++j) {  // kStepBatch is even: the parity repeats
        launch_step_i8(k.P, k.g, k.pp, qb[j & 1u], qb[(j + 1) & 1u], k.X, k.R, slot[j & 1u],
                       slot[(j + 1) & 1u], k.stats, counter, k.flag + 3, j & 1u, s);
        float* colmax = reinterpret_cast<float*>(k.flag + 16);
        k_check<<<1, kMaxP, 0, s>>>(k.stats, k.flag + 3, k.P, k.tol, 0u, counter, slot[j & 1u],
                                    nullptr, k.flag + 12, true, colmax, colmax + 3 * kMaxP, 2,
                                    slot[(j + 1) & 1u]);
        FCU_LAUNCH("k_check");
        launch_scene_check(k.g, k.P, j & 1u, k.tol, s);
    }
}

cudaGraphExec_t step_graph(BatchState& st, const StepGraphKey& key)
{
    if (st.step_graph && std::memcmp(st.step_graph_key, &key, sizeof(key)) == 0)
        return st.step_graph;
    // FACETCU_TEST_NO_LOOP_GRAPH=1 (read when a context first needs the
    // graph): take the path of drivers without conditional nodes, for tests
    const char* no_loop = std::getenv("FACETCU_TEST_NO_LOOP_GRAPH");
    if (no_loop && no_loop[0] == '1') {
        st.no_loop_graph = true;
        return nullptr;
    }
    release_graphs(st);
    switch (key.P) {  // size the grids before capture starts
    case 32: step_grid<32, false>(); step_grid<32, true>(); break;
    case 64:
        step_grid<64, false>();
        step_grid<64, true>();
        async_step_grid<64, false>();
        async_step_grid<64, true>();
        break;
    default:
        step_grid<128, false>();
        step_grid<128, true>();
        async_step_grid<128, false>();
        async_step_grid<128, true>();
        break;
    }
    cudaGraph_t graph = nullptr;
    FCU_CHECK(cudaGraphCreate(&graph, 0));
    cudaGraphExec_t exec = nullptr;
    try {
        cudaGraphConditionalHandle loop;
        cudaGraphNodeParams cp = {};
        cudaGraphNode_t node = nullptr;
        cudaError_t e = cudaGraphConditionalHandleCreate(&loop, graph, 1u, cudaGraphCondAssignDefault);
        if (e == cudaSuccess) {
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = loop;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp);
        }
        if (e == cudaErrorNotSupported || e == cudaErrorInvalidValue) {
            // no conditional nodes with this driver: the caller launches
            // the steps one by one (the same bits)
            cudaGetLastError();
            cudaGraphDestroy(graph);
            st.no_loop_graph = true;
            return nullptr;
        }
        FCU_CHECK(e);
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        FCU_CHECK(cudaStreamBeginCaptureToGraph(key.stream, body, nullptr, nullptr, 0,
                                                cudaStreamCaptureModeThreadLocal));
        try {
            record_steps(key, key.stream);
            k_steps_continue<<<1, 1, 0, key.stream>>>(loop, key.flag + 3, key.flag + 12,
                                                      key.limit);
            FCU_LAUNCH("k_steps_continue");
        } catch (...) {
            cudaGraph_t dummy = nullptr;
            cudaStreamEndCapture(key.stream, &dummy);
            throw;
        }
        cudaGraph_t captured = nullptr;
        FCU_CHECK(cudaStreamEndCapture(key.stream, &captured));
        FCU_CHECK(cudaGraphInstantiate(&exec, graph, 0));
    } catch (...) {
        cudaGraphDestroy(graph);
        throw;
    }
    cudaGraphDestroy(graph);
    st.step_graph = exec;
    static_assert(sizeof(StepGraphKey) <= sizeof(st.step_graph_key), "graph key size");
    std::memcpy(st.step_graph_key, &key, sizeof(key));
    return exec;
}

// Panel widths: the widest power of two not above the remaining columns
// (and `cap`: 128 for FP32/MIXED, 32 for FP64, or the caller's request), so
// 65 columns run as 64 + 1 rather than one half-empty 128-wide panel; a
// remainder below 32 columns is covered by one narrow panel.
int panel_width(uint32_t remaining, uint32_t requested, uint32_t cap)
{
    const uint32_t p = requested ? std::min(requested, cap) : cap;
    uint32_t w = 1;
    while (w * 2 <= p && w * 2 <= remaining) w <<= 1;
    if (w < 32) {
        w = 1;
        while (w < p && w < remaining) w <<= 1;
    }
    return int(std::min(w, cap));
}

// Build (once per graph) the Morton-renumbered copy used by the solver.
void ensure_permuted(DeviceGraph& gr, const BatchProblem& p, Workspace& ws, cudaStream_t s)
{
    if (gr.perm_valid || !gr.packed_valid || !p.vertices) return;
    const uint32_t S = gr.surfaces, F = S / 2u;
    uint32_t* order = static_cast<uint32_t*>(gr.order.reserve(size_t(F) * 4 + 4));
    uint32_t* rank = static_cast<uint32_t*>(gr.rank.reserve(size_t(F) * 4 + 4));
    morton_order(p.vertices, F, p.lo, p.hi, order, ws, s);
    k_rank<<<blocks_for(F, 256), 256, 0, s>>>(order, F, rank);
    FCU_LAUNCH("k_rank");
    uint32_t* prows = static_cast<uint32_t*>(gr.p_rows.reserve((size_t(S) + 1) * 4));
    uint32_t* pden = static_cast<uint32_t*>(gr.p_denom.reserve(size_t(S) * 4));
    uint32_t* psky = static_cast<uint32_t*>(gr.p_sky.reserve(size_t(S) * 4));
    k_perm_lengths<<<blocks_for(size_t(S) * 32, 256), 256, 0, s>>>(
        order, S, gr.row_offsets.as<uint32_t>(), gr.packed.as<uint32_t>(), gr.nb_bits,
        gr.denominators.as<uint32_t>(), gr.sky.as<uint32_t>(), prows, pden, psky);
    FCU_LAUNCH("k_perm_lengths");
    unsigned long long* total = static_cast<unsigned long long*>(ws.e.reserve(64));
    exclusive_scan_u32(prows, prows, S, total, ws, s);
    k_set_last<<<1, 1, 0, s>>>(prows, S, total);
    FCU_LAUNCH("k_set_last");
    unsigned long long split_nnz = 0;
    FCU_CHECK(cudaMemcpyAsync(&split_nnz, total, 8, cudaMemcpyDeviceToHost, s));
    FCU_CHECK(cudaStreamSynchronize(s));
    if (split_nnz > 0xffffffffull)
        throw Error(FACETCU_OVERFLOW_ERROR, "the solver's graph copy exceeds 2^32 edges");
    gr.p_nnz = size_t(split_nnz);
    uint32_t* ppk = static_cast<uint32_t*>(gr.p_packed.reserve(gr.p_nnz * 4 + 4));
    k_perm_copy<<<blocks_for(size_t(S) * 32, 256), 256, 0, s>>>(
        order, rank, S, gr.row_offsets.as<uint32_t>(), gr.packed.as<uint32_t>(), prows, ppk,
        gr.nb_bits);
    FCU_LAUNCH("k_perm_copy");
    const size_t scenes = gr.scene_facets.size() >= 3 ? gr.scene_facets.size() - 1 : 0;
    if (scenes >= 2 && scenes <= 65535 && gr.scene_facets.back() == F) {
        std::vector<uint16_t> h(F);
        for (size_t k = 0; k < scenes; ++k)
            for (uint32_t f = gr.scene_facets[k]; f < gr.scene_facets[k + 1]; ++f) h[f] = uint16_t(k);
        uint16_t* d_orig = static_cast<uint16_t*>(ws.e.reserve(size_t(F) * 2 + 64));
        uint16_t* d_perm = static_cast<uint16_t*>(gr.p_scene.reserve(size_t(F) * 2 + 64));
        FCU_CHECK(cudaMemcpyAsync(d_orig, h.data(), size_t(F) * 2, cudaMemcpyHostToDevice, s));
        k_perm_scene<<<blocks_for(F, 256), 256, 0, s>>>(order, d_orig, F, d_perm);
        FCU_LAUNCH("k_perm_scene");
    } else {
        gr.p_scene.release();
    }
    FCU_CHECK(cudaStreamSynchronize(s));
    gr.perm_valid = true;
}

}  // namespace

// Host driver.  Returns FACETCU_OK or FACETCU_NOT_CONVERGED.
namespace {
// Input checks of the batched solve on the device (the host loop over
// bands x sides would cost more than the solve): bit 1 = an optical value
// that is not finite, negative, or with reflectance + transmittance > 1;
// bit 2 = a sky value not finite or negative; bit 4 = the same for beam.
__global__ void k_validate_inputs(const float* __restrict__ rho, const float* __restrict__ tau,
                                  const float* __restrict__ emis, size_t n,
                                  const float* __restrict__ sky, const float* __restrict__ beam,
                                  uint32_t bands, uint32_t* flags)
{
    uint32_t f = 0;
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    const size_t first = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    for (size_t i = first; i < n; i += stride) {
        const float r = rho[i], t = tau[i], e = emis ? emis[i] : 0.0f;
        if (!isfinite(r) || !isfinite(t) || !isfinite(e) || r < 0.0f || t < 0.0f || e < 0.0f ||
            r + t > 1.0001f)
            f |= 1u;
    }
    if (first < bands) {
        const float k = sky[first], b = beam[first];
        if (!isfinite(k) || k < 0.0f) f |= 2u;
        if (!isfinite(b) || b < 0.0f) f |= 4u;
    }
    f = __reduce_or_sync(0xffffffffu, f);
    if ((threadIdx.x & 31) == 0 && f) atomicOr(flags, f);
}
}  // namespace

uint32_t validate_inputs(const float* rho, const float* tau, const float* emis, size_t n,
                         const float* sky, const float* beam, uint32_t bands, DeviceBuffer& scratch,
                         cudaStream_t s)
{
    uint32_t* d = static_cast<uint32_t*>(scratch.reserve(64));
    FCU_CHECK(cudaMemsetAsync(d, 0, 4, s));
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t need = std::max<size_t>((n + 255) / 256, (bands + 255) / 256);
    const unsigned grid = unsigned(std::max<size_t>(1, std::min<size_t>(need, size_t(sms) * 8)));
    k_validate_inputs<<<grid, 256, 0, s>>>(rho, tau, emis, n, sky, beam, bands, d);
    FCU_LAUNCH("k_validate_inputs");
    uint32_t h = 0;
    FCU_CHECK(cudaMemcpyAsync(&h, d, 4, cudaMemcpyDeviceToHost, s));
    FCU_CHECK(cudaStreamSynchronize(s));
    return h;
}

void release_graphs(BatchState& st)
{
    if (st.step_graph) cudaGraphExecDestroy(st.step_graph);
    st.step_graph = nullptr;
    std::memset(st.step_graph_key, 0, sizeof(st.step_graph_key));
}

int batched_solve(const DeviceGraph& gr_in, const BatchProblem& p, const facetcu_batch_config& cfg,
                  const float* d_initial, float* d_out, BatchState& st, Workspace& ws,
                  cudaStream_t s, facetcu_batch_result* result)
{
    DeviceGraph& gr = const_cast<DeviceGraph&>(gr_in);
    const uint32_t S = p.S, R = p.bands * p.suns;
    const bool fp64 = cfg.precision == FACETCU_PRECISION_FP64;
    const bool mixed = cfg.precision == FACETCU_PRECISION_MIXED;
    const size_t elem = fp64 ? 8 : 4;
    ensure_permuted(gr, p, ws, s);
    const bool perm = gr.perm_valid;
    // caller facet -> solver facet, for the panel transposes
    const uint32_t* rank = perm ? gr.rank.as<uint32_t>() : nullptr;
    GraphView g;
    g.rows = perm ? gr.p_rows.as<uint32_t>() : gr.row_offsets.as<uint32_t>();
    g.packed = perm ? gr.p_packed.as<uint32_t>()
                    : (gr.packed_valid ? gr.packed.as<uint32_t>() : nullptr);
    g.edges = gr.edges.as<facetcu_csr_edge>();
    g.denom = perm ? gr.p_denom.as<uint32_t>() : gr.denominators.as<uint32_t>();
    g.skyc = perm ? gr.p_sky.as<uint32_t>() : gr.sky.as<uint32_t>();
    g.facets = S / 2u;
    g.nb_bits = gr.nb_bits;
    g.scene = nullptr;
    g.scenes = 0;
    g.scene_stats = nullptr;
    g.scene_md = nullptr;
    g.scene_sig = nullptr;
    g.scene_cheb = nullptr;
    g.scene_done = nullptr;
    g.legacy_step = (cfg.flags & FACETCU_BATCH_LEGACY_STEP) != 0u ? 1u : 0u;
    g.counts8 = perm ? 1u : 0u;
    g.step_ctas = p.step_ctas_per_sm;
    if (FCU_SCENE_SKIP && perm && mixed && gr.p_scene.ptr && gr.p_scene.bytes >= size_t(S / 2u) * 2 &&
        gr.scene_facets.size() >= 3) {
        // scene batch: converged scenes leave the int8 steps
        g.scene = gr.p_scene.as<uint16_t>();
        g.scenes = uint32_t(gr.scene_facets.size() - 1);
        // [scenes][kMaxP] ratio, [scenes][kMaxP] max|R|, 2 x [scenes][kMaxP]
        // scales, [scenes][4 kMaxP] Chebyshev state, [scenes] done
        g.scene_stats = static_cast<uint32_t*>(
            st.scene_state.reserve(size_t(g.scenes) * (8 * kMaxP + 1) * 4));
        g.scene_md = g.scene_stats + size_t(g.scenes) * kMaxP;
        g.scene_sig = reinterpret_cast<float*>(g.scene_md + size_t(g.scenes) * kMaxP);
        g.scene_cheb = g.scene_sig + size_t(g.scenes) * 2 * kMaxP;
        g.scene_done = g.scene_stats + size_t(g.scenes) * 8 * kMaxP;
    }
    const uint32_t cap = fp64 ? 32u : uint32_t(kMaxP);
    const int Pmax = panel_width(R, cfg.panel_width, cap);
    const size_t cells_max = size_t(S) * Pmax;
    char* x0 = static_cast<char*>(st.x0.reserve(cells_max * elem));
    char* x1 = static_cast<char*>(st.x1.reserve(cells_max * elem));
    float* prm = static_cast<float*>(st.q.reserve(cells_max * 4 * 4 + kMaxP * 4));
    // [3 kMaxP stats: max|dB|, max|B|, max per-side change][16 flags]
    // [kMaxP colmax][2 kMaxP int8 step scales][4 kMaxP Chebyshev state]
    uint32_t* stats = static_cast<uint32_t*>(st.colstats.reserve((10 * kMaxP + 16) * 4));
    uint32_t* flag = stats + 3 * kMaxP;
    uint32_t* counter = flag + 8;
    float* colmax = reinterpret_cast<float*>(flag + 16);
    float* sig = colmax + kMaxP;  // two slots of kMaxP int8 step scales
    float* cheb = sig + 2 * kMaxP;
    // MIXED: wide panels run int8 steps (two int8 panels + the FP32
    // residual), narrow ones BF16 defect cycles (two BF16 panels).
    const bool wide_mixed = mixed && Pmax >= 32;
    __nv_bfloat16* dbuf = nullptr;
    int8_t* qbuf = nullptr;
    float* rbuf = nullptr;
    // (a trailing panel of fewer than 32 columns takes the BF16 path)
    if (mixed) dbuf = static_cast<__nv_bfloat16*>(st.half.reserve(cells_max * 2 * 2));
    if (wide_mixed) {
        qbuf = static_cast<int8_t*>(st.i8.reserve(cells_max * 2));
        rbuf = static_cast<float*>(st.corr.reserve(cells_max * 4));
    }

    uint32_t worst_iterations = 0, corrections = 0, launches = 0, sweeps = 0, timed_sweeps = 0;
    uint32_t graph_launches = 0;
    double sweep_seconds = 0.0, sweep_bytes = 0.0;
    const bool timed = (cfg.flags & FACETCU_BATCH_TIME_SWEEPS) != 0u;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (timed) {
        FCU_CHECK(cudaEventCreate(&t0));
        FCU_CHECK(cudaEventCreate(&t1));
    }
    // Algorithmic HBM bytes of one sweep: the graph once (packed or 8-byte
    // edges, row offsets, denominators, sky counts), the panel read and
    // written once, and the four per-side parameter planes.
    const double edge_bytes = g.packed ? 4.0 : 8.0;
    const double graph_bytes = double(gr.nnz) * edge_bytes + double(S + 1) * 4.0 + double(S) * 8.0;
    bool all_converged = true;
    float worst_change = 0.0f;
    const uint32_t max_it = cfg.maximum_iterations ? cfg.maximum_iterations : 1000u;
    const float tol = cfg.tolerance;
    const uint32_t check_every = 8;

    for (uint32_t c0 = 0; c0 < R;) {
        const int P = panel_width(R - c0, cfg.panel_width, uint32_t(Pmax));
        const size_t cells = size_t(S) * P;
        float* prho = prm;
        float* ptau = prm + cells;
        float* pemis = prm + 2 * cells;
        float* pdir = prm + 3 * cells;
        float* psky = prm + 4 * cells;
        PanelParams pp{prho, ptau, pemis, pdir, psky, colmax,
                       mixed && P >= 32 ? cheb + 2 * kMaxP : nullptr};
        __nv_bfloat16* d0 = dbuf;
        __nv_bfloat16* d1 = dbuf ? dbuf + cells : nullptr;
        // Per-cell bytes: full sweep = state in + out + rho, tau, emission,
        // direct; defect sweep = BF16 defect in + out + X read-modify-write +
        // rho, tau.  Only the dominant kind is timed (defect sweeps in MIXED).
        // int8 step: own Q in + Q out (1 + 1), X and R read-modify-write
        // (8 + 8), rho and tau (8) per cell.
        const double full_bytes = graph_bytes + double(cells) * (double(elem) * 2.0 + 16.0);
        const double defect_bytes = graph_bytes + double(cells) * (P >= 32 ? 26.0 : 20.0);
        auto timed_sweep = [&](bool defect, auto&& launch) {
            const bool count = timed && (defect == mixed);
            if (count) FCU_CHECK(cudaEventRecord(t0, s));
            launch();
            ++launches;
            ++sweeps;
            if (count) {
                FCU_CHECK(cudaEventRecord(t1, s));
                FCU_CHECK(cudaEventSynchronize(t1));
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, t0, t1);
                sweep_seconds += double(ms) * 1e-3;
                sweep_bytes += defect ? defect_bytes : full_bytes;
                ++timed_sweeps;
            }
        };
        launches += 4;  // prepare, sky, panel in, panel out
        k_prepare_panel<<<blocks_for(S, kPanelTile), 256, 0, s>>>(S, p.bands, R, c0, P, rank, p.rho,
                                                                p.tau, p.emis, p.beam, p.dgeo,
                                                                prho, ptau, pemis, pdir);
        FCU_LAUNCH("k_prepare_panel");
        k_panel_sky<<<1, 128, 0, s>>>(p.bands, R, c0, P, p.sky, psky);
        FCU_LAUNCH("k_panel_sky");
        FCU_CHECK(cudaMemsetAsync(stats, 0, (4 * kMaxP + 16) * 4, s));  // stats, flags, colmax
        const float* init = cfg.warm_start == FACETCU_WARM_GIVEN ? d_initial : nullptr;
        if (fp64)
            k_panel_in<double><<<blocks_for(S, kPanelTile), 256, 0, s>>>(
                init, S, R, c0, P, rank, reinterpret_cast<double*>(x0));
        else
            k_panel_in<float><<<blocks_for(S, kPanelTile), 256, 0, s>>>(
                init, S, R, c0, P, rank, reinterpret_cast<float*>(x0));
        FCU_LAUNCH("k_panel_in");
        // A solve from zero: its first sweep gathers nothing (null input).
        const bool zero_start = init == nullptr;

        uint32_t it = 0;
        int cur = 0;
        uint32_t host_flag[3] = {0, 0, 0};
        if (!mixed) {
            while (it < max_it) {
                const uint32_t batch = std::min(timed ? 1u : check_every, max_it - it);
                for (uint32_t k = 0; k < batch; ++k) {
                    const uint32_t sweep = it + k;
                    char* in = sweep == 0 && zero_start ? nullptr : (sweep & 1u) ? x1 : x0;
                    char* out = (sweep & 1u) ? x0 : x1;
                    timed_sweep(false, [&] {
                        if (fp64)
                            launch_sweep<double>(P, g, pp, reinterpret_cast<const double*>(in),
                                                 reinterpret_cast<double*>(out), stats, counter,
                                                 flag, s);
                        else
                            launch_sweep<float>(P, g, pp, reinterpret_cast<const float*>(in),
                                                reinterpret_cast<float*>(out), stats, counter,
                                                flag, s);
                    });
                    k_check<<<1, kMaxP, 0, s>>>(stats, flag, P, tol, sweep, counter, nullptr,
                                                nullptr, nullptr, true, colmax);
                    FCU_LAUNCH("k_check");
                    ++launches;
                }
                it += batch;
                FCU_CHECK(cudaMemcpyAsync(host_flag, flag, 12, cudaMemcpyDeviceToHost, s));
                FCU_CHECK(cudaStreamSynchronize(s));
                if (host_flag[0]) {
                    sweeps -= it - host_flag[1];  // launched after the done flag: no work
                    break;
                }
            }
            cur = int(host_flag[1] & 1u);
        } else if (P >= 32) {
            // FP32 sweep; then residual-tracked int8 steps until the
            // per-side test holds on their exact residual R (R_s is the
            // change the next Jacobi sweep would make to side s); then an
            // FP32 sweep verifies the per-side test.  If it fails there and
            // even the absolute test fails, the steps restart from the fresh
            // residual; if only sides far below the column's maximum are
            // still moving, plain FP32 sweeps finish them.  (The int8 steps
            // resolve a side only to about sigma/2 = max|R|/254 absolute;
            // every step shrinks sigma, so dim sides converge as the steps
            // go on.)
            const float step_tol = tol;
            float* X = reinterpret_cast<float*>(x0);
            float* Y = reinterpret_cast<float*>(x1);
            int8_t* qb[2] = {qbuf, qbuf + cells};
            float* slot[2] = {sig, sig + kMaxP};
            while (it < max_it) {
                timed_sweep(false, [&] {
                    launch_sweep<float>(P, g, pp, it == 0 && zero_start ? nullptr : X, Y, stats,
                                        counter, flag, s);
                });
                k_check<<<1, kMaxP, 0, s>>>(stats, flag, P, tol, it, counter, slot[0], slot[1],
                                            nullptr, true, colmax, cheb, 1);
                FCU_LAUNCH("k_check");
                launches += 1;
                ++it;
                ++corrections;
                uint32_t verdict[7];
                FCU_CHECK(cudaMemcpyAsync(verdict, flag, sizeof(verdict), cudaMemcpyDeviceToHost, s));
                FCU_CHECK(cudaStreamSynchronize(s));
                std::memcpy(host_flag, verdict, 12);
                if (host_flag[0] || it >= max_it) {
                    std::swap(X, Y);  // the newest iterate is the FP32 sweep's
                    break;
                }
                if (verdict[6]) {
                    // The absolute test holds and only sides far below the
                    // column's maximum are still moving: plain FP32 sweeps
                    // finish them (their error shrinks with every sweep).
                    std::swap(X, Y);
                    continue;
                }
                if (g.scene) {
                    // every scene takes part in a new int8 phase, with its
                    // own first scales max|Y - X| / 127
                    FCU_CHECK(cudaMemsetAsync(g.scene_stats, 0,
                                              size_t(g.scenes) * (8 * kMaxP + 1) * 4, s));
                    k_scene_init_md<<<(S + 255) / 256, P, 0, s>>>(X, Y, g.scene, S, P, g.scene_md);
                    FCU_LAUNCH("k_scene_init_md");
                    k_scene_init_sigma<<<g.scenes, kMaxP, 0, s>>>(g.scene_md, g.scene_sig,
                                                                  g.scene_cheb, g.scenes, P);
                    FCU_LAUNCH("k_scene_init_sigma");
                    launches += 2;
                }
                k_init_i8<<<blocks_for(cells, 256), 256, 0, s>>>(X, Y, rbuf, qb[0], slot[0], cells,
                                                                 P, flag + 12, it, g.scene,
                                                                 g.scene_sig);
                FCU_LAUNCH("k_init_i8");
                ++launches;
                uint32_t j = 0;
                bool steps_done = false;
                while (!steps_done && it < max_it) {
                    const uint32_t batch = std::min(timed ? 1u : check_every, max_it - it);
                    if (!timed && !st.no_loop_graph && max_it - it >= kStepBatch && (j & 1u) == 0u) {
                        // the rest of the phase as one launch (j even: the
                        // captured parity pattern applies)
                        StepGraphKey key;
                        std::memset(&key, 0, sizeof(key));  // padding takes part in the compare
                        key.P = P;
                        key.g = g;
                        key.pp = pp;
                        key.q0 = qb[0];
                        key.q1 = qb[1];
                        key.X = X;
                        key.R = rbuf;
                        key.slot0 = slot[0];
                        key.slot1 = slot[1];
                        key.stats = stats;
                        key.flag = flag;
                        key.tol = step_tol;
                        key.limit = max_it;
                        key.stream = s;
                        const cudaGraphExec_t loop_graph = step_graph(st, key);
                        if (!loop_graph) continue;  // launch the steps one by one
                        FCU_CHECK(cudaGraphLaunch(loop_graph, s));
                        ++graph_launches;
                        uint32_t fl[10];  // flag[3 .. 12]: the phase's flags, the device counter
                        FCU_CHECK(cudaMemcpyAsync(fl, flag + 3, sizeof(fl), cudaMemcpyDeviceToHost, s));
                        FCU_CHECK(cudaStreamSynchronize(s));
                        const uint32_t ran = fl[9] - it;  // steps launched (each one checked)
                        launches += (g.scene ? 3 : 2) * ran + ran / kStepBatch;
                        sweeps += ran;
                        j += ran;
                        it += ran;
                        if (fl[0]) {
                            steps_done = true;
                            sweeps -= it - fl[1];  // launched after the target: no work
                            it = fl[1];
                            FCU_CHECK(cudaMemsetAsync(flag + 3, 0, 12, s));
                        }
                        continue;
                    } else
                    for (uint32_t k = 0; k < batch; ++k, ++j) {
                        const float* sin = slot[j & 1u];
                        const float* sout = slot[(j + 1) & 1u];
                        timed_sweep(true, [&] {
                            launch_step_i8(P, g, pp, qb[j & 1u], qb[(j + 1) & 1u], X, rbuf, sin,
                                           sout, stats, counter, flag + 3, j & 1u, s);
                        });
                        // slot j & 1 (sigma of the panel just consumed) takes
                        // max|R_new| / 127 for the step after next
                        k_check<<<1, kMaxP, 0, s>>>(stats, flag + 3, P, step_tol, it + k,
                                                    counter, slot[j & 1u], nullptr, nullptr,
                                                    true, colmax, cheb, 2, slot[(j + 1) & 1u]);
                        FCU_LAUNCH("k_check");
                        launch_scene_check(g, P, j & 1u, step_tol, s);
                        launches += g.scene ? 2 : 1;
                    }
                    it += batch;
                    uint32_t sub_flag[3];
                    FCU_CHECK(cudaMemcpyAsync(sub_flag, flag + 3, 12, cudaMemcpyDeviceToHost, s));
                    FCU_CHECK(cudaStreamSynchronize(s));
                    if (sub_flag[0]) {
                        steps_done = true;
                        sweeps -= it - sub_flag[1];  // launched after the target: no work
                        it = sub_flag[1];
                        FCU_CHECK(cudaMemsetAsync(flag + 3, 0, 12, s));
                    }
                }
            }
            cur = X == reinterpret_cast<float*>(x0) ? 0 : 1;
            host_flag[1] = it;
        } else {
            // FP32 sweep, then BF16 defect sweeps until the defect has shrunk
            // by `cycle_drop`, then a fresh FP32 sweep (residual correction).
            const float cycle_drop = 1.0f / 64.0f;
            float* X = reinterpret_cast<float*>(x0);
            float* Y = reinterpret_cast<float*>(x1);
            while (it < max_it) {
                timed_sweep(false, [&] {
                    launch_sweep<float>(P, g, pp, it == 0 && zero_start ? nullptr : X, Y, stats,
                                        counter, flag, s);
                });
                k_check<<<1, kMaxP, 0, s>>>(stats, flag, P, tol, it, counter, nullptr, nullptr,
                                            nullptr, true, colmax);
                FCU_LAUNCH("k_check");
                ++launches;
                ++it;
                ++corrections;
                FCU_CHECK(cudaMemcpyAsync(host_flag, flag, 12, cudaMemcpyDeviceToHost, s));
                FCU_CHECK(cudaStreamSynchronize(s));
                if (host_flag[0]) {
                    std::swap(X, Y);
                    break;
                }
                float start_change;
                std::memcpy(&start_change, &host_flag[2], 4);
                k_defect_init<<<blocks_for(cells, 256), 256, 0, s>>>(X, Y, d0, cells, flag);
                FCU_LAUNCH("k_defect_init");
                ++launches;
                std::swap(X, Y);  // X = newest FP32 iterate
                __nv_bfloat16* din = d0;
                __nv_bfloat16* dout = d1;
                bool cycle_done = false;
                // The defect sweeps read the cycle's own done flag (flag + 3):
                // once k_check has seen the target drop, the remaining sweeps
                // of the batch return at once and leave X and the defect
                // buffers untouched.  Timed runs check after every sweep so
                // that no such empty launch is timed.
                while (!cycle_done && it < max_it) {
                    const uint32_t batch = std::min(timed ? 1u : check_every, max_it - it);
                    uint32_t sub_flag[3];
                    for (uint32_t k = 0; k < batch; ++k) {
                        timed_sweep(true, [&] {
                            launch_defect(P, g, pp, din, dout, X, stats, counter, flag + 3, s);
                        });
                        std::swap(din, dout);
                        k_check<<<1, kMaxP, 0, s>>>(stats, flag + 3, P,
                                                    std::max(tol, start_change * cycle_drop),
                                                    it + k, counter, nullptr, nullptr, nullptr,
                                                    false, colmax);
                        FCU_LAUNCH("k_check");
                        launches += g.scene ? 2 : 1;
                    }
                    it += batch;
                    FCU_CHECK(cudaMemcpyAsync(sub_flag, flag + 3, 12, cudaMemcpyDeviceToHost, s));
                    FCU_CHECK(cudaStreamSynchronize(s));
                    if (sub_flag[0]) {
                        cycle_done = true;
                        sweeps -= it - sub_flag[1];  // skipped after the target drop
                        it = sub_flag[1];
                        FCU_CHECK(cudaMemsetAsync(flag + 3, 0, 12, s));
                    }
                }
            }
            cur = X == reinterpret_cast<float*>(x0) ? 0 : 1;
            host_flag[1] = it;
        }
        const char* final_buf = cur ? x1 : x0;
        if (fp64)
            k_panel_out<double><<<blocks_for(S, kPanelTile), 256, 0, s>>>(
                reinterpret_cast<const double*>(final_buf), S, R, c0, P, rank, d_out);
        else
            k_panel_out<float><<<blocks_for(S, kPanelTile), 256, 0, s>>>(
                reinterpret_cast<const float*>(final_buf), S, R, c0, P, rank, d_out);
        FCU_LAUNCH("k_panel_out");
        worst_iterations = std::max(worst_iterations, host_flag[1]);
        float change;
        std::memcpy(&change, &host_flag[2], 4);
        worst_change = std::max(worst_change, change);
        if (!host_flag[0]) all_converged = false;
        FCU_CHECK(cudaMemsetAsync(flag, 0, 48, s));
        c0 += uint32_t(P);
    }
    FCU_CHECK(cudaStreamSynchronize(s));
    if (timed) {
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
    }
    if (result) {
        result->kernel_launches = launches;
        result->sweeps = sweeps;
        result->sweep_seconds = sweep_seconds;
        result->sweep_bytes = sweep_bytes;
        result->timed_sweeps = timed_sweeps;
        result->iterations = worst_iterations;
        result->residual_corrections = corrections;
        result->converged = all_converged ? 1u : 0u;
        result->max_relative_change = worst_change;
        result->graph_launches = graph_launches;
    }
    return all_converged ? FACETCU_OK : FACETCU_NOT_CONVERGED;
}

}  // namespace facetcu
