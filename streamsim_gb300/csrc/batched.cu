// batched.cu — many right-hand sides (bands x suns) against one graph.
//
// The sweep is the reference's two-sided Jacobi update (radiosity.comp:63-106,
// solveCpu facetrtcore.cpp:1476-1529) applied to a panel of P RHS columns at
// once:
//   H_s,c  = (sky_s * L_c + sum_e count_e * B_{n_e,c}) / denom_s + D_s,c
//   B'_s,c = e_s,c + rho_s,c * H_s,c + tau_s,c * H_{s^1},c
// (denom_s = 0: H = L_c + D_s,c).
//
// GB300 mapping.  The panel is stored side-major ([S][P], P <= 32 floats per
// side), so one warp owns one facet (both sides) and the gather of neighbour
// n reads one contiguous P-float row: for P = 32 a single 128-byte line per
// edge, shared by every column.  The graph is read once per sweep for all
// P columns, from a packed 4-byte edge array (22-bit neighbour, 10-bit
// count) when it fits.  The grid is persistent (a multiple of the SM count);
// each warp keeps per-column max|dB| and max|B| in registers and one
// atomicMax per CTA and column publishes them.  A one-block check kernel
// after every sweep sets a device-side done flag, so sweeps run in batches
// without host round trips and stop at the exact sweep that converged.
//
// Precision modes:
//   FP32  — panel and gather in FP32 (the plain batched solver);
//   FP64  — the same sweep in double (the truth the 1e-4 bar is checked on);
//   MIXED — defect iteration: an FP32 sweep gives d = B' - B; then
//           d <- K d runs with d stored in BF16 (half the gather bytes),
//           accumulated in FP32 and added to the FP32 panel; every cycle
//           restarts from a fresh FP32 sweep (the FP32 residual correction).
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>

#include "internal.h"

namespace facetcu {
namespace {

constexpr int kWarps = 8;  // warps per CTA
constexpr uint32_t kNeighborMask = (1u << 22) - 1u;

struct PanelParams {
    // per side and column, [S][P]
    const float* rho;
    const float* tau;
    const float* emis;
    const float* direct;
    const float* skyL;  // [P]
};

struct GraphView {
    const uint32_t* rows;
    const uint32_t* packed;            // when non-null
    const facetcu_csr_edge* edges;     // otherwise
    const uint32_t* denom;
    const uint32_t* skyc;
    uint32_t facets;
};

__device__ __forceinline__ void edge_at(const GraphView& g, uint32_t e, uint32_t& nb, float& c)
{
    if (g.packed) {
        const uint32_t p = __ldg(g.packed + e);
        nb = p & kNeighborMask;
        c = float(p >> 22);
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

// Row gather: sum over the edges of side s of count * X[n*P + col], for the
// lane's column; lanes are split into 32/P groups that take every
// (32/P)-th edge, then reduced.  Acc is float for FP32/BF16 and double for FP64.
template <int P, typename T, typename Acc>
__device__ __forceinline__ Acc gather_row(const GraphView& g, uint32_t s, const T* X, int lane)
{
    constexpr int G = 32 / P;
    const int grp = lane / P, col = lane % P;
    const uint32_t start = g.rows[s], end = g.rows[s + 1];
    Acc acc = 0;
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
#pragma unroll
    for (int o = P; o < 32; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}

template <typename T> __device__ __forceinline__ float absf(T x) { return float(x < T(0) ? -x : x); }

__device__ __forceinline__ void publish_stats(float md, float mb, int lane, int P, uint32_t* stats)
{
    // CTA-level max over warps, then one atomic per column.
    __shared__ float s_md[kWarps][32], s_mb[kWarps][32];
    const int warp = threadIdx.x >> 5;
    s_md[warp][lane] = md;
    s_mb[warp][lane] = mb;
    __syncthreads();
    if (warp == 0 && lane < P) {
        float a = 0.0f, b = 0.0f;
        for (int w = 0; w < kWarps; ++w) {
            a = fmaxf(a, s_md[w][lane]);
            b = fmaxf(b, s_mb[w][lane]);
        }
        atomicMax(stats + lane, __float_as_uint(a));
        atomicMax(stats + 32 + lane, __float_as_uint(b));
    }
}

// One full sweep B_out = Q + K B_in over the panel (FP32 or FP64 state).
template <int P, typename T>
__global__ void __launch_bounds__(kWarps * 32) k_sweep(GraphView g, PanelParams pp, const T* Bin,
                                                       T* Bout, uint32_t* stats,
                                                       const uint32_t* done)
{
    if (*done) return;
    using Acc = T;
    const int lane = threadIdx.x & 31;
    const int col = lane % P;
    const uint32_t warps_total = gridDim.x * kWarps;
    float md = 0.0f, mb = 0.0f;
    const Acc L = Acc(pp.skyL[col]);
    for (uint32_t f = blockIdx.x * kWarps + (threadIdx.x >> 5); f < g.facets; f += warps_total) {
        const uint32_t s0 = 2u * f, s1 = s0 + 1u;
        Acc h[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const uint32_t s = s0 + k;
            const Acc acc = gather_row<P, T, Acc>(g, s, Bin, lane);
            const uint32_t d = g.denom[s];
            const Acc dir = Acc(pp.direct[size_t(s) * P + col]);
            h[k] = (d == 0u ? L : (Acc(g.skyc[s]) * L + acc) / Acc(d)) + dir;
        }
        if (lane < P) {
            const size_t i0 = size_t(s0) * P + col, i1 = size_t(s1) * P + col;
            const Acc b0 = Acc(pp.emis[i0]) + Acc(pp.rho[i0]) * h[0] + Acc(pp.tau[i0]) * h[1];
            const Acc b1 = Acc(pp.emis[i1]) + Acc(pp.rho[i1]) * h[1] + Acc(pp.tau[i1]) * h[0];
            const Acc o0 = Bin[i0], o1 = Bin[i1];
            Bout[i0] = b0;
            Bout[i1] = b1;
            md = fmaxf(md, fmaxf(absf(b0 - o0), absf(b1 - o1)));
            mb = fmaxf(mb, fmaxf(absf(b0), absf(b1)));
        }
    }
    publish_stats(md, mb, lane, P, stats);
}

// Defect sweep of the MIXED mode: d_out = K d_in with d in BF16, FP32
// accumulation; X += d_out (FP32 panel).  Stats: max|d_out|, max|X|.
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
    const uint32_t warps_total = gridDim.x * kWarps;
    float md = 0.0f, mb = 0.0f;
    for (uint32_t f = blockIdx.x * kWarps + (threadIdx.x >> 5); f < g.facets; f += warps_total) {
        const uint32_t s0 = 2u * f, s1 = s0 + 1u;
        float h[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const uint32_t s = s0 + k;
            const float acc = gather_row<P, __nv_bfloat16, float>(g, s, Din, lane);
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
            md = fmaxf(md, fmaxf(fabsf(d0), fabsf(d1)));
            mb = fmaxf(mb, fmaxf(fabsf(x0), fabsf(x1)));
        }
    }
    publish_stats(md, mb, lane, P, stats);
}

// d = Bnew - Bold (FP32) -> BF16, and keep Bnew as the FP32 panel in place.
__global__ void k_defect_init(const float* Bold, const float* Bnew, __nv_bfloat16* D, size_t n,
                              const uint32_t* done)
{
    if (*done) return;
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) D[i] = __float2bfloat16_rn(Bnew[i] - Bold[i]);
}

// Convergence check after sweep `it` (0-based): every active column must
// satisfy max|dB| <= tol * max|B|.  flag[0] = done, flag[1] = sweeps run,
// flag[2] = max relative change bits of the last sweep.
__global__ void k_check(uint32_t* stats, uint32_t* flag, int P, float tol, uint32_t it)
{
    __shared__ int all_ok;
    __shared__ float worst;
    if (threadIdx.x == 0) {
        all_ok = 1;
        worst = 0.0f;
    }
    __syncthreads();
    const bool already = flag[0] != 0u;
    if (threadIdx.x < uint32_t(P)) {
        const float md = __uint_as_float(stats[threadIdx.x]);
        const float mb = __uint_as_float(stats[32 + threadIdx.x]);
        const float rel = mb > 0.0f ? md / mb : (md > 0.0f ? INFINITY : 0.0f);
        if (!(md <= tol * mb) && !(md == 0.0f)) atomicExch(&all_ok, 0);
        atomicMax(reinterpret_cast<int*>(&worst), __float_as_int(rel));
    }
    __syncthreads();
    if (threadIdx.x == 0 && !already) {
        flag[1] = it + 1;
        flag[2] = __float_as_uint(worst);
        if (all_ok) flag[0] = 1;
    }
    if (threadIdx.x < 64) stats[threadIdx.x] = 0;
}

// Panel parameters for columns [c0, c0 + P) (column c = sun * bands + band).
__global__ void k_prepare_panel(uint32_t S, uint32_t bands, uint32_t R, uint32_t c0, int P,
                                const float* rho, const float* tau, const float* emis,
                                const float* beam, const float* dgeo, float* prho, float* ptau,
                                float* pemis, float* pdir)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= size_t(S) * P) return;
    const uint32_t s = uint32_t(i / P);
    const uint32_t j = uint32_t(i % P);
    const uint32_t c = c0 + j;
    if (c >= R) {
        prho[i] = 0.0f;
        ptau[i] = 0.0f;
        pemis[i] = 0.0f;
        pdir[i] = 0.0f;
        return;
    }
    const uint32_t b = c % bands, k = c / bands;
    const size_t bi = size_t(b) * S + s;
    prho[i] = rho[bi];
    ptau[i] = tau[bi];
    pemis[i] = emis ? emis[bi] : 0.0f;
    pdir[i] = dgeo ? beam[b] * dgeo[size_t(k) * S + s] : 0.0f;
}

__global__ void k_panel_sky(uint32_t bands, uint32_t R, uint32_t c0, int P, const float* sky,
                            float* psky)
{
    const int j = threadIdx.x;
    if (j >= P) return;
    const uint32_t c = c0 + j;
    psky[j] = c < R ? sky[c % bands] : 0.0f;
}

// [R][S] <-> [S][P] panel copies.
template <typename T>
__global__ void k_panel_in(const float* src, uint32_t S, uint32_t R, uint32_t c0, int P, T* dst)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= size_t(S) * P) return;
    const uint32_t s = uint32_t(i / P), j = uint32_t(i % P), c = c0 + j;
    dst[i] = (src && c < R) ? T(src[size_t(c) * S + s]) : T(0);
}

template <typename T>
__global__ void k_panel_out(const T* src, uint32_t S, uint32_t R, uint32_t c0, int P, float* dst)
{
    // tile transpose through shared memory: 32 sides x P columns per block
    __shared__ float tile[32][33];
    const uint32_t sb = blockIdx.x * 32;
    const int t = threadIdx.x;  // 256 threads
    for (int k = t; k < 32 * P; k += blockDim.x) {
        const int ls = k / P, j = k % P;
        const uint32_t s = sb + ls;
        tile[ls][j] = s < S ? float(src[size_t(s) * P + j]) : 0.0f;
    }
    __syncthreads();
    for (int k = t; k < 32 * P; k += blockDim.x) {
        const int j = k / 32, ls = k % 32;
        const uint32_t s = sb + ls, c = c0 + j;
        if (s < S && c < R) dst[size_t(c) * S + s] = tile[ls][j];
    }
}

inline unsigned blocks_for(size_t n, unsigned b) { return unsigned((n + b - 1) / b); }

int persistent_grid()
{
    static int grid = 0;
    if (!grid) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        grid = (sms > 0 ? sms : 148) * 6;  // 6 CTAs x 8 warps = 48 warps per SM
    }
    return grid;
}

template <typename T>
void launch_sweep(int P, const GraphView& g, const PanelParams& pp, const T* in, T* out,
                  uint32_t* stats, const uint32_t* done, cudaStream_t s)
{
    const int grid = persistent_grid();
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

void launch_defect(int P, const GraphView& g, const PanelParams& pp, const __nv_bfloat16* in,
                   __nv_bfloat16* out, float* X, uint32_t* stats, const uint32_t* done,
                   cudaStream_t s)
{
    const int grid = persistent_grid();
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

int panel_width_for(uint32_t R, uint32_t requested)
{
    uint32_t p = requested ? requested : 32u;
    if (p > 32u) p = 32u;
    uint32_t w = 1;
    while (w < p && w < R) w <<= 1;
    return int(w);
}

}  // namespace

// Host driver.  Returns FACETCU_OK or FACETCU_NOT_CONVERGED.
int batched_solve(const DeviceGraph& gr, const BatchProblem& p, const facetcu_batch_config& cfg,
                  const float* d_initial, float* d_out, BatchState& st, Workspace& ws,
                  cudaStream_t s, facetcu_batch_result* result)
{
    (void)ws;
    const uint32_t S = p.S, R = p.bands * p.suns;
    const int P = panel_width_for(R, cfg.panel_width);
    const size_t cells = size_t(S) * P;
    const bool fp64 = cfg.precision == 2u;
    const bool mixed = cfg.precision == FACETCU_PRECISION_MIXED;
    const size_t elem = fp64 ? 8 : 4;
    char* x0 = static_cast<char*>(st.x0.reserve(cells * elem));
    char* x1 = static_cast<char*>(st.x1.reserve(cells * elem));
    float* prm = static_cast<float*>(st.q.reserve(cells * 4 * 4 + 64 * 4));
    float* prho = prm;
    float* ptau = prm + cells;
    float* pemis = prm + 2 * cells;
    float* pdir = prm + 3 * cells;
    float* psky = prm + 4 * cells;
    uint32_t* stats = static_cast<uint32_t*>(st.colstats.reserve(256 * 4));
    uint32_t* flag = stats + 64;
    __nv_bfloat16* d0 = nullptr;
    __nv_bfloat16* d1 = nullptr;
    if (mixed) {
        d0 = static_cast<__nv_bfloat16*>(st.half.reserve(cells * 2 * 2));
        d1 = d0 + cells;
    }
    GraphView g;
    g.rows = gr.row_offsets.as<uint32_t>();
    g.packed = gr.packed_valid ? gr.packed.as<uint32_t>() : nullptr;
    g.edges = gr.edges.as<facetcu_csr_edge>();
    g.denom = gr.denominators.as<uint32_t>();
    g.skyc = gr.sky.as<uint32_t>();
    g.facets = S / 2u;
    PanelParams pp{prho, ptau, pemis, pdir, psky};

    uint32_t worst_iterations = 0, corrections = 0, launches = 0, sweeps = 0;
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
    const double edge_bytes = gr.packed_valid ? 4.0 : 8.0;
    const double graph_bytes = double(gr.nnz) * edge_bytes + double(S + 1) * 4.0 + double(S) * 8.0;
    const double panel_bytes = double(cells) * double(elem) * 2.0 + double(cells) * 16.0;
    auto timed_sweep = [&](auto&& launch) {
        if (timed) FCU_CHECK(cudaEventRecord(t0, s));
        launch();
        ++launches;
        ++sweeps;
        if (timed) {
            FCU_CHECK(cudaEventRecord(t1, s));
            FCU_CHECK(cudaEventSynchronize(t1));
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, t0, t1);
            sweep_seconds += double(ms) * 1e-3;
            sweep_bytes += graph_bytes + panel_bytes;
        }
    };
    bool all_converged = true;
    float worst_change = 0.0f;
    const uint32_t max_it = cfg.maximum_iterations ? cfg.maximum_iterations : 1000u;
    const float tol = cfg.tolerance;
    const uint32_t check_every = 8;

    for (uint32_t c0 = 0; c0 < R; c0 += uint32_t(P)) {
        launches += 4;  // prepare, sky, panel in, panel out
        k_prepare_panel<<<blocks_for(cells, 256), 256, 0, s>>>(S, p.bands, R, c0, P, p.rho, p.tau,
                                                                p.emis, p.beam, p.dgeo, prho, ptau,
                                                                pemis, pdir);
        FCU_LAUNCH("k_prepare_panel");
        k_panel_sky<<<1, 32, 0, s>>>(p.bands, R, c0, P, p.sky, psky);
        FCU_LAUNCH("k_panel_sky");
        FCU_CHECK(cudaMemsetAsync(stats, 0, 128 * 4, s));
        const float* init = cfg.warm_start == FACETCU_WARM_GIVEN ? d_initial : nullptr;
        if (fp64)
            k_panel_in<double><<<blocks_for(cells, 256), 256, 0, s>>>(
                init, S, R, c0, P, reinterpret_cast<double*>(x0));
        else
            k_panel_in<float><<<blocks_for(cells, 256), 256, 0, s>>>(
                init, S, R, c0, P, reinterpret_cast<float*>(x0));
        FCU_LAUNCH("k_panel_in");

        uint32_t it = 0;
        int cur = 0;  // buffer holding the current iterate (FP32/FP64 modes)
        uint32_t host_flag[3] = {0, 0, 0};
        if (!mixed) {
            while (it < max_it) {
                const uint32_t batch = std::min(check_every, max_it - it);
                for (uint32_t k = 0; k < batch; ++k) {
                    const uint32_t sweep = it + k;
                    char* in = (sweep & 1u) ? x1 : x0;
                    char* out = (sweep & 1u) ? x0 : x1;
                    timed_sweep([&] {
                        if (fp64)
                            launch_sweep<double>(P, g, pp, reinterpret_cast<const double*>(in),
                                                 reinterpret_cast<double*>(out), stats, flag, s);
                        else
                            launch_sweep<float>(P, g, pp, reinterpret_cast<const float*>(in),
                                                reinterpret_cast<float*>(out), stats, flag, s);
                    });
                    k_check<<<1, 64, 0, s>>>(stats, flag, P, tol, sweep);
                    FCU_LAUNCH("k_check");
                    ++launches;
                }
                it += batch;
                FCU_CHECK(cudaMemcpyAsync(host_flag, flag, 12, cudaMemcpyDeviceToHost, s));
                FCU_CHECK(cudaStreamSynchronize(s));
                if (host_flag[0]) break;
            }
            const uint32_t done_sweeps = host_flag[1];
            cur = int(done_sweeps & 1u);
        } else {
            // FP32 sweep, then BF16 defect sweeps until the defect has shrunk
            // by `cycle_drop`, then a fresh FP32 sweep (residual correction).
            const float cycle_drop = 1.0f / 64.0f;
            float* X = reinterpret_cast<float*>(x0);
            float* Y = reinterpret_cast<float*>(x1);
            while (it < max_it) {
                // FP32 residual sweep: Y = Q + K X; converged check on it.
                timed_sweep([&] { launch_sweep<float>(P, g, pp, X, Y, stats, flag, s); });
                k_check<<<1, 64, 0, s>>>(stats, flag, P, tol, it);
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
                // defect sweeps in batches; stop the cycle when the relative
                // defect fell below start_change * cycle_drop or under tol
                __nv_bfloat16* din = d0;
                __nv_bfloat16* dout = d1;
                bool cycle_done = false;
                while (!cycle_done && it < max_it) {
                    const uint32_t batch = std::min(check_every, max_it - it);
                    uint32_t sub_flag[3];
                    for (uint32_t k = 0; k < batch; ++k) {
                        timed_sweep([&] { launch_defect(P, g, pp, din, dout, X, stats, flag, s); });
                        std::swap(din, dout);
                        k_check<<<1, 64, 0, s>>>(stats, flag + 3, P,
                                                 std::max(tol, start_change * cycle_drop),
                                                 it + k);
                        FCU_LAUNCH("k_check");
                        ++launches;
                    }
                    it += batch;
                    FCU_CHECK(cudaMemcpyAsync(sub_flag, flag + 3, 12, cudaMemcpyDeviceToHost, s));
                    FCU_CHECK(cudaStreamSynchronize(s));
                    if (sub_flag[0]) {
                        cycle_done = true;
                        // sweeps after the one that met the cycle target still
                        // ran (no early exit inside a batch); count them
                        FCU_CHECK(cudaMemsetAsync(flag + 3, 0, 12, s));
                    }
                }
            }
            cur = X == reinterpret_cast<float*>(x0) ? 0 : 1;
            host_flag[1] = it;
        }
        const char* final_buf = cur ? x1 : x0;
        if (fp64) {
            // FP64 panels are returned rounded to float
            k_panel_out<double><<<blocks_for(S, 32), 256, 0, s>>>(
                reinterpret_cast<const double*>(final_buf), S, R, c0, P, d_out);
        } else {
            k_panel_out<float><<<blocks_for(S, 32), 256, 0, s>>>(
                reinterpret_cast<const float*>(final_buf), S, R, c0, P, d_out);
        }
        FCU_LAUNCH("k_panel_out");
        worst_iterations = std::max(worst_iterations, host_flag[1]);
        float change;
        std::memcpy(&change, &host_flag[2], 4);
        worst_change = std::max(worst_change, change);
        if (!host_flag[0]) all_converged = false;
        FCU_CHECK(cudaMemsetAsync(flag, 0, 32, s));
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
        result->iterations = worst_iterations;
        result->residual_corrections = corrections;
        result->converged = all_converged ? 1u : 0u;
        result->max_relative_change = worst_change;
    }
    return all_converged ? FACETCU_OK : FACETCU_NOT_CONVERGED;
}

}  // namespace facetcu
