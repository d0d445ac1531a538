/*
 * facet_oracle.c — TEST INFRASTRUCTURE ONLY (see facet_oracle.h).
 *
 * CPU restatement of StreamSim HiStream FacetRT (eFacetRT) for parity tests.
 * Every function cites the reference lines it follows.  Compile with
 * -ffp-contract=off: the expressions below keep the reference's operation
 * order so that each float rounds exactly as the reference's does.
 */
#include "facet_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct { float v[3]; } vec3;

static vec3 v3(float x, float y, float z) { vec3 r = {{x, y, z}}; return r; }
static vec3 vadd(vec3 a, vec3 b) { return v3(a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2]); }
static vec3 vsub(vec3 a, vec3 b) { return v3(a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2]); }
static vec3 vmul(vec3 a, float s) { return v3(a.v[0] * s, a.v[1] * s, a.v[2] * s); }
static float vdot(vec3 a, vec3 b) { return a.v[0] * b.v[0] + a.v[1] * b.v[1] + a.v[2] * b.v[2]; }
static vec3 vcross(vec3 a, vec3 b)
{
    return v3(a.v[1] * b.v[2] - a.v[2] * b.v[1],
              a.v[2] * b.v[0] - a.v[0] * b.v[2],
              a.v[0] * b.v[1] - a.v[1] * b.v[0]);
}
/* facetrtcore.cpp:262-269: multiply by the reciprocal of the length. */
static int vnormalized(vec3 a, vec3 *out)
{
    const float length = sqrtf(vdot(a, a));
    if (!(length > 1.0e-8f)) return -1;
    *out = vmul(a, 1.0f / length);
    return 0;
}

/* std::min / std::max semantics (first argument wins ties). */
static float stdmin(float a, float b) { return b < a ? b : a; }
static float stdmax(float a, float b) { return a < b ? b : a; }

void orc_free(void *p) { free(p); }

/* facetrtcore.cpp:475-489 */
void orc_hemisphere_directions(uint32_t count, orc_direction *out)
{
    const float golden = 2.39996322972865332f;
    for (uint32_t i = 0; i < count; ++i) {
        const float y = ((float)i + 0.5f) / (float)count;
        const float r = sqrtf(fmaxf(0.0f, 1.0f - y * y));
        const float az = golden * (float)i;
        out[i].x = r * cosf(az);
        out[i].y = y;
        out[i].z = r * sinf(az);
    }
}

/* facetrtcore.cpp:491-498 */
orc_direction orc_sun_direction(float zenith_deg, float azimuth_deg)
{
    const float pi = 3.14159265358979323846f;
    const float zen = zenith_deg * pi / 180.0f;
    const float az = azimuth_deg * pi / 180.0f;
    orc_direction d = {sinf(zen) * cosf(az), cosf(zen), sinf(zen) * sinf(az)};
    return d;
}

/* facetrtcore.cpp:168-188 */
uint32_t orc_adaptive_layers(uint32_t facet_count, uint32_t periodic_count,
                             uint32_t raster_size, uint32_t base_layers)
{
    const double pixels = (double)raster_size * raster_size;
    if (pixels <= 0.0) return base_layers;
    const double avg = (double)facet_count * (double)(periodic_count + 1U) / pixels;
    double est = avg * 16.0;
    if (est < 1.0) est = 1.0;
    const uint32_t estimated = (uint32_t)ceil(est);
    uint32_t layers = base_layers;
    while (layers < estimated && layers < 64U) {
        layers = layers * 2U < 64U ? layers * 2U : 64U;
    }
    return layers;
}

/* facetrtcore.cpp:226-237 */
static void periodic_tile(uint32_t index, int *tx, int *tz)
{
    static const int off[20][2] = {
        {-1, 0}, {1, 0}, {0, -1}, {0, 1}, {-1, -1}, {-1, 1}, {1, -1}, {1, 1},
        {-2, 0}, {2, 0}, {0, -2}, {0, 2}, {-2, -1}, {-2, 1}, {2, -1}, {2, 1},
        {-1, -2}, {1, -2}, {-1, 2}, {1, 2}};
    if (index == 0U) { *tx = 0; *tz = 0; return; }
    const uint32_t k = index - 1U < 19U ? index - 1U : 19U;
    *tx = off[k][0];
    *tz = off[k][1];
}

/* ------------------------------------------------------------------------ */
/* A-buffer rasterizer: facetrtcore.cpp:1212-1344 (CpuRasterizer).          */
/* ------------------------------------------------------------------------ */
typedef struct { float depth; uint32_t side; } fragment;

typedef struct {
    const orc_vertex *vertices;
    uint32_t facets;
    const orc_raster_config *cfg;
    uint32_t width, height, layers;
    vec3 center;
    float radius;
    uint32_t *counts;
    fragment *frags;
} rasterizer;

static int raster_init(rasterizer *r, const orc_vertex *v, uint32_t facets,
                       const orc_raster_config *cfg)
{
    r->vertices = v;
    r->facets = facets;
    r->cfg = cfg;
    r->width = cfg->raster_size;
    r->height = cfg->raster_size;
    r->layers = cfg->layers;
    vec3 emin = v3(cfg->bounds_min[0], cfg->bounds_min[1], cfg->bounds_min[2]);
    vec3 emax = v3(cfg->bounds_max[0], cfg->bounds_max[1], cfg->bounds_max[2]);
    for (uint32_t t = 1U; t <= cfg->periodic_count; ++t) {
        int tx, tz;
        periodic_tile(t, &tx, &tz);
        const float ox = (float)tx * cfg->periodic_size_x;
        const float oz = (float)tz * cfg->periodic_size_z;
        emin.v[0] = stdmin(emin.v[0], cfg->bounds_min[0] + ox);
        emax.v[0] = stdmax(emax.v[0], cfg->bounds_max[0] + ox);
        emin.v[2] = stdmin(emin.v[2], cfg->bounds_min[2] + oz);
        emax.v[2] = stdmax(emax.v[2], cfg->bounds_max[2] + oz);
    }
    const vec3 diag = vsub(emax, emin);
    r->center = vmul(vadd(emin, emax), 0.5f);
    r->radius = stdmax(0.5f * sqrtf(vdot(diag, diag)) * 1.001f, 1.0e-4f);
    const size_t pixels = (size_t)r->width * r->height;
    r->counts = (uint32_t *)calloc(pixels, sizeof(uint32_t));
    r->frags = (fragment *)malloc(pixels * r->layers * sizeof(fragment));
    return (r->counts && r->frags) ? 0 : -1;
}

static void raster_free(rasterizer *r)
{
    free(r->counts);
    free(r->frags);
}

static float edgef(float ax, float ay, float bx, float by, float px, float py)
{
    return (px - ax) * (by - ay) - (py - ay) * (bx - ax);
}

static float min3f(float a, float b, float c) { float m = a; if (b < m) m = b; if (c < m) m = c; return m; }
static float max3f(float a, float b, float c) { float m = a; if (m < b) m = b; if (m < c) m = c; return m; }

/* facetrtcore.cpp:1292-1334 */
static void raster_triangle(rasterizer *r, const float px[3], const float py[3],
                            const float pd[3], uint32_t side, uint32_t *overflow)
{
    const float area = edgef(px[0], py[0], px[1], py[1], px[2], py[2]);
    if (fabsf(area) < 1.0e-8f) return;
    int x0 = (int)floorf(min3f(px[0], px[1], px[2]));
    if (x0 < 0) x0 = 0;
    int x1 = (int)ceilf(max3f(px[0], px[1], px[2]));
    if (x1 > (int)r->width - 1) x1 = (int)r->width - 1;
    int y0 = (int)floorf(min3f(py[0], py[1], py[2]));
    if (y0 < 0) y0 = 0;
    int y1 = (int)ceilf(max3f(py[0], py[1], py[2]));
    if (y1 > (int)r->height - 1) y1 = (int)r->height - 1;
    for (int y = y0; y <= y1; ++y) {
        for (int x = x0; x <= x1; ++x) {
            const float qx = (float)x + 0.5f;
            const float qy = (float)y + 0.5f;
            const float w0 = edgef(px[1], py[1], px[2], py[2], qx, qy);
            const float w1 = edgef(px[2], py[2], px[0], py[0], qx, qy);
            const float w2 = edgef(px[0], py[0], px[1], py[1], qx, qy);
            const int inside = area > 0.0f ? (w0 >= 0.0f && w1 >= 0.0f && w2 >= 0.0f)
                                           : (w0 <= 0.0f && w1 <= 0.0f && w2 <= 0.0f);
            if (!inside) continue;
            const size_t pixel = (size_t)y * r->width + (size_t)x;
            const uint32_t layer = r->counts[pixel]++;
            if (layer >= r->layers) { ++*overflow; continue; }
            const float inv = 1.0f / area;
            fragment f;
            f.depth = (w0 * pd[0] + w1 * pd[1] + w2 * pd[2]) * inv;
            f.side = side;
            r->frags[pixel * r->layers + layer] = f;
        }
    }
}

/* facetrtcore.cpp:1244-1282 */
static int raster_direction(rasterizer *r, orc_direction dir, uint32_t *overflow_out)
{
    memset(r->counts, 0, (size_t)r->width * r->height * sizeof(uint32_t));
    vec3 view;
    if (vnormalized(v3(dir.x, dir.y, dir.z), &view)) return -1;
    const vec3 ref = fabsf(view.v[2]) < 0.9f ? v3(0.0f, 0.0f, 1.0f) : v3(0.0f, 1.0f, 0.0f);
    vec3 right;
    if (vnormalized(vcross(ref, view), &right)) return -1;
    const vec3 up = vcross(view, right);
    uint32_t overflow = 0;
    const orc_raster_config *cfg = r->cfg;
    for (uint32_t t = 0; t <= cfg->periodic_count; ++t) {
        int tx, tz;
        periodic_tile(t, &tx, &tz);
        const float offx = (float)tx * cfg->periodic_size_x;
        const float offz = (float)tz * cfg->periodic_size_z;
        for (uint32_t f = 0; f < r->facets; ++f) {
            float px[3], py[3], pd[3];
            for (uint32_t c = 0; c < 3U; ++c) {
                const orc_vertex *vx = &r->vertices[f * 3U + c];
                const vec3 pos = v3(vx->position[0] + offx, vx->position[1],
                                    vx->position[2] + offz);
                const vec3 rel = vsub(pos, r->center);
                px[c] = (0.5f + 0.5f * vdot(rel, right) / r->radius) * (float)r->width;
                py[c] = (0.5f + 0.5f * vdot(rel, up) / r->radius) * (float)r->height;
                pd[c] = 0.5f - vdot(rel, view) / (2.0f * r->radius);
            }
            const orc_vertex *first = &r->vertices[f * 3U];
            const vec3 n = v3(first->normal[0], first->normal[1], first->normal[2]);
            const uint32_t side = f * 2U + (vdot(n, view) >= 0.0f ? 0U : 1U);
            raster_triangle(r, px, py, pd, side, &overflow);
        }
    }
    *overflow_out = overflow;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* std::sort over fragments by depth, restated step for step from the       */
/* introsort that GCC's libstdc++ ships (median-of-three pivot, unguarded   */
/* partition, heap-sort fallback at depth 2*floor(log2 n), final insertion  */
/* sort with threshold 16), so that equal-depth fragments end in the same   */
/* order as in the reference's buildCpuGraph (facetrtcore.cpp:1371-1372).    */
/* ------------------------------------------------------------------------ */
#define LESS(a, b) ((a).depth < (b).depth)

static void swapf(fragment *a, fragment *b) { fragment t = *a; *a = *b; *b = t; }

static void unguarded_linear_insert(fragment *last)
{
    fragment val = *last;
    fragment *next = last - 1;
    while (LESS(val, *next)) { *last = *next; last = next; --next; }
    *last = val;
}

static void insertion_sort(fragment *first, fragment *last)
{
    if (first == last) return;
    for (fragment *i = first + 1; i != last; ++i) {
        if (LESS(*i, *first)) {
            fragment val = *i;
            memmove(first + 1, first, (size_t)(i - first) * sizeof(fragment));
            *first = val;
        } else {
            unguarded_linear_insert(i);
        }
    }
}

static void adjust_heap(fragment *first, long hole, long len, fragment value)
{
    const long top = hole;
    long child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (LESS(first[child], first[child - 1])) child--;
        first[hole] = first[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        first[hole] = first[child - 1];
        hole = child - 1;
    }
    long parent = (hole - 1) / 2;
    while (hole > top && LESS(first[parent], value)) {
        first[hole] = first[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    first[hole] = value;
}

static void heap_sort(fragment *first, fragment *last)
{
    const long len = last - first;
    if (len >= 2) {
        long parent = (len - 2) / 2;
        for (;;) {
            adjust_heap(first, parent, len, first[parent]);
            if (parent == 0) break;
            parent--;
        }
    }
    while (last - first > 1) {
        --last;
        fragment value = *last;
        *last = *first;
        adjust_heap(first, 0, last - first, value);
    }
}

static void median_to_first(fragment *result, fragment *a, fragment *b, fragment *c)
{
    if (LESS(*a, *b)) {
        if (LESS(*b, *c)) swapf(result, b);
        else if (LESS(*a, *c)) swapf(result, c);
        else swapf(result, a);
    } else if (LESS(*a, *c)) swapf(result, a);
    else if (LESS(*b, *c)) swapf(result, c);
    else swapf(result, b);
}

static fragment *unguarded_partition(fragment *first, fragment *last, fragment *pivot)
{
    for (;;) {
        while (LESS(*first, *pivot)) ++first;
        --last;
        while (LESS(*pivot, *last)) --last;
        if (!(first < last)) return first;
        swapf(first, last);
        ++first;
    }
}

static void introsort_loop(fragment *first, fragment *last, long depth)
{
    while (last - first > 16) {
        if (depth == 0) { heap_sort(first, last); return; }
        --depth;
        fragment *mid = first + (last - first) / 2;
        median_to_first(first, first + 1, mid, last - 1);
        fragment *cut = unguarded_partition(first + 1, last, first);
        introsort_loop(cut, last, depth);
        last = cut;
    }
}

static void std_sort_by_depth(fragment *first, fragment *last)
{
    const long n = last - first;
    if (n <= 0) return;
    long lg = 0;
    while ((1L << (lg + 1)) <= n) ++lg;
    introsort_loop(first, last, 2 * lg);
    if (n > 16) {
        insertion_sort(first, first + 16);
        for (fragment *i = first + 16; i != last; ++i) unguarded_linear_insert(i);
    } else {
        insertion_sort(first, last);
    }
}

/* ------------------------------------------------------------------------ */
/* Edge accumulation: a sorted run of (lo,hi) keys replaces the reference's   */
/* unordered_map (facetrtcore.cpp:1358, :1390); CSR rows sorted by neighbour.*/
/* ------------------------------------------------------------------------ */
typedef struct { uint64_t *keys; size_t n, cap; } keybuf;

static int keybuf_push(keybuf *b, uint64_t k)
{
    if (b->n == b->cap) {
        size_t cap = b->cap ? b->cap * 2 : 1 << 16;
        uint64_t *p = (uint64_t *)realloc(b->keys, cap * sizeof(uint64_t));
        if (!p) return -1;
        b->keys = p;
        b->cap = cap;
    }
    b->keys[b->n++] = k;
    return 0;
}

static int cmp_u64(const void *a, const void *b)
{
    const uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* Build a symmetric CSR from undirected (lo,hi,count) runs (facetrtcore.cpp:1398-1412). */
static int graph_from_keys(keybuf *kb, uint32_t S, orc_graph *g)
{
    qsort(kb->keys, kb->n, sizeof(uint64_t), cmp_u64);
    /* run-length encode to unique undirected edges */
    size_t uniq = 0;
    uint32_t *ucount = (uint32_t *)malloc((kb->n ? kb->n : 1) * sizeof(uint32_t));
    if (!ucount) return -1;
    for (size_t i = 0; i < kb->n;) {
        size_t j = i;
        while (j < kb->n && kb->keys[j] == kb->keys[i]) ++j;
        kb->keys[uniq] = kb->keys[i];
        ucount[uniq] = (uint32_t)(j - i);
        ++uniq;
        i = j;
    }
    /* directed entries sorted by (row, neighbour) */
    uint64_t *dir = (uint64_t *)malloc((2 * uniq + 1) * sizeof(uint64_t));
    uint32_t *dcount = (uint32_t *)malloc((2 * uniq + 1) * sizeof(uint32_t));
    uint64_t *idx = (uint64_t *)malloc((2 * uniq + 1) * sizeof(uint64_t));
    if (!dir || !dcount || !idx) return -1;
    for (size_t e = 0; e < uniq; ++e) {
        const uint64_t lo = kb->keys[e] >> 32, hi = kb->keys[e] & 0xffffffffULL;
        dir[2 * e] = (lo << 32) | hi;
        dir[2 * e + 1] = (hi << 32) | lo;
    }
    /* sort directed keys; counts follow via a (key -> undirected index) map */
    for (size_t e = 0; e < 2 * uniq; ++e) idx[e] = dir[e];
    qsort(idx, 2 * uniq, sizeof(uint64_t), cmp_u64);
    g->surface_count = S;
    g->nnz = 2 * uniq;
    g->row_offsets = (uint32_t *)calloc((size_t)S + 1, sizeof(uint32_t));
    g->neighbors = (uint32_t *)malloc((2 * uniq + 1) * sizeof(uint32_t));
    g->counts = (uint32_t *)malloc((2 * uniq + 1) * sizeof(uint32_t));
    if (!g->row_offsets || !g->neighbors || !g->counts) return -1;
    for (size_t e = 0; e < 2 * uniq; ++e) {
        const uint32_t row = (uint32_t)(idx[e] >> 32), nb = (uint32_t)(idx[e] & 0xffffffffULL);
        g->row_offsets[row + 1]++;
        g->neighbors[e] = nb;
        const uint64_t ukey = row < nb ? (((uint64_t)row << 32) | nb) : (((uint64_t)nb << 32) | row);
        /* binary search the undirected key */
        size_t lo = 0, hi = uniq;
        while (lo < hi) {
            const size_t m = (lo + hi) / 2;
            if (kb->keys[m] < ukey) lo = m + 1; else hi = m;
        }
        g->counts[e] = ucount[lo];
    }
    for (uint32_t s = 0; s < S; ++s) g->row_offsets[s + 1] += g->row_offsets[s];
    free(dir);
    free(dcount);
    free(idx);
    free(ucount);
    return 0;
}

static float closure_error(const orc_graph *g)
{
    float err = 0.0f;
    for (uint32_t s = 0; s < g->surface_count; ++s) {
        uint64_t visible = g->sky_counts[s];
        for (uint32_t e = g->row_offsets[s]; e < g->row_offsets[s + 1]; ++e) visible += g->counts[e];
        if (g->denominators[s] != 0U) {
            const float c = (float)visible / (float)g->denominators[s];
            const float d = fabsf(c - 1.0f);
            if (d > err) err = d;
        }
    }
    return err;
}

/* facetrtcore.cpp:1348-1436 */
int orc_build_graph(const orc_vertex *vertices, uint32_t facet_count,
                    const orc_raster_config *cfg,
                    const orc_direction *directions, uint32_t direction_count,
                    orc_graph *out)
{
    memset(out, 0, sizeof(*out));
    rasterizer r;
    if (raster_init(&r, vertices, facet_count, cfg)) return -2;
    const uint32_t S = facet_count * 2U;
    out->denominators = (uint32_t *)calloc(S, sizeof(uint32_t));
    out->sky_counts = (uint32_t *)calloc(S, sizeof(uint32_t));
    fragment *local = (fragment *)malloc((size_t)r.layers * sizeof(fragment));
    keybuf kb = {0};
    uint32_t overflow_total = 0;
    uint32_t max_depth = 0;
    for (uint32_t d = 0; d < direction_count; ++d) {
        uint32_t overflow = 0;
        if (raster_direction(&r, directions[d], &overflow)) return -3;
        overflow_total += overflow;
        const size_t pixels = (size_t)r.width * r.height;
        for (size_t p = 0; p < pixels; ++p) {
            const uint32_t count = r.counts[p] < r.layers ? r.counts[p] : r.layers;
            if (count == 0U) continue;
            if (r.counts[p] > max_depth) max_depth = r.counts[p];
            memcpy(local, &r.frags[p * r.layers], count * sizeof(fragment));
            std_sort_by_depth(local, local + count);
            for (uint32_t i = 0; i < count; ++i) {
                out->denominators[local[i].side]++;
                out->denominators[local[i].side ^ 1U]++;
            }
            out->sky_counts[local[0].side]++;
            out->sky_counts[local[count - 1].side ^ 1U]++;
            for (uint32_t i = 0; i + 1U < count; ++i) {
                const uint32_t a = local[i].side ^ 1U;
                const uint32_t b = local[i + 1U].side;
                if ((a >> 1U) == (b >> 1U)) continue;
                const uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
                if (keybuf_push(&kb, ((uint64_t)lo << 32) | hi)) return -2;
            }
        }
    }
    free(local);
    raster_free(&r);
    if (graph_from_keys(&kb, S, out)) return -2;
    free(kb.keys);
    out->fragment_overflow = overflow_total;
    out->max_depth = max_depth;
    out->max_closure_error = closure_error(out);
    return overflow_total ? 1 : 0;
}

void orc_free_graph(orc_graph *g)
{
    free(g->row_offsets);
    free(g->neighbors);
    free(g->counts);
    free(g->denominators);
    free(g->sky_counts);
    memset(g, 0, sizeof(*g));
}

/* facetrtcore.cpp:1438-1474 */
int orc_sunlit(const orc_vertex *vertices, uint32_t facet_count,
               const orc_raster_config *cfg, orc_direction sun, float *fraction)
{
    rasterizer r;
    if (raster_init(&r, vertices, facet_count, cfg)) return -2;
    uint32_t overflow = 0;
    if (raster_direction(&r, sun, &overflow)) return -3;
    const uint32_t S = facet_count * 2U;
    uint32_t *total = (uint32_t *)calloc(S, sizeof(uint32_t));
    uint32_t *visible = (uint32_t *)calloc(S, sizeof(uint32_t));
    const size_t pixels = (size_t)r.width * r.height;
    for (size_t p = 0; p < pixels; ++p) {
        const uint32_t count = r.counts[p] < r.layers ? r.counts[p] : r.layers;
        if (count == 0U) continue;
        float nearest = FLT_MAX;
        uint32_t nearest_side = 0U;
        for (uint32_t l = 0; l < count; ++l) {
            const fragment *f = &r.frags[p * r.layers + l];
            total[f->side]++;
            if (f->depth < nearest) { nearest = f->depth; nearest_side = f->side; }
        }
        visible[nearest_side]++;
    }
    for (uint32_t s = 0; s < S; ++s)
        fraction[s] = total[s] ? (float)visible[s] / (float)total[s] : 0.0f;
    free(total);
    free(visible);
    raster_free(&r);
    return overflow ? 1 : 0;
}

/* facetrtcore.cpp:1476-1529: the reference's CPU Jacobi (FP64 gather). */
float orc_solve(const orc_graph *g, const orc_optics *o, float sky,
                uint32_t iterations, float relaxation, float *out)
{
    const uint32_t S = g->surface_count;
    float *cur = (float *)calloc(S, sizeof(float));
    float *nxt = (float *)calloc(S, sizeof(float));
    float max_delta = 0.0f;
    if (iterations < 1U) iterations = 1U;
    if (relaxation < 0.01f) relaxation = 0.01f;
    if (relaxation > 1.0f) relaxation = 1.0f;
    for (uint32_t it = 0; it < iterations; ++it) {
        max_delta = 0.0f;
        for (uint32_t f = 0; f < S / 2U; ++f) {
            float h[2];
            for (uint32_t k = 0; k < 2U; ++k) {
                const uint32_t s = 2U * f + k;
                float inc;
                if (g->denominators[s] == 0U) {
                    inc = sky;
                } else {
                    double value = (double)g->sky_counts[s] * sky;
                    for (uint32_t e = g->row_offsets[s]; e < g->row_offsets[s + 1]; ++e)
                        value += (double)g->counts[e] * cur[g->neighbors[e]];
                    inc = (float)(value / g->denominators[s]);
                }
                h[k] = inc + o[s].direct;
            }
            const uint32_t s0 = 2U * f, s1 = s0 + 1U;
            const float c0 = o[s0].emission + o[s0].reflectance * h[0] + o[s0].transmittance * h[1];
            const float c1 = o[s1].emission + o[s1].reflectance * h[1] + o[s1].transmittance * h[0];
            nxt[s0] = cur[s0] + relaxation * (c0 - cur[s0]);
            nxt[s1] = cur[s1] + relaxation * (c1 - cur[s1]);
            const float d0 = fabsf(nxt[s0] - cur[s0]), d1 = fabsf(nxt[s1] - cur[s1]);
            if (d0 > max_delta) max_delta = d0;
            if (d1 > max_delta) max_delta = d1;
        }
        float *t = cur; cur = nxt; nxt = t;
    }
    memcpy(out, cur, S * sizeof(float));
    free(cur);
    free(nxt);
    return max_delta;
}

/* FP64 restatement of the same sweep (the truth the 1e-4 bar is measured
 * against).  Gauss-free Jacobi in double until max|dB| <= tol * max|B|. */
uint32_t orc_solve_f64(const orc_graph *g, const orc_optics *o, double sky,
                       uint32_t max_iterations, double tol, double *out)
{
    const uint32_t S = g->surface_count;
    double *cur = (double *)calloc(S, sizeof(double));
    double *nxt = (double *)calloc(S, sizeof(double));
    uint32_t it = 0;
    for (; it < max_iterations; ++it) {
        double md = 0.0, mb = 0.0;
        for (uint32_t f = 0; f < S / 2U; ++f) {
            double h[2];
            for (uint32_t k = 0; k < 2U; ++k) {
                const uint32_t s = 2U * f + k;
                double inc;
                if (g->denominators[s] == 0U) {
                    inc = sky;
                } else {
                    double value = (double)g->sky_counts[s] * sky;
                    for (uint32_t e = g->row_offsets[s]; e < g->row_offsets[s + 1]; ++e)
                        value += (double)g->counts[e] * cur[g->neighbors[e]];
                    inc = value / (double)g->denominators[s];
                }
                h[k] = inc + (double)o[s].direct;
            }
            const uint32_t s0 = 2U * f, s1 = s0 + 1U;
            nxt[s0] = (double)o[s0].emission + (double)o[s0].reflectance * h[0] + (double)o[s0].transmittance * h[1];
            nxt[s1] = (double)o[s1].emission + (double)o[s1].reflectance * h[1] + (double)o[s1].transmittance * h[0];
            const double d0 = fabs(nxt[s0] - cur[s0]), d1 = fabs(nxt[s1] - cur[s1]);
            if (d0 > md) md = d0;
            if (d1 > md) md = d1;
            if (fabs(nxt[s0]) > mb) mb = fabs(nxt[s0]);
            if (fabs(nxt[s1]) > mb) mb = fabs(nxt[s1]);
        }
        double *t = cur; cur = nxt; nxt = t;
        if (md <= tol * mb) { ++it; break; }
    }
    memcpy(out, cur, S * sizeof(double));
    free(cur);
    free(nxt);
    return it;
}

/* facetrtcore.cpp:1531-1559 */
void orc_incident(const orc_graph *g, const float *B, const orc_optics *o,
                  float sky, float *out)
{
    for (uint32_t s = 0; s < g->surface_count; ++s) {
        double diffuse = sky;
        if (g->denominators[s] != 0U) {
            diffuse = (double)g->sky_counts[s] * sky;
            for (uint32_t e = g->row_offsets[s]; e < g->row_offsets[s + 1]; ++e)
                diffuse += (double)g->counts[e] * B[g->neighbors[e]];
            diffuse /= g->denominators[s];
        }
        const float v = (float)diffuse + o[s].direct;
        out[s] = v > 0.0f ? v : 0.0f;
    }
}

/* Energy budget of a converged count-form solution, derived from the sweep
 * above (facetrtcore.cpp:1490-1520) with side weight w_s = denom_s:
 *   sum_s w_s D_s + sum_s sky_s L + sum_s w_s e_s
 *     = sum_s w_s (1 - rho_s - tau_{s^1}) H_s + sum_s sky_s B_s
 * (exact when counts are symmetric and each facet's two sides share the
 * same denominator, which the global-line raster guarantees). */
void orc_energy_closure(const orc_graph *g, const orc_optics *o, double sky,
                        const double *B, double *lhs, double *rhs)
{
    double l = 0.0, r = 0.0;
    const uint32_t S = g->surface_count;
    double *H = (double *)malloc(S * sizeof(double));
    for (uint32_t s = 0; s < S; ++s) {
        double inc = sky;
        if (g->denominators[s]) {
            double v = (double)g->sky_counts[s] * sky;
            for (uint32_t e = g->row_offsets[s]; e < g->row_offsets[s + 1]; ++e)
                v += (double)g->counts[e] * B[g->neighbors[e]];
            inc = v / (double)g->denominators[s];
        }
        H[s] = inc + (double)o[s].direct;
    }
    for (uint32_t s = 0; s < S; ++s) {
        const double w = (double)g->denominators[s];
        l += w * (double)o[s].direct + (double)g->sky_counts[s] * sky + w * (double)o[s].emission;
        r += w * (1.0 - (double)o[s].reflectance - (double)o[s ^ 1U].transmittance) * H[s] +
             (double)g->sky_counts[s] * B[s];
    }
    free(H);
    *lhs = l;
    *rhs = r;
}

/* ------------------------------------------------------------------------ */
/* Scene input: facetrtcore.cpp:287-306 (appendTriangle), :362-473          */
/* (loadTreeWithSoil).                                                       */
/* ------------------------------------------------------------------------ */
typedef struct { orc_vertex *v; uint32_t *m; uint32_t n, cap; } tribuf;

static int append_triangle(tribuf *b, vec3 a, vec3 bb, vec3 c, uint32_t material)
{
    const vec3 nv = vcross(vsub(bb, a), vsub(c, a));
    if (vdot(nv, nv) <= 1.0e-16f) return 0;
    vec3 n;
    if (vnormalized(nv, &n)) return -1;
    if (b->n == b->cap) {
        uint32_t cap = b->cap ? b->cap * 2U : 1024U;
        orc_vertex *v = (orc_vertex *)realloc(b->v, (size_t)cap * 3U * sizeof(orc_vertex));
        uint32_t *m = (uint32_t *)realloc(b->m, (size_t)cap * sizeof(uint32_t));
        if (!v || !m) return -1;
        b->v = v;
        b->m = m;
        b->cap = cap;
    }
    const vec3 corners[3] = {a, bb, c};
    for (int k = 0; k < 3; ++k) {
        orc_vertex *vx = &b->v[(size_t)b->n * 3U + (size_t)k];
        for (int i = 0; i < 3; ++i) { vx->position[i] = corners[k].v[i]; vx->normal[i] = n.v[i]; }
    }
    b->m[b->n] = material;
    b->n++;
    return 1;
}

int orc_load_tree_with_soil(const char *path, orc_vertex **vertices,
                            uint32_t **materials, uint32_t *facet_count,
                            uint32_t *leaf_facet_count, float bmin[3], float bmax[3])
{
    FILE *fp = fopen(path, "r");
    if (!fp) return -1;
    size_t np = 0, capp = 1024, nt = 0, capt = 1024;
    vec3 *pos = (vec3 *)malloc(capp * sizeof(vec3));
    int (*tri)[3] = malloc(capt * sizeof(*tri));
    size_t terrain_start = (size_t)-1;
    char line[4096];
    while (fgets(line, sizeof line, fp)) {
        char rec[64] = {0};
        int off = 0;
        if (sscanf(line, "%63s%n", rec, &off) != 1) continue;
        if (strcmp(rec, "o") == 0) {
            char name[256] = {0};
            if (sscanf(line + off, "%255s", name) == 1 &&
                strcmp(name, "STREAMSIM_TERRAIN") == 0 && terrain_start == (size_t)-1)
                terrain_start = nt;
        } else if (strcmp(rec, "v") == 0) {
            char *p = line + off, *end;
            vec3 q;
            for (int i = 0; i < 3; ++i) {
                q.v[i] = strtof(p, &end);
                if (end == p) { fclose(fp); return -2; }
                p = end;
            }
            if (np == capp) { capp *= 2; pos = (vec3 *)realloc(pos, capp * sizeof(vec3)); }
            pos[np++] = q;
        } else if (strcmp(rec, "f") == 0) {
            int face[64], nf = 0;
            char *p = line + off;
            char tok[128];
            int used;
            while (nf < 64 && sscanf(p, "%127s%n", tok, &used) == 1) {
                p += used;
                const long raw = strtol(tok, NULL, 10);
                const long idx = raw > 0 ? raw - 1 : (long)np + raw;
                if (idx < 0 || (size_t)idx >= np) { fclose(fp); return -3; }
                face[nf++] = (int)idx;
            }
            for (int i = 1; i + 1 < nf; ++i) {
                if (nt == capt) { capt *= 2; tri = realloc(tri, capt * sizeof(*tri)); }
                tri[nt][0] = face[0]; tri[nt][1] = face[i]; tri[nt][2] = face[i + 1];
                ++nt;
            }
        }
    }
    fclose(fp);
    if (np == 0 || nt == 0) return -4;
    vec3 mn = v3(FLT_MAX, FLT_MAX, FLT_MAX), mx = v3(-FLT_MAX, -FLT_MAX, -FLT_MAX);
    for (size_t i = 0; i < np; ++i)
        for (int a = 0; a < 3; ++a) {
            if (pos[i].v[a] < mn.v[a]) mn.v[a] = pos[i].v[a];
            if (mx.v[a] < pos[i].v[a]) mx.v[a] = pos[i].v[a];
        }
    for (size_t i = 0; i < np; ++i) pos[i].v[1] -= mn.v[1];
    const int has_terrain = terrain_start != (size_t)-1 && terrain_start < nt;
    tribuf b = {0};
    uint32_t leaf = 0;
    for (size_t t = 0; t < nt; ++t) {
        const uint32_t material = has_terrain && t >= terrain_start ? 1U : 0U;
        const int ok = append_triangle(&b, pos[tri[t][0]], pos[tri[t][1]], pos[tri[t][2]], material);
        if (ok < 0) return -5;
        if (ok && (!has_terrain || t < terrain_start)) ++leaf;
    }
    *leaf_facet_count = has_terrain ? leaf : b.n;
    float x0 = mn.v[0], x1 = mx.v[0], z0 = mn.v[2], z1 = mx.v[2];
    if (!has_terrain) {
        const float wx = mx.v[0] - mn.v[0], wz = mx.v[2] - mn.v[2];
        const float margin = 0.5f * (wx < wz ? wz : wx);
        x0 -= margin; x1 += margin; z0 -= margin; z1 += margin;
        const uint32_t R = 48U;
        for (uint32_t row = 0; row < R; ++row) {
            const float za = z0 + (z1 - z0) * (float)row / (float)R;
            const float zb = z0 + (z1 - z0) * (float)(row + 1U) / (float)R;
            for (uint32_t col = 0; col < R; ++col) {
                const float xa = x0 + (x1 - x0) * (float)col / (float)R;
                const float xb = x0 + (x1 - x0) * (float)(col + 1U) / (float)R;
                if (append_triangle(&b, v3(xa, -0.01f, za), v3(xb, -0.01f, zb), v3(xb, -0.01f, za), 1U) < 0) return -5;
                if (append_triangle(&b, v3(xa, -0.01f, za), v3(xa, -0.01f, zb), v3(xb, -0.01f, zb), 1U) < 0) return -5;
            }
        }
    }
    bmin[0] = x0; bmin[1] = has_terrain ? 0.0f : -0.01f; bmin[2] = z0;
    bmax[0] = x1; bmax[1] = mx.v[1] - mn.v[1]; bmax[2] = z1;
    *vertices = b.v;
    *materials = b.m;
    *facet_count = b.n;
    free(pos);
    free(tri);
    return 0;
}

/* facetrtcore.cpp:500-522 */
void orc_make_optics(const orc_vertex *v, uint32_t F, uint32_t leaf_count,
                     const float *sunlit, orc_direction sun, float beam,
                     float leaf_rho, float leaf_tau, float ground_rho, float ground_tau,
                     orc_optics *o)
{
    const vec3 s = v3(sun.x, sun.y, sun.z);
    for (uint32_t f = 0; f < F; ++f) {
        const int leaf = f < leaf_count;
        const vec3 n = v3(v[f * 3U].normal[0], v[f * 3U].normal[1], v[f * 3U].normal[2]);
        for (uint32_t k = 0; k < 2U; ++k) {
            const uint32_t side = f * 2U + k;
            const vec3 sn = vmul(n, k == 0U ? 1.0f : -1.0f);
            o[side].reflectance = leaf ? leaf_rho : ground_rho;
            o[side].transmittance = leaf ? leaf_tau : ground_tau;
            o[side].emission = 0.0f;
            const float c = vdot(sn, s);
            o[side].direct = sunlit[side] * (c > 0.0f ? c : 0.0f) * beam;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Hemisphere ray-cast view factors (no reference counterpart).  Ray j of   */
/* side s uses sample set (s mod sets): origin a + u*(b-a) + v*(c-a) and    */
/* direction T*dx + Bt*dy + N*dz in the side's local frame.  The device     */
/* kernel evaluates exactly these expressions.  A facet is hit when the     */
/* Moller-Trumbore test accepts the ray at t > 0 and the computed point     */
/* o + t*d lies in the facet's box widened by the hit margin (below); the   */
/* nearest hit = smallest t, ties to the lower facet index; the origin      */
/* facet is skipped.                                                        */
/* ------------------------------------------------------------------------ */
static void side_frame(vec3 N, vec3 *T, vec3 *Bt)
{
    const vec3 helper = fabsf(N.v[1]) < 0.9f ? v3(0.0f, 1.0f, 0.0f) : v3(1.0f, 0.0f, 0.0f);
    vec3 t = vcross(helper, N);
    const float len = sqrtf(vdot(t, t));
    *T = vmul(t, 1.0f / len);
    *Bt = vcross(N, *T);
}

/* Moller-Trumbore; returns t or -1. */
static inline __attribute__((always_inline)) float ray_triangle(vec3 o, vec3 d, vec3 a, vec3 e1, vec3 e2)
{
    const vec3 p = vcross(d, e2);
    const float det = vdot(e1, p);
    if (det == 0.0f) return -1.0f;
    const float inv = 1.0f / det;
    const vec3 t0 = vsub(o, a);
    const float u = vdot(t0, p) * inv;
    if (u < 0.0f || u > 1.0f) return -1.0f;
    const vec3 q = vcross(t0, e1);
    const float v = vdot(d, q) * inv;
    if (v < 0.0f || u + v > 1.0f) return -1.0f;
    const float t = vdot(e2, q) * inv;
    return t > 0.0f ? t : -1.0f;
}

static vec3 vpos(const orc_vertex *v) { return v3(v->position[0], v->position[1], v->position[2]); }

/* The hit margin: 1e-5 of the scene's reach (largest coordinate magnitude,
 * plus two periods when periodic copies are traced) and extent, plus 1e-7.
 * The Moller-Trumbore distance of a long thin facet met at a grazing angle
 * can place o + t*d millimetres outside the facet (measured: 3 mm beyond a
 * 7.9 m x 3 cm trunk facet, 28 m from the origin); such a point is not a
 * hit.  With this rule a bounding volume whose boxes are widened by twice
 * the margin provably never culls a hit (the rounding of o + t*d and of the
 * slab distances is below 1e-7 of the reach), so any such traversal finds
 * exactly the brute force's nearest hit. */
static float hit_margin(const orc_vertex *V, uint32_t F, uint32_t periodic_count,
                        float size_x, float size_z)
{
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t k = 0; k < 3U * F; ++k)
        for (int a = 0; a < 3; ++a) {
            if (V[k].position[a] < lo[a]) lo[a] = V[k].position[a];
            if (V[k].position[a] > hi[a]) hi[a] = V[k].position[a];
        }
    float extent = 0.0f, reach = 0.0f;
    for (int a = 0; a < 3 && F > 0U; ++a) {
        extent = stdmax(extent, hi[a] - lo[a]);
        reach = stdmax(reach, stdmax(fabsf(lo[a]), fabsf(hi[a])));
    }
    if (periodic_count > 0U) reach = reach + 2.0f * stdmax(fabsf(size_x), fabsf(size_z));
    return 1.0e-5f * (reach + extent) + 1.0e-7f;
}

static int in_hit_box(const orc_vertex *V, uint32_t g, vec3 o, vec3 d, float t, float m)
{
    for (int a = 0; a < 3; ++a) {
        const float p = o.v[a] + t * d.v[a];
        const float v0 = V[g * 3U].position[a], v1 = V[g * 3U + 1U].position[a],
                    v2 = V[g * 3U + 2U].position[a];
        const float lo = fminf(v0, fminf(v1, v2)) - m, hi = fmaxf(v0, fmaxf(v1, v2)) + m;
        if (!(p >= lo && p <= hi)) return 0;
    }
    return 1;
}

/* Nearest hit over the scene and its periodic copies (the raster mode's
 * tiles): copy t is met by shifting the origin back by its offset; the hit
 * names the original facet; the origin facet is skipped in tile 0 only;
 * the smallest (t, facet) wins. */
static int closest_hit_tiles(const orc_vertex *V, uint32_t F, uint32_t skip, vec3 o, vec3 d,
                             uint32_t periodic_count, float size_x, float size_z, float m,
                             float *tbest)
{
    int best = -1;
    float bt = FLT_MAX;
    const uint32_t tiles = (periodic_count < 20U ? periodic_count : 20U) + 1U;
    for (uint32_t tile = 0; tile < tiles; ++tile) {
        int tx, tz;
        periodic_tile(tile, &tx, &tz);
        const float ox = (float)tx * size_x, oz = (float)tz * size_z;
        const vec3 ot = v3(o.v[0] - ox, o.v[1], o.v[2] - oz);
        for (uint32_t g = 0; g < F; ++g) {
            if (tile == 0U && g == skip) continue;
            const vec3 a = vpos(&V[g * 3U]);
            const vec3 e1 = vsub(vpos(&V[g * 3U + 1U]), a);
            const vec3 e2 = vsub(vpos(&V[g * 3U + 2U]), a);
            const float t = ray_triangle(ot, d, a, e1, e2);
            if (t > 0.0f && (t < bt || (t == bt && (int)g < best)) && in_hit_box(V, g, ot, d, t, m)) {
                bt = t;
                best = (int)g;
            }
        }
    }
    *tbest = bt;
    return best;
}

static int closest_hit(const orc_vertex *V, uint32_t F, uint32_t skip, vec3 o, vec3 d, float m,
                       float *tbest)
{
    return closest_hit_tiles(V, F, skip, o, d, 0U, 1.0f, 1.0f, m, tbest);
}

static vec3 sample_origin(const orc_vertex *V, uint32_t f, float u, float v)
{
    const vec3 a = vpos(&V[f * 3U]);
    const vec3 e1 = vsub(vpos(&V[f * 3U + 1U]), a);
    const vec3 e2 = vsub(vpos(&V[f * 3U + 2U]), a);
    return vadd(vadd(a, vmul(e1, u)), vmul(e2, v));
}

typedef struct { uint32_t side, count; } hitcount;

static int cmp_hit_side(const void *a, const void *b)
{
    const uint32_t x = ((const hitcount *)a)->side, y = ((const hitcount *)b)->side;
    return x < y ? -1 : (x > y ? 1 : 0);
}
static int cmp_hit_rank(const void *a, const void *b)
{
    const hitcount *x = (const hitcount *)a, *y = (const hitcount *)b;
    if (x->count != y->count) return x->count > y->count ? -1 : 1;
    return x->side < y->side ? -1 : (x->side > y->side ? 1 : 0);
}
static int cmp_u32(const void *a, const void *b)
{
    const uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* One side's row from its ray hits (side ids of the sides seen, sky rays
 * excluded): run counts, the top_k largest counts kept (ties: lower side
 * first), written sorted by side.  Returns the row length; adds the kept
 * ray count to *kept and the dropped ones to *dropped. */
static uint32_t hemi_row(uint32_t *hits, uint32_t nh, hitcount *h, uint32_t top_k,
                         uint32_t *neighbors, uint32_t *counts, uint32_t *kept,
                         uint64_t *dropped)
{
    qsort(hits, nh, sizeof(uint32_t), cmp_u32);
    uint32_t nu = 0;
    for (uint32_t i = 0; i < nh;) {
        uint32_t j = i;
        while (j < nh && hits[j] == hits[i]) ++j;
        h[nu].side = hits[i];
        h[nu].count = j - i;
        ++nu;
        i = j;
    }
    qsort(h, nu, sizeof(hitcount), cmp_hit_rank);
    const uint32_t keep = nu < top_k ? nu : top_k;
    for (uint32_t i = keep; i < nu; ++i) *dropped += h[i].count;
    for (uint32_t i = 0; i < keep; ++i) *kept += h[i].count;
    qsort(h, keep, sizeof(hitcount), cmp_hit_side);
    for (uint32_t i = 0; i < keep; ++i) {
        neighbors[i] = h[i].side;
        counts[i] = h[i].count;
    }
    return keep;
}

int orc_hemisphere_graph(const orc_vertex *V, uint32_t F, const float *uv,
                         const float *dirs, uint32_t rays, uint32_t sets, uint32_t top_k,
                         orc_graph *g, uint64_t *dropped_out)
{
    return orc_hemisphere_graph_periodic(V, F, uv, dirs, rays, sets, top_k, 0U, 1.0f, 1.0f, g,
                                         dropped_out);
}

int orc_hemisphere_graph_periodic(const orc_vertex *V, uint32_t F, const float *uv,
                                  const float *dirs, uint32_t rays, uint32_t sets,
                                  uint32_t top_k, uint32_t periodic_count, float size_x,
                                  float size_z, orc_graph *g, uint64_t *dropped_out)
{
    memset(g, 0, sizeof(*g));
    const uint32_t S = 2U * F;
    g->surface_count = S;
    g->row_offsets = (uint32_t *)calloc((size_t)S + 1, sizeof(uint32_t));
    g->denominators = (uint32_t *)calloc(S, sizeof(uint32_t));
    g->sky_counts = (uint32_t *)calloc(S, sizeof(uint32_t));
    size_t cap = (size_t)S * (top_k < rays ? top_k : rays) + 1;
    g->neighbors = (uint32_t *)malloc(cap * sizeof(uint32_t));
    g->counts = (uint32_t *)malloc(cap * sizeof(uint32_t));
    uint32_t *hits = (uint32_t *)malloc((size_t)rays * sizeof(uint32_t));
    hitcount *h = (hitcount *)malloc((size_t)rays * sizeof(hitcount));
    uint64_t dropped = 0, nnz = 0;
    const float m = hit_margin(V, F, periodic_count, size_x, size_z);
    for (uint32_t s = 0; s < S; ++s) {
        const uint32_t f = s >> 1U;
        const uint32_t set = s % sets;
        vec3 N = v3(V[f * 3U].normal[0], V[f * 3U].normal[1], V[f * 3U].normal[2]);
        if (s & 1U) N = v3(-N.v[0], -N.v[1], -N.v[2]);
        vec3 T, Bt;
        side_frame(N, &T, &Bt);
        uint32_t nh = 0, sky = 0;
        for (uint32_t j = 0; j < rays; ++j) {
            const size_t k = (size_t)set * rays + j;
            const vec3 o = sample_origin(V, f, uv[2 * k], uv[2 * k + 1]);
            const float dx = dirs[3 * k], dy = dirs[3 * k + 1], dz = dirs[3 * k + 2];
            const vec3 d = v3(T.v[0] * dx + Bt.v[0] * dy + N.v[0] * dz,
                              T.v[1] * dx + Bt.v[1] * dy + N.v[1] * dz,
                              T.v[2] * dx + Bt.v[2] * dy + N.v[2] * dz);
            float t;
            const int hit = closest_hit_tiles(V, F, f, o, d, periodic_count, size_x, size_z, m, &t);
            if (hit < 0) { ++sky; continue; }
            const vec3 ng = v3(V[hit * 3U].normal[0], V[hit * 3U].normal[1], V[hit * 3U].normal[2]);
            hits[nh++] = 2U * (uint32_t)hit + (vdot(ng, d) < 0.0f ? 0U : 1U);
        }
        uint32_t kept = 0;
        const uint32_t keep = hemi_row(hits, nh, h, top_k, g->neighbors + nnz, g->counts + nnz,
                                       &kept, &dropped);
        nnz += keep;
        g->row_offsets[s + 1] = (uint32_t)nnz;
        g->sky_counts[s] = sky;
        g->denominators[s] = kept + sky;
    }
    g->nnz = nnz;
    free(hits);
    free(h);
    if (dropped_out) *dropped_out = dropped;
    g->max_closure_error = closure_error(g);
    return 0;
}

int orc_hemisphere_sunlit(const orc_vertex *V, uint32_t F, const float *uv,
                          uint32_t samples, uint32_t sets, orc_direction sun, float *fraction)
{
    return orc_hemisphere_sunlit_periodic(V, F, uv, samples, sets, sun, 0U, 1.0f, 1.0f, fraction);
}

int orc_hemisphere_sunlit_periodic(const orc_vertex *V, uint32_t F, const float *uv,
                                   uint32_t samples, uint32_t sets, orc_direction sun,
                                   uint32_t periodic_count, float size_x, float size_z,
                                   float *fraction)
{
    const vec3 d = v3(sun.x, sun.y, sun.z);
    const float m = hit_margin(V, F, periodic_count, size_x, size_z);
    for (uint32_t s = 0; s < 2U * F; ++s) {
        const uint32_t f = s >> 1U;
        const uint32_t set = s % sets;
        vec3 N = v3(V[f * 3U].normal[0], V[f * 3U].normal[1], V[f * 3U].normal[2]);
        if (s & 1U) N = v3(-N.v[0], -N.v[1], -N.v[2]);
        if (!(vdot(N, d) > 0.0f)) { fraction[s] = 0.0f; continue; }
        uint32_t lit = 0;
        for (uint32_t j = 0; j < samples; ++j) {
            const size_t k = (size_t)set * samples + j;
            const vec3 o = sample_origin(V, f, uv[2 * k], uv[2 * k + 1]);
            float t;
            if (closest_hit_tiles(V, F, f, o, d, periodic_count, size_x, size_z, m, &t) < 0) ++lit;
        }
        fraction[s] = (float)lit / (float)samples;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* The same hemisphere graph and sun visibility with a BVH over the facets   */
/* and host threads, for scenes too large for the brute force (the          */
/* 200k-facet forest: 2 x 10^8 rays).  The rays, the hit rule and the tie   */
/* rules are those above; the BVH only skips facets whose box the ray       */
/* misses.  Boxes are widened by four hit margins, so no hit is skipped:    */
/* the nearest hit (smallest t, then lowest facet) equals the brute         */
/* force's, and so does every row.                                          */
/* ------------------------------------------------------------------------ */
#include <pthread.h>
#include <stdatomic.h>
#include <unistd.h>

typedef struct {
    float lo[3], hi[3];
    int32_t left, right; /* internal: child indices; leaf: left = -1 - first, right = count */
} bvh_node;

typedef struct {
    bvh_node *nodes;
    uint32_t count;
    uint32_t *facet;  /* facet of each leaf slot */
    float *tri;       /* per leaf slot: a, b - a, c - a (9 floats) */
    const orc_vertex *V;
    float m;          /* hit margin */
} bvh_tree;

typedef struct {
    const orc_vertex *V;
    float *box;      /* per facet lo[3], hi[3] (widened) */
    float *centroid; /* per facet */
    uint32_t *idx;
    bvh_node *nodes;
    uint32_t count;
} bvh_build;

static void idx_swap(uint32_t *a, uint32_t i, uint32_t j) { uint32_t t = a[i]; a[i] = a[j]; a[j] = t; }

static float box_area(const float lo[3], const float hi[3])
{
    const float x = hi[0] - lo[0], y = hi[1] - lo[1], z = hi[2] - lo[2];
    return x * y + y * z + z * x;
}

/* Top-down build with the surface-area heuristic over 16 centroid bins per
 * axis; ranges of at most 2 facets are leaves.  A range whose centroids
 * coincide, and every range below depth 64, is halved by index, so the tree
 * is at most 64 + 32 levels deep (kBvhMaxDepth). */
enum { kBvhMaxDepth = 96 };
static int32_t bvh_build_node(bvh_build *b, uint32_t lo, uint32_t hi, uint32_t depth)
{
    enum { kBins = 16, kLeaf = 2 };
    const int32_t me = (int32_t)b->count++;
    bvh_node *n = &b->nodes[me];
    float clo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, chi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int a = 0; a < 3; ++a) { n->lo[a] = FLT_MAX; n->hi[a] = -FLT_MAX; }
    for (uint32_t i = lo; i < hi; ++i) {
        const uint32_t f = b->idx[i];
        for (int a = 0; a < 3; ++a) {
            if (b->box[6 * f + a] < n->lo[a]) n->lo[a] = b->box[6 * f + a];
            if (b->box[6 * f + 3 + a] > n->hi[a]) n->hi[a] = b->box[6 * f + 3 + a];
            if (b->centroid[3 * f + a] < clo[a]) clo[a] = b->centroid[3 * f + a];
            if (b->centroid[3 * f + a] > chi[a]) chi[a] = b->centroid[3 * f + a];
        }
    }
    const uint32_t cnt = hi - lo;
    if (cnt <= kLeaf) {
        n->left = -1 - (int32_t)lo;
        n->right = (int32_t)cnt;
        return me;
    }
    int best_axis = -1;
    int best_split = 0;
    float best_cost = FLT_MAX;
    for (int a = 0; a < 3 && depth < 64U; ++a) {
        const float ext = chi[a] - clo[a];
        if (!(ext > 0.0f)) continue;
        uint32_t bc[kBins] = {0};
        float blo[kBins][3], bhi[kBins][3];
        for (int k = 0; k < kBins; ++k)
            for (int c = 0; c < 3; ++c) { blo[k][c] = FLT_MAX; bhi[k][c] = -FLT_MAX; }
        const float scale = (float)kBins / ext;
        for (uint32_t i = lo; i < hi; ++i) {
            const uint32_t f = b->idx[i];
            int k = (int)((b->centroid[3 * f + a] - clo[a]) * scale);
            if (k >= kBins) k = kBins - 1;
            if (k < 0) k = 0;
            ++bc[k];
            for (int c = 0; c < 3; ++c) {
                if (b->box[6 * f + c] < blo[k][c]) blo[k][c] = b->box[6 * f + c];
                if (b->box[6 * f + 3 + c] > bhi[k][c]) bhi[k][c] = b->box[6 * f + 3 + c];
            }
        }
        /* sweep: cost of splitting after bin k */
        float rarea[kBins];
        uint32_t rcnt[kBins];
        float rl[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rh[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        uint32_t rc = 0;
        for (int k = kBins - 1; k > 0; --k) {
            rc += bc[k];
            for (int c = 0; c < 3; ++c) {
                if (blo[k][c] < rl[c]) rl[c] = blo[k][c];
                if (bhi[k][c] > rh[c]) rh[c] = bhi[k][c];
            }
            rcnt[k] = rc;
            rarea[k] = rc ? box_area(rl, rh) : 0.0f;
        }
        float ll[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, lh[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        uint32_t lc = 0;
        for (int k = 0; k < kBins - 1; ++k) {
            lc += bc[k];
            for (int c = 0; c < 3; ++c) {
                if (blo[k][c] < ll[c]) ll[c] = blo[k][c];
                if (bhi[k][c] > lh[c]) lh[c] = bhi[k][c];
            }
            if (lc == 0 || rcnt[k + 1] == 0) continue;
            const float cost = (float)lc * box_area(ll, lh) + (float)rcnt[k + 1] * rarea[k + 1];
            if (cost < best_cost) { best_cost = cost; best_axis = a; best_split = k; }
        }
    }
    uint32_t mid;
    if (best_axis < 0) {
        mid = lo + cnt / 2U; /* coincident centroids: halve by index */
    } else {
        const int a = best_axis;
        const float scale = (float)kBins / (chi[a] - clo[a]);
        uint32_t i = lo, j = hi;
        while (i < j) {
            const uint32_t f = b->idx[i];
            int k = (int)((b->centroid[3 * f + a] - clo[a]) * scale);
            if (k >= kBins) k = kBins - 1;
            if (k < 0) k = 0;
            if (k <= best_split) ++i; else idx_swap(b->idx, i, --j);
        }
        mid = i;
        if (mid == lo || mid == hi) mid = lo + cnt / 2U;
    }
    const int32_t l = bvh_build_node(b, lo, mid, depth + 1U);
    const int32_t r = bvh_build_node(b, mid, hi, depth + 1U);
    b->nodes[me].left = l;
    b->nodes[me].right = r;
    return me;
}

static int bvh_make(const orc_vertex *V, uint32_t F, float hit_m, bvh_tree *t)
{
    memset(t, 0, sizeof(*t));
    t->V = V;
    t->m = hit_m;
    if (F == 0U) return 0;
    const float margin = 4.0f * hit_m; /* twice what the hit rule needs */
    bvh_build b;
    b.V = V;
    b.box = (float *)malloc((size_t)F * 6 * sizeof(float));
    b.centroid = (float *)malloc((size_t)F * 3 * sizeof(float));
    b.idx = (uint32_t *)malloc((size_t)F * sizeof(uint32_t));
    b.nodes = (bvh_node *)malloc((size_t)2 * F * sizeof(bvh_node));
    b.count = 0;
    if (!b.box || !b.centroid || !b.idx || !b.nodes) {
        free(b.box); free(b.centroid); free(b.idx); free(b.nodes);
        return -1;
    }
    for (uint32_t f = 0; f < F; ++f) {
        for (int a = 0; a < 3; ++a) {
            const float p0 = V[3 * f].position[a], p1 = V[3 * f + 1].position[a],
                        p2 = V[3 * f + 2].position[a];
            const float lo = fminf(p0, fminf(p1, p2)), hi = fmaxf(p0, fmaxf(p1, p2));
            b.box[6 * f + a] = lo - margin;
            b.box[6 * f + 3 + a] = hi + margin;
            b.centroid[3 * f + a] = 0.5f * (lo + hi);
        }
        b.idx[f] = f;
    }
    bvh_build_node(&b, 0, F, 0U);
    t->nodes = b.nodes;
    t->count = b.count;
    t->facet = b.idx;
    t->tri = (float *)malloc((size_t)F * 9 * sizeof(float));
    free(b.box);
    free(b.centroid);
    if (!t->tri) return -1;
    for (uint32_t k = 0; k < F; ++k) {
        const uint32_t g = t->facet[k];
        const vec3 a = vpos(&V[g * 3U]);
        const vec3 e1 = vsub(vpos(&V[g * 3U + 1U]), a);
        const vec3 e2 = vsub(vpos(&V[g * 3U + 2U]), a);
        for (int i = 0; i < 3; ++i) {
            t->tri[9 * k + i] = a.v[i];
            t->tri[9 * k + 3 + i] = e1.v[i];
            t->tri[9 * k + 6 + i] = e2.v[i];
        }
    }
    return 0;
}

static void bvh_free(bvh_tree *t)
{
    free(t->nodes);
    free(t->facet);
    free(t->tri);
    memset(t, 0, sizeof(*t));
}

/* 1/d with |d| raised to at least 1e-30: the slab distances below stay
 * finite (no infinity, no NaN), so plain comparisons order them. */
static float safe_inv(float d)
{
    return 1.0f / (fabsf(d) < 1.0e-30f ? copysignf(1.0e-30f, d) : d);
}

static inline __attribute__((always_inline)) void leaf_test(const bvh_tree *t,
                                                             const bvh_node *n, vec3 o, vec3 d,
                                                             uint32_t skip, float *bt, int *best)
{
    const uint32_t first = (uint32_t)(-1 - n->left);
    for (uint32_t k = first; k < first + (uint32_t)n->right; ++k) {
        const uint32_t g = t->facet[k];
        if (g == skip) continue;
        const float *p = t->tri + 9 * (size_t)k;
        const float th = ray_triangle(o, d, v3(p[0], p[1], p[2]), v3(p[3], p[4], p[5]),
                                      v3(p[6], p[7], p[8]));
        if (th > 0.0f && (th < *bt || (th == *bt && (int)g < *best)) &&
            in_hit_box(t->V, g, o, d, th, t->m)) {
            *bt = th;
            *best = (int)g;
        }
    }
}

static inline __attribute__((always_inline)) int slab_near(const bvh_node *n, vec3 o,
                                                           const float inv[3], float tmax,
                                                           float *tnear)
{
    float tn = 0.0f, tf = FLT_MAX;
    for (int a = 0; a < 3; ++a) {
        const float t0 = (n->lo[a] - o.v[a]) * inv[a], t1 = (n->hi[a] - o.v[a]) * inv[a];
        const float near = t0 < t1 ? t0 : t1, far = t0 < t1 ? t1 : t0;
        tn = near > tn ? near : tn;
        tf = far < tf ? far : tf;
    }
    *tnear = tn;
    return tn <= tf && tn <= tmax;
}

/* Nearest hit (any = 0) or any hit (any = 1) over the tree, improving on
 * (*bt, *best) with the brute force's update rule.  Both children are
 * tested at their parent; the nearer one is entered first and the other
 * stacked, and a stacked node is tested again (against the then nearest
 * hit) when it is taken off the stack. */
static void bvh_trace(const bvh_tree *t, vec3 o, vec3 d, uint32_t skip, int any, float *bt,
                      int *best)
{
    if (t->count == 0U) return;
    const float inv[3] = {safe_inv(d.v[0]), safe_inv(d.v[1]), safe_inv(d.v[2])};
    float tn;
    const bvh_node *n = &t->nodes[0];
    if (!slab_near(n, o, inv, *bt, &tn)) return;
    int32_t stack[kBvhMaxDepth + 2];
    int sp = 0;
    for (;;) {
        if (n->left < 0) {
            leaf_test(t, n, o, d, skip, bt, best);
            if (any && *best >= 0) return;
        } else {
            const bvh_node *l = &t->nodes[n->left], *r = &t->nodes[n->right];
            float tl, tr;
            const int hl = slab_near(l, o, inv, *bt, &tl);
            const int hr = slab_near(r, o, inv, *bt, &tr);
            if (hl && hr) {
                if (tl <= tr) { stack[sp++] = n->right; n = l; }
                else { stack[sp++] = n->left; n = r; }
                continue;
            }
            if (hl) { n = l; continue; }
            if (hr) { n = r; continue; }
        }
        /* next stacked node still in reach */
        for (;;) {
            if (sp == 0) return;
            n = &t->nodes[stack[--sp]];
            if (slab_near(n, o, inv, *bt, &tn)) break;
        }
    }
}

static int bvh_hit_tiles(const bvh_tree *t, uint32_t skip, vec3 o, vec3 d, int any,
                         uint32_t periodic_count, float size_x, float size_z)
{
    int best = -1;
    float bt = FLT_MAX;
    const uint32_t tiles = (periodic_count < 20U ? periodic_count : 20U) + 1U;
    for (uint32_t tile = 0; tile < tiles; ++tile) {
        int tx, tz;
        periodic_tile(tile, &tx, &tz);
        const float ox = (float)tx * size_x, oz = (float)tz * size_z;
        const vec3 ot = v3(o.v[0] - ox, o.v[1], o.v[2] - oz);
        bvh_trace(t, ot, d, tile == 0U ? skip : 0xFFFFFFFFu, any, &bt, &best);
        if (any && best >= 0) break;
    }
    return best;
}

typedef struct {
    const orc_vertex *V;
    const bvh_tree *tree;
    const float *uv, *dirs;
    uint32_t F, rays, sets, top_k, periodic_count;
    float size_x, size_z;
    orc_direction sun;
    float *fraction;           /* sunlit mode */
    uint32_t *row_len, *denom, *sky;
    uint32_t **chunk_nb, **chunk_cnt;
    uint64_t *chunk_dropped;
    atomic_uint next;
    uint32_t chunks;
    int failed;
} hemi_job;

enum { kHemiChunk = 64 };

static void *hemi_graph_worker(void *arg)
{
    hemi_job *j = (hemi_job *)arg;
    const uint32_t S = 2U * j->F;
    const uint32_t cap = j->top_k < j->rays ? j->top_k : j->rays;
    uint32_t *hits = (uint32_t *)malloc((size_t)j->rays * sizeof(uint32_t) + 4);
    hitcount *h = (hitcount *)malloc((size_t)j->rays * sizeof(hitcount) + 8);
    uint32_t *nb = (uint32_t *)malloc((size_t)kHemiChunk * cap * sizeof(uint32_t) + 4);
    uint32_t *cn = (uint32_t *)malloc((size_t)kHemiChunk * cap * sizeof(uint32_t) + 4);
    if (!hits || !h || !nb || !cn) { j->failed = 1; goto done; }
    for (;;) {
        const uint32_t c = atomic_fetch_add(&j->next, 1U);
        if (c >= j->chunks) break;
        const uint32_t s0 = c * kHemiChunk, s1 = s0 + kHemiChunk < S ? s0 + kHemiChunk : S;
        uint64_t used = 0, dropped = 0;
        for (uint32_t s = s0; s < s1; ++s) {
            const uint32_t f = s >> 1U;
            const uint32_t set = s % j->sets;
            const orc_vertex *V = j->V;
            vec3 N = v3(V[f * 3U].normal[0], V[f * 3U].normal[1], V[f * 3U].normal[2]);
            if (s & 1U) N = v3(-N.v[0], -N.v[1], -N.v[2]);
            vec3 T, Bt;
            side_frame(N, &T, &Bt);
            uint32_t nh = 0, skyc = 0;
            for (uint32_t r = 0; r < j->rays; ++r) {
                const size_t k = (size_t)set * j->rays + r;
                const vec3 o = sample_origin(V, f, j->uv[2 * k], j->uv[2 * k + 1]);
                const float dx = j->dirs[3 * k], dy = j->dirs[3 * k + 1], dz = j->dirs[3 * k + 2];
                const vec3 d = v3(T.v[0] * dx + Bt.v[0] * dy + N.v[0] * dz,
                                  T.v[1] * dx + Bt.v[1] * dy + N.v[1] * dz,
                                  T.v[2] * dx + Bt.v[2] * dy + N.v[2] * dz);
                const int hit = bvh_hit_tiles(j->tree, f, o, d, 0, j->periodic_count, j->size_x,
                                              j->size_z);
                if (hit < 0) { ++skyc; continue; }
                const vec3 ng = v3(V[hit * 3U].normal[0], V[hit * 3U].normal[1],
                                   V[hit * 3U].normal[2]);
                hits[nh++] = 2U * (uint32_t)hit + (vdot(ng, d) < 0.0f ? 0U : 1U);
            }
            uint32_t kept = 0;
            const uint32_t keep = hemi_row(hits, nh, h, j->top_k, nb + used, cn + used, &kept,
                                           &dropped);
            used += keep;
            j->row_len[s] = keep;
            j->sky[s] = skyc;
            j->denom[s] = kept + skyc;
        }
        j->chunk_nb[c] = (uint32_t *)malloc(used * sizeof(uint32_t) + 4);
        j->chunk_cnt[c] = (uint32_t *)malloc(used * sizeof(uint32_t) + 4);
        if (!j->chunk_nb[c] || !j->chunk_cnt[c]) { j->failed = 1; break; }
        memcpy(j->chunk_nb[c], nb, used * sizeof(uint32_t));
        memcpy(j->chunk_cnt[c], cn, used * sizeof(uint32_t));
        j->chunk_dropped[c] = dropped;
    }
done:
    free(hits);
    free(h);
    free(nb);
    free(cn);
    return NULL;
}

static void *hemi_sunlit_worker(void *arg)
{
    hemi_job *j = (hemi_job *)arg;
    const uint32_t S = 2U * j->F;
    const vec3 d = v3(j->sun.x, j->sun.y, j->sun.z);
    for (;;) {
        const uint32_t c = atomic_fetch_add(&j->next, 1U);
        if (c >= j->chunks) break;
        const uint32_t s0 = c * kHemiChunk, s1 = s0 + kHemiChunk < S ? s0 + kHemiChunk : S;
        for (uint32_t s = s0; s < s1; ++s) {
            const uint32_t f = s >> 1U;
            const uint32_t set = s % j->sets;
            const orc_vertex *V = j->V;
            vec3 N = v3(V[f * 3U].normal[0], V[f * 3U].normal[1], V[f * 3U].normal[2]);
            if (s & 1U) N = v3(-N.v[0], -N.v[1], -N.v[2]);
            if (!(vdot(N, d) > 0.0f)) { j->fraction[s] = 0.0f; continue; }
            uint32_t lit = 0;
            for (uint32_t r = 0; r < j->rays; ++r) {
                const size_t k = (size_t)set * j->rays + r;
                const vec3 o = sample_origin(V, f, j->uv[2 * k], j->uv[2 * k + 1]);
                if (bvh_hit_tiles(j->tree, f, o, d, 1, j->periodic_count, j->size_x,
                                  j->size_z) < 0)
                    ++lit;
            }
            j->fraction[s] = (float)lit / (float)j->rays;
        }
    }
    return NULL;
}

static int run_workers(hemi_job *j, uint32_t threads, void *(*fn)(void *))
{
    if (threads == 0U) {
        const long n = sysconf(_SC_NPROCESSORS_ONLN);
        threads = n > 0 ? (uint32_t)n : 1U;
    }
    if (threads > 256U) threads = 256U;
    pthread_t tid[256];
    uint32_t started = 0;
    for (uint32_t i = 1; i < threads; ++i)
        if (pthread_create(&tid[started], NULL, fn, j) == 0) ++started;
    fn(j);
    for (uint32_t i = 0; i < started; ++i) pthread_join(tid[i], NULL);
    return j->failed ? -1 : 0;
}

int orc_hemisphere_graph_bvh(const orc_vertex *V, uint32_t F, const float *uv,
                             const float *dirs, uint32_t rays, uint32_t sets, uint32_t top_k,
                             uint32_t periodic_count, float size_x, float size_z,
                             uint32_t threads, orc_graph *g, uint64_t *dropped_out)
{
    memset(g, 0, sizeof(*g));
    const uint32_t S = 2U * F;
    bvh_tree tree;
    if (bvh_make(V, F, hit_margin(V, F, periodic_count, size_x, size_z), &tree) != 0) return -1;
    hemi_job j;
    memset(&j, 0, sizeof(j));
    j.V = V;
    j.tree = &tree;
    j.uv = uv;
    j.dirs = dirs;
    j.F = F;
    j.rays = rays;
    j.sets = sets;
    j.top_k = top_k;
    j.periodic_count = periodic_count;
    j.size_x = size_x;
    j.size_z = size_z;
    j.chunks = (S + kHemiChunk - 1U) / kHemiChunk;
    atomic_init(&j.next, 0U);
    g->surface_count = S;
    g->row_offsets = (uint32_t *)calloc((size_t)S + 1, sizeof(uint32_t));
    g->denominators = (uint32_t *)calloc((size_t)S + 1, sizeof(uint32_t));
    g->sky_counts = (uint32_t *)calloc((size_t)S + 1, sizeof(uint32_t));
    j.row_len = (uint32_t *)calloc((size_t)S + 1, sizeof(uint32_t));
    j.chunk_nb = (uint32_t **)calloc((size_t)j.chunks + 1, sizeof(uint32_t *));
    j.chunk_cnt = (uint32_t **)calloc((size_t)j.chunks + 1, sizeof(uint32_t *));
    j.chunk_dropped = (uint64_t *)calloc((size_t)j.chunks + 1, sizeof(uint64_t));
    j.denom = g->denominators;
    j.sky = g->sky_counts;
    int rc = -1;
    if (g->row_offsets && g->denominators && g->sky_counts && j.row_len && j.chunk_nb &&
        j.chunk_cnt && j.chunk_dropped)
        rc = run_workers(&j, threads, hemi_graph_worker);
    uint64_t nnz = 0, dropped = 0;
    if (rc == 0) {
        for (uint32_t s = 0; s < S; ++s) {
            nnz += j.row_len[s];
            g->row_offsets[s + 1] = (uint32_t)nnz;
        }
        g->neighbors = (uint32_t *)malloc(nnz * sizeof(uint32_t) + 4);
        g->counts = (uint32_t *)malloc(nnz * sizeof(uint32_t) + 4);
        if (!g->neighbors || !g->counts) rc = -1;
    }
    if (rc == 0) {
        for (uint32_t c = 0; c < j.chunks; ++c) {
            const uint32_t s0 = c * kHemiChunk, s1 = s0 + kHemiChunk < S ? s0 + kHemiChunk : S;
            const uint32_t b = g->row_offsets[s0], n = g->row_offsets[s1] - b;
            memcpy(g->neighbors + b, j.chunk_nb[c], (size_t)n * sizeof(uint32_t));
            memcpy(g->counts + b, j.chunk_cnt[c], (size_t)n * sizeof(uint32_t));
            dropped += j.chunk_dropped[c];
        }
        g->nnz = nnz;
        g->max_closure_error = closure_error(g);
        if (dropped_out) *dropped_out = dropped;
    }
    for (uint32_t c = 0; j.chunk_nb && c < j.chunks; ++c) {
        free(j.chunk_nb[c]);
        free(j.chunk_cnt[c]);
    }
    free(j.chunk_nb);
    free(j.chunk_cnt);
    free(j.chunk_dropped);
    free(j.row_len);
    bvh_free(&tree);
    if (rc != 0) orc_free_graph(g);
    return rc;
}

int orc_hemisphere_sunlit_bvh(const orc_vertex *V, uint32_t F, const float *uv,
                              uint32_t samples, uint32_t sets, orc_direction sun,
                              uint32_t periodic_count, float size_x, float size_z,
                              uint32_t threads, float *fraction)
{
    bvh_tree tree;
    if (bvh_make(V, F, hit_margin(V, F, periodic_count, size_x, size_z), &tree) != 0) return -1;
    hemi_job j;
    memset(&j, 0, sizeof(j));
    j.V = V;
    j.tree = &tree;
    j.uv = uv;
    j.F = F;
    j.rays = samples;
    j.sets = sets;
    j.periodic_count = periodic_count;
    j.size_x = size_x;
    j.size_z = size_z;
    j.sun = sun;
    j.fraction = fraction;
    j.chunks = (2U * F + kHemiChunk - 1U) / kHemiChunk;
    atomic_init(&j.next, 0U);
    const int rc = run_workers(&j, threads, hemi_sunlit_worker);
    bvh_free(&tree);
    return rc;
}

/* Per-ray results of chosen sides (diagnostics of a graph difference): for
 * ray j of side sides[i], hit_side[i * rays + j] is the side seen (or
 * 0xFFFFFFFF for sky) and hit_t the distance, by the brute force
 * (use_bvh = 0) or the BVH (use_bvh = 1). */
int orc_hemisphere_rays(const orc_vertex *V, uint32_t F, const float *uv, const float *dirs,
                        uint32_t rays, uint32_t sets, const uint32_t *sides, uint32_t nsides,
                        int use_bvh, uint32_t *hit_side, float *hit_t)
{
    bvh_tree tree;
    memset(&tree, 0, sizeof(tree));
    const float m = hit_margin(V, F, 0U, 1.0f, 1.0f);
    if (use_bvh && bvh_make(V, F, m, &tree) != 0) return -1;
    for (uint32_t i = 0; i < nsides; ++i) {
        const uint32_t s = sides[i], f = s >> 1U, set = s % sets;
        vec3 N = v3(V[f * 3U].normal[0], V[f * 3U].normal[1], V[f * 3U].normal[2]);
        if (s & 1U) N = v3(-N.v[0], -N.v[1], -N.v[2]);
        vec3 T, Bt;
        side_frame(N, &T, &Bt);
        for (uint32_t j = 0; j < rays; ++j) {
            const size_t k = (size_t)set * rays + j;
            const vec3 o = sample_origin(V, f, uv[2 * k], uv[2 * k + 1]);
            const float dx = dirs[3 * k], dy = dirs[3 * k + 1], dz = dirs[3 * k + 2];
            const vec3 d = v3(T.v[0] * dx + Bt.v[0] * dy + N.v[0] * dz,
                              T.v[1] * dx + Bt.v[1] * dy + N.v[1] * dz,
                              T.v[2] * dx + Bt.v[2] * dy + N.v[2] * dz);
            float t = FLT_MAX;
            int hit = -1;
            if (use_bvh) bvh_trace(&tree, o, d, f, 0, &t, &hit);
            else hit = closest_hit(V, F, f, o, d, m, &t);
            if (hit < 0) {
                hit_side[(size_t)i * rays + j] = 0xFFFFFFFFu;
                hit_t[(size_t)i * rays + j] = -1.0f;
                continue;
            }
            const vec3 ng = v3(V[hit * 3U].normal[0], V[hit * 3U].normal[1], V[hit * 3U].normal[2]);
            hit_side[(size_t)i * rays + j] = 2U * (uint32_t)hit + (vdot(ng, d) < 0.0f ? 0U : 1U);
            hit_t[(size_t)i * rays + j] = t;
        }
    }
    bvh_free(&tree);
    return 0;
}
