// euc_kernels.cuh — the GB300 triangle pipeline kernels.
//
// Stages (all scenes of a batch go through each stage in one launch):
//   k_vertex<F>   one thread per unique vertex: the vertex functor
//                 (pipeline.rs:273-276; shading once per vertex instead of once
//                 per index gives the same bits because the functor is pure)
//   k_setup       one thread per primitive: index fetch and bounds check
//                 (index.rs:52-54), flip, perspective divide, winding, cull /
//                 reverse, weight matrix, screen bbox, per-pixel weight deltas,
//                 vertices by y, z-clip class (triangles.rs:55-199)
//   k_prep        per batch: clears the error, statistics, covered-rectangle
//                 and setup-sum entries (done by the first k_vertex launch
//                 when the batch has one)
//   k_scan_plan   exclusive scan of per-primitive row counts, compaction of the
//                 primitives that cover at least one row; one more block
//                 plans the init / resolve chunks of every scene
//   k_init        per pixel: the visibility key of the depth already in place
//   k_raster      one thread per (primitive, row): euc's serial f32 weight
//                 walk along the row span (triangles.rs:219-303), inside test,
//                 z, z-clip and the depth test against a 64-bit visibility
//                 key per pixel, merged with atomicMin
//   k_resolve<F>  per pixel: the winning primitive is shaded once
//                 (get_v_data, fragment, coarse-grid MSAA, blend) and the
//                 colour and depth are written (pipeline.rs:529-578)
//
// Why an arg-min is exact.  With a blend that ignores the old pixel (every
// blend in euc's examples), euc's sequential loop leaves in each pixel the
// fragment of the LAST primitive that passed the depth test.  With a strict
// test (Less / Greater) and depth writes, that is the first primitive (in
// submission order) whose z reaches the extreme value, provided it beats the
// depth already stored; with any other mode the test compares against the
// unchanged initial depth and the last passing primitive wins.  Both are
// min-reductions over a 64-bit key, order-independent, so the per-pixel
// result is bit-identical to euc's loop while rows run in parallel.
#pragma once

#include <cstddef>
#include "euc_device.cuh"

namespace eucg {

constexpr int kBlock = 256;           // threads per block in every kernel
constexpr int kScanPer = 8;           // primitives per thread in the scan
constexpr int kScanBlock = kBlock * kScanPer;

// VertexData floats per vertex in vdata[]: three are padded to four, and more
// than four to a multiple of four, so that a vertex's outputs are whole
// 16-byte loads in the resolve (whose loads, L1 hits mostly, are what limits
// it); one, two and four are stored as they are.
__host__ __device__ constexpr int vd_stride(int nv) { return nv == 3 ? 4 : nv <= 4 ? nv : (nv + 3) & ~3; }

template <class F>
EUC_DEV void load_vd(const float *__restrict__ p, float out[vd_stride(F::NV)]) {
    constexpr int S = vd_stride(F::NV);
    if constexpr (S % 4 == 0) {
#pragma unroll
        for (int i = 0; i < S; i += 4) {
            const float4 q = __ldg(reinterpret_cast<const float4 *>(p + i));
            out[i] = q.x;
            out[i + 1] = q.y;
            out[i + 2] = q.z;
            out[i + 3] = q.w;
        }
    } else if constexpr (S == 2) {  // 8-byte aligned: scene regions are 16-byte aligned
        const float2 q = __ldg(reinterpret_cast<const float2 *>(p));
        out[0] = q.x;
        out[1] = q.y;
    } else {
#pragma unroll
        for (int i = 0; i < S; ++i) out[i] = p[i];
    }
}

template <class F>
EUC_DEV void store_vd(float *__restrict__ p, const float *v) {
    constexpr int S = vd_stride(F::NV);
    if constexpr (S % 4 == 0) {
#pragma unroll
        for (int i = 0; i < S; i += 4)
            *reinterpret_cast<float4 *>(p + i) = make_float4(i < F::NV ? v[i] : 0.0f, i + 1 < F::NV ? v[i + 1] : 0.0f,
                                                             i + 2 < F::NV ? v[i + 2] : 0.0f,
                                                             i + 3 < F::NV ? v[i + 3] : 0.0f);
    } else if constexpr (S == 2) {
        *reinterpret_cast<float2 *>(p) = make_float2(v[0], v[1]);
    } else {
#pragma unroll
        for (int i = 0; i < S; ++i) p[i] = v[i];
    }
}

// KEY_MIN / KEY_LAST: order-independent visibility keys (see above).
// KEY_ORDERED: every candidate fragment is kept in a per-pixel list and the
// lists are replayed in submission order (blends that read the old pixel).
enum KeyType : uint32_t { KEY_NONE = 0, KEY_MIN = 1, KEY_LAST = 2, KEY_ORDERED = 3 };

// One scene of a batch as the kernels see it.
struct SceneDev {
    const uint8_t *verts;
    const uint32_t *idx;      // nullptr: vertices drawn in order
    const void *uniforms;     // device copy of the shader's uniform struct
    uint8_t *pixel;
    uint8_t *depth;
    uint64_t nverts;
    uint64_t nstream;         // stream elements (indices, or vertices)
    uint64_t vtx_base;        // first slot of this scene in clip[]
    uint64_t vd_base;         // first float of this scene in vdata[]
    uint64_t tri_base;        // first primitive record (multiple of kBlock)
    uint64_t pix_base;        // first visibility key (multiple of kBlock)
    euc_vertex_layout lay;
    uint32_t ntris;           // complete primitives (triangles or lines)
    uint32_t ngroups;         // primitive slots whose indices are checked (partial one included)
    uint32_t W, H, gr, level;
    uint32_t ppitch, dpitch, pfmt;
    uint32_t pixel_write, depth_test, depth_write, yflip, zclip, cull, blend, keytype;
    float zmin, zmax;
    uint32_t shader, prim;    // enum euc_shader, enum euc_primitives
    // geometry stage (geom != EUC_GEOM_NONE): k_geometry turns the ntin
    // complete input triangles (ngin groups with the partial one) into
    // gratio output slots each, written non-indexed at gvtx_base / gvd_base;
    // setup and resolve then read those (slot lt: vertices 3 lt .. 3 lt + 2)
    uint64_t gvtx_base, gvd_base;
    uint32_t geom, gratio, ngin, ntin;
    float gparam;
    // strip path (strip_h > 0, strip_rows): the target's rows in strips of
    // strip_h, global strips strip_base .. strip_base + nstrips - 1
    uint32_t strip_h;
    uint32_t strip_base, nstrips;
    // 2 / W and -2 / H, divided once by the host (IEEE, as every setup
    // thread would): the NDC-to-screen matrix of triangles.rs:86-102
    float ndc_x, ndc_y;
};

// Per-primitive record written by k_setup (128 bytes, 16-byte aligned).
// The fields are ordered so that a triangle's raster walk needs the first six
// 16-byte words and its shading words 0-2 and 6 (load_rec).
struct __align__(16) TriRec {
    float o[3];    // w_hom_origin   (triangles.rs:143)
    float dx[3];   // w_hom_dx       (triangles.rs:144)
    float dy[3];   // w_hom_dy       (triangles.rs:145)
    float zc[3];   // clip-space z of the (reordered) vertices (triangles.rs:269)
    uint32_t bx0, bx1, by0, by1;  // bbox clamped to the target (band clamp is per row)
    float vby[6];  // screen vertices ordered by y (triangles.rs:148-171)
    uint32_t scene;
    uint32_t flags;               // bit 0: all vertices pass the z clip; bit 1: every row spans the
                                  // whole bbox; bit 2: every row lies in one band (k_setup)
    uint32_t v[3];                // vertex ids after the winding reversal
    uint32_t pad[5];
};
static_assert(sizeof(TriRec) == 128, "TriRec must stay 128 bytes");
static_assert(offsetof(TriRec, bx0) == 48 && offsetof(TriRec, scene) == 88 && offsetof(TriRec, v) == 96,
              "load_rec reads the record by 16-byte words");

// The 16-byte words of record *p that `words` selects (bit k: word k) as a
// local TriRec, one vector load each instead of a load per field: rows and
// pixels of one primitive share it, so the loads hit L1 and what limits them
// is their count.  Unselected fields are left unset.
EUC_DEV TriRec load_rec(const TriRec *__restrict__ p, uint32_t words) {
    const uint4 *q = reinterpret_cast<const uint4 *>(p);
    uint4 w[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) w[k] = (words >> k) & 1u ? __ldg(q + k) : make_uint4(0u, 0u, 0u, 0u);
    TriRec r;
    r.o[0] = __uint_as_float(w[0].x); r.o[1] = __uint_as_float(w[0].y); r.o[2] = __uint_as_float(w[0].z);
    r.dx[0] = __uint_as_float(w[0].w); r.dx[1] = __uint_as_float(w[1].x); r.dx[2] = __uint_as_float(w[1].y);
    r.dy[0] = __uint_as_float(w[1].z); r.dy[1] = __uint_as_float(w[1].w); r.dy[2] = __uint_as_float(w[2].x);
    r.zc[0] = __uint_as_float(w[2].y); r.zc[1] = __uint_as_float(w[2].z); r.zc[2] = __uint_as_float(w[2].w);
    r.bx0 = w[3].x; r.bx1 = w[3].y; r.by0 = w[3].z; r.by1 = w[3].w;
    r.vby[0] = __uint_as_float(w[4].x); r.vby[1] = __uint_as_float(w[4].y);
    r.vby[2] = __uint_as_float(w[4].z); r.vby[3] = __uint_as_float(w[4].w);
    r.vby[4] = __uint_as_float(w[5].x); r.vby[5] = __uint_as_float(w[5].y);
    r.scene = w[5].z; r.flags = w[5].w;
    r.v[0] = w[6].x; r.v[1] = w[6].y; r.v[2] = w[6].z; r.pad[0] = w[6].w;
    r.pad[1] = w[7].x; r.pad[2] = w[7].y; r.pad[3] = w[7].z; r.pad[4] = w[7].w;
    return r;
}
constexpr uint32_t kRecRaster = 0x3Fu;  // words 0-5: weights, z, bbox, vertices by y, scene, flags
constexpr uint32_t kRecShade = 0x47u;   // words 0-2 and 6: weights, z, vertex ids
constexpr uint32_t kRecAll = 0xFFu;

struct SceneStats {
    unsigned long long culled;
    unsigned long long candidates;
    unsigned long long walked;  // fragments the live triangles may make (their screen areas, each at most its bbox)
    unsigned long long live;    // primitives with at least one row
};

// ---------------------------------------------------------------------------
// Small helpers
// ---------------------------------------------------------------------------
EUC_DEV int find_scene(const uint64_t *base, int n, uint64_t pos) {
    int lo = 0, hi = n;  // largest i with base[i] <= pos
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (base[mid] <= pos) lo = mid; else hi = mid;
    }
    return lo;
}

// Order-preserving map of a non-NaN float onto uint32.
EUC_DEV uint32_t ord_f32(float f) {
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
EUC_DEV float unord_f32(uint32_t o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o);
}

// Visibility key of the depth already stored, for KEY_MIN scenes.  A NaN
// depth fails every comparison, so its key (0) can never be beaten.
EUC_DEV unsigned long long init_key_min(float d0, bool greater) {
    if (isnan(d0)) return 0ull;
    const float c = d0 == 0.0f ? 0.0f : d0;  // -0 and +0 compare equal
    const uint32_t o = greater ? ~ord_f32(c) : ord_f32(c);
    return (unsigned long long)o << 32;
}

template <typename T>
EUC_DEV T warp_incl_scan(T v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T n = __shfl_up_sync(0xFFFFFFFFu, v, d);
        if (lane >= d) v += n;
    }
    return v;
}

template <typename T>
EUC_DEV T warp_sum(T v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, d);
    return v;
}

// Block-wide exclusive scan over kBlock threads; returns the exclusive prefix
// and writes the block total to *total.
template <typename T>
EUC_DEV T block_excl_scan(T v, T *smem /* >= kBlock/32 + 1 */, T *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T inc = warp_incl_scan(v);
    if (lane == 31) smem[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T s = lane < kBlock / 32 ? smem[lane] : T(0);
        T si = warp_incl_scan(s);
        if (lane < kBlock / 32) smem[lane] = si - s;
        if (lane == kBlock / 32 - 1) smem[kBlock / 32] = si;
    }
    __syncthreads();
    T r = smem[warp] + inc - v;
    *total = smem[kBlock / 32];
    __syncthreads();
    return r;
}

// ---------------------------------------------------------------------------
// The per-batch clears before k_setup: each scene's error, statistics and
// covered rectangle, the setup-chunk sums, the strip counts and the strip
// path's counters (totals[6]: entries taken, totals[7]: k_strip's work
// counter).  Entry i of the n = max(scenes, chunks, strips, 2) covers index i
// of each.  The first vertex launch of a batch does them (nothing it reads or
// writes is cleared), which saves a launch; k_prep does them when a batch has
// no vertex launch, and on the no-allocation path.
// ---------------------------------------------------------------------------
struct PrepArgs {
    int *err;
    SceneStats *stats;
    uint4 *cov;
    uint2 *chunk_sums;
    uint32_t *strip_cnt, *strip_fill;
    unsigned long long *totals;
    uint64_t nchunks, n;  // n = 0: nothing to clear
    uint32_t nsc, nstrips;
};

EUC_DEV void prep_clear(const PrepArgs &a, uint64_t i) {
    if (i < a.nsc) {
        a.err[i] = 0;
        a.stats[i] = SceneStats{};
        a.cov[i] = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
    }
    if (i < a.nchunks) a.chunk_sums[i] = make_uint2(0u, 0u);
    if (i < a.nstrips) {
        a.strip_cnt[i] = 0;
        a.strip_fill[i] = 0;
    }
    if (i < 2) a.totals[6 + i] = 0;
}

// ---------------------------------------------------------------------------
// k_vertex
// ---------------------------------------------------------------------------
template <class F>
__global__ void __launch_bounds__(kBlock) k_vertex(const SceneDev *__restrict__ sc, const uint64_t *__restrict__ vtx_base,
                                                   int s_begin, int s_end, uint64_t blk_begin, float4 *__restrict__ clip,
                                                   float *__restrict__ vdata, const PrepArgs prep) {
    for (uint64_t i = (uint64_t)blockIdx.x * kBlock + threadIdx.x; i < prep.n; i += (uint64_t)gridDim.x * kBlock)
        prep_clear(prep, i);
    __shared__ int s_scene;
    const uint64_t pos = (blk_begin + blockIdx.x) * (uint64_t)kBlock;
    if (threadIdx.x == 0) s_scene = s_begin + find_scene(vtx_base + s_begin, s_end - s_begin, pos);
    __syncthreads();
    const SceneDev &s = sc[s_scene];
    const uint64_t v = pos + threadIdx.x - s.vtx_base;
    if (v >= s.nverts) return;
    const typename F::U &u = *reinterpret_cast<const typename F::U *>(s.uniforms);
    float c[4], vd[F::NV];
    F::vertex(u, s.lay, s.verts + v * s.lay.stride, c, vd);
    clip[s.vtx_base + v] = make_float4(c[0], c[1], c[2], c[3]);
    store_vd<F>(vdata + s.vd_base + v * vd_stride(F::NV), vd);
}

// ---------------------------------------------------------------------------
// k_geometry<F>: the built-in geometry stages (enum euc_geometry), one thread
// per input triangle; outputs keep submission order (slot gratio * g + k).
// ---------------------------------------------------------------------------
__host__ __device__ inline uint32_t geometry_ratio(uint32_t g) {
    return g == EUC_GEOM_SUBDIVIDE ? 4u : g == EUC_GEOM_DUPLICATE ? 2u : 1u;
}

// Output k of geometry `g` for the triangle (c, v); false when it emits
// fewer than k + 1 triangles.
template <int NV>
EUC_DEV bool geometry_out(uint32_t g, float param, const float c[3][4], const float v[3][NV], int k, float oc[3][4],
                          float ov[3][NV]) {
    if (g == EUC_GEOM_SUBDIVIDE) {
        // corners a, b, c and midpoints ab, bc, ca as (i, j) pairs: (i, i) is a corner
        const int tri[4][3][2] = {{{0, 0}, {0, 1}, {2, 0}}, {{0, 1}, {1, 1}, {1, 2}},
                                  {{2, 0}, {1, 2}, {2, 2}}, {{0, 1}, {1, 2}, {2, 0}}};
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int p = tri[k][j][0], q = tri[k][j][1];
            if (p == q) {
#pragma unroll
                for (int i = 0; i < 4; ++i) oc[j][i] = c[p][i];
#pragma unroll
                for (int i = 0; i < NV; ++i) ov[j][i] = v[p][i];
            } else {
#pragma unroll
                for (int i = 0; i < 4; ++i) oc[j][i] = c[p][i] * 0.5f + c[q][i] * 0.5f;
#pragma unroll
                for (int i = 0; i < NV; ++i) ov[j][i] = v[p][i] * 0.5f + v[q][i] * 0.5f;
            }
        }
        return true;
    }
    if (g == EUC_GEOM_DISCARD) {
        bool beyond = true;
#pragma unroll
        for (int j = 0; j < 3; ++j) beyond = beyond && (c[j][2] / c[j][3] > param);
        if (beyond) return false;
    }
    if (k > 0 && g != EUC_GEOM_DUPLICATE) return false;
    float m[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) m[i] = ((c[0][i] + c[1][i]) + c[2][i]) / 3.0f;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
#pragma unroll
        for (int i = 0; i < 4; ++i) oc[j][i] = g == EUC_GEOM_SHRINK ? m[i] + (c[j][i] - m[i]) * param : c[j][i];
        if (k == 1) oc[j][0] = c[j][0] + param * c[j][3];
#pragma unroll
        for (int i = 0; i < NV; ++i) ov[j][i] = v[j][i];
    }
    return true;
}

template <class F>
__global__ void __launch_bounds__(kBlock) k_geometry(const SceneDev *__restrict__ sc, const uint64_t *__restrict__ gin_base,
                                                     int s_begin, int s_end, uint64_t blk_begin, float4 *__restrict__ clip,
                                                     float *__restrict__ vdata, uint8_t *__restrict__ galive,
                                                     int *__restrict__ err) {
    __shared__ int s_scene;
    const uint64_t pos = (blk_begin + blockIdx.x) * (uint64_t)kBlock;
    if (threadIdx.x == 0) s_scene = s_begin + find_scene(gin_base + s_begin, s_end - s_begin, pos);
    __syncthreads();
    const int si = s_scene;
    const SceneDev &s = sc[si];
    const uint64_t g = pos + threadIdx.x - gin_base[si];
    if (g >= s.ngin) return;
    bool ok = true;
    uint32_t vid[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const uint64_t e = 3 * g + k;
        if (e < s.nstream) {
            const uint64_t id = s.idx ? (uint64_t)__ldg(s.idx + e) : e;
            if (id >= s.nverts) ok = false;  // index.rs:53
            vid[k] = (uint32_t)id;
        }
    }
    if (!ok) atomicCAS(err + si, 0, EUC_ERR_INDEX_OOB);
    if (g >= s.ntin) return;  // a trailing partial triangle has no output slots
    const uint32_t R = s.gratio;
    uint8_t *alive = galive + s.tri_base + (uint64_t)R * g;
    float c[3][4], v[3][F::NV];
    if (ok) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const float4 q = clip[s.vtx_base + vid[j]];
            c[j][0] = q.x; c[j][1] = q.y; c[j][2] = q.z; c[j][3] = q.w;
            const float *src = vdata + s.vd_base + (uint64_t)vid[j] * vd_stride(F::NV);
#pragma unroll
            for (int i = 0; i < F::NV; ++i) v[j][i] = src[i];
        }
    }
    for (uint32_t k = 0; k < R; ++k) {
        float oc[3][4], ov[3][F::NV];
        const bool live = ok && geometry_out<F::NV>(s.geom, s.gparam, c, v, (int)k, oc, ov);
        alive[k] = live ? 1 : 0;
        if (!live) continue;
        const uint64_t o = 3 * ((uint64_t)R * g + k);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            clip[s.gvtx_base + o + j] = make_float4(oc[j][0], oc[j][1], oc[j][2], oc[j][3]);
            store_vd<F>(vdata + s.gvd_base + (o + j) * vd_stride(F::NV), ov[j]);
        }
    }
}

// ---------------------------------------------------------------------------
// Lines (lines.rs:30-119).  A line record reuses TriRec's storage:
//   o = {screen x0, screen y0, norm}, zc = {euclidean z0, z1},
//   ln = {major start a1, minor start b1, |dmajor|, |dminor|, first step},
//   bx0 / bx1 = the window's minor-axis range (inclusive), by0 = 0,
//   by1 = steps in the window's major range, v = {vertex 0, vertex 1},
//   flags: kLineUseX (frac along x), kLineXMajor, kLineNegMaj, kLineNegMin.
// ---------------------------------------------------------------------------
constexpr uint32_t kLineUseX = 4u, kLineXMajor = 8u, kLineNegMaj = 16u, kLineNegMin = 32u;

// `f as isize` (saturating, NaN -> 0).
EUC_DEV long long as_isize(float v) {
    if (isnan(v)) return 0;
    if (v >= 9.2233720368547758e18f) return 0x7FFFFFFFFFFFFFFFll;
    if (v <= -9.2233720368547758e18f) return (long long)0x8000000000000000ull;
    return (long long)v;
}
// f32::clamp with ordered bounds (a NaN stays NaN).
EUC_DEV float fclamp(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }
// isize subtraction / abs with wrapping (euc builds without overflow checks).
EUC_DEV long long wsub(long long a, long long b) { return (long long)((unsigned long long)a - (unsigned long long)b); }
EUC_DEV long long wabs(long long a) { return a < 0 ? (long long)(0ull - (unsigned long long)a) : a; }

// Setup of line slot lt.  The pixels are clipline's: the Bresenham line
// between the truncated end points, both ends included, inside the window
// (x in [wx1, wx2), y in [wy1, wy2)) -- see the oracle's bresenham_clipped
// for the restatement and why the band clamp of the window does not change
// the pixel set.  Lines with a coordinate beyond 2^30 draw nothing.
EUC_DEV void setup_line(const SceneDev &s, int si, uint64_t lt, uint64_t t, const float4 *__restrict__ clip,
                        TriRec *__restrict__ recs, int *__restrict__ err, uint32_t &nrows, uint32_t &cx0,
                        uint32_t &cy0, uint32_t &cx1, uint32_t &cy1) {
    uint64_t e[2];
    bool ok = true;
    if (s.prim == EUC_PRIM_LINE_LIST) {
        e[0] = 2 * lt;
        e[1] = 2 * lt + 1;
    } else {
        const uint64_t j = lt / 3, k = lt % 3;
        e[0] = 3 * j + k;
        e[1] = 3 * j + (k + 1) % 3;
        if (k == 0)  // the first edge checks the whole group of three
            for (uint64_t q = 3 * j; q < 3 * j + 3 && q < s.nstream; ++q) {
                const uint64_t id = s.idx ? (uint64_t)__ldg(s.idx + q) : q;
                if (id >= s.nverts) ok = false;  // index.rs:53
            }
    }
    uint32_t vid[2] = {0, 0};
    bool mine = true;  // both end indices valid, so their clip positions may be read
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (e[k] < s.nstream) {
            const uint64_t id = s.idx ? (uint64_t)__ldg(s.idx + e[k]) : e[k];
            if (id >= s.nverts) {
                ok = false;
                mine = false;
            }
            vid[k] = (uint32_t)id;
        } else {
            mine = false;
        }
    }
    if (!ok) atomicCAS(err + si, 0, EUC_ERR_INDEX_OOB);
    if (!ok || !mine || lt >= s.ntris) return;
    const float flip1 = s.yflip ? -1.0f : 1.0f;
    const float size_x = (float)s.W, size_y = (float)s.H;
    float ez[2], sx[2], sy[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float4 c = clip[s.vtx_base + vid[k]];
        const float w = rmax(c.w, 0.0001f);  // lines.rs:45-48
        const float ex = (c.x * 1.0f) / w, ey = (c.y * flip1) / w;
        ez[k] = c.z / w;
        sx[k] = size_x * (ex * 0.5f + 0.5f);  // lines.rs:53-55
        sy[k] = size_y * (ey * -0.5f + 0.5f);
    }
    const long long x1 = as_isize(sx[0]), y1 = as_isize(sy[0]), x2 = as_isize(sx[1]), y2 = as_isize(sy[1]);
    const long long wx1 = as_isize(fclamp(rmin(sx[0], sx[1]) + 0.0f, 0.0f, size_x));
    const long long wy1 = as_isize(fclamp(rmin(sy[0], sy[1]) + 0.0f, 0.0f, size_y));
    const long long wx2 = as_isize(fclamp(rmax(sx[0], sx[1]) + 1.0f, 0.0f, size_x));
    const long long wy2 = as_isize(fclamp(rmax(sy[0], sy[1]) + 1.0f, 0.0f, size_y));
    const bool use_x = wabs(wsub(x1, x2)) > wabs(wsub(y1, y2));  // lines.rs:73
    const float norm = 1.0f / (use_x ? sx[1] - sx[0] : sy[1] - sy[0]);
    const long long lim = 1ll << 30;
    if (wx2 <= wx1 || wy2 <= wy1) return;  // empty window
    if (x1 <= -lim || x1 >= lim || x2 <= -lim || x2 >= lim || y1 <= -lim || y1 >= lim || y2 <= -lim || y2 >= lim)
        return;
    const long long dx = x2 - x1, dy = y2 - y1;
    const bool xmaj = (dx < 0 ? -dx : dx) >= (dy < 0 ? -dy : dy);
    const long long a1 = xmaj ? x1 : y1, b1 = xmaj ? y1 : x1;
    const long long dmaj = xmaj ? dx : dy, dmin = xmaj ? dy : dx;
    const long long amaj = dmaj < 0 ? -dmaj : dmaj, amin = dmin < 0 ? -dmin : dmin;
    const long long wa1 = xmaj ? wx1 : wy1, wa2 = (xmaj ? wx2 : wy2) - 1;
    const long long wb1 = xmaj ? wy1 : wx1, wb2 = (xmaj ? wy2 : wx2) - 1;
    long long i_lo, i_hi;
    if (dmaj >= 0) {
        i_lo = wa1 - a1;
        i_hi = wa2 - a1;
    } else {
        i_lo = a1 - wa2;
        i_hi = a1 - wa1;
    }
    if (i_lo < 0) i_lo = 0;
    if (i_hi > amaj) i_hi = amaj;
    if (i_hi < i_lo) return;
    TriRec r;
    r.o[0] = sx[0];
    r.o[1] = sy[0];
    r.o[2] = norm;
    r.zc[0] = ez[0];
    r.zc[1] = ez[1];
    r.zc[2] = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) r.dx[k] = r.dy[k] = 0.0f;
#pragma unroll
    for (int k = 0; k < 6; ++k) r.vby[k] = 0.0f;
    r.pad[0] = (uint32_t)(int32_t)a1;
    r.pad[1] = (uint32_t)(int32_t)b1;
    r.pad[2] = (uint32_t)amaj;
    r.pad[3] = (uint32_t)amin;
    r.pad[4] = (uint32_t)i_lo;
    r.bx0 = (uint32_t)wb1;
    r.bx1 = (uint32_t)wb2;
    r.by0 = 0;
    r.by1 = (uint32_t)(i_hi - i_lo + 1);
    r.v[0] = vid[0];
    r.v[1] = vid[1];
    r.v[2] = vid[1];
    r.scene = (uint32_t)si;
    r.flags = (use_x ? kLineUseX : 0u) | (xmaj ? kLineXMajor : 0u) | (dmaj < 0 ? kLineNegMaj : 0u) |
              (dmin < 0 ? kLineNegMin : 0u);
    const float4 *src = reinterpret_cast<const float4 *>(&r);
    float4 *dst = reinterpret_cast<float4 *>(recs + t);
#pragma unroll
    for (int k = 0; k < 8; ++k) dst[k] = src[k];
    nrows = r.by1;
    cx0 = (uint32_t)wx1;
    cx1 = (uint32_t)wx2;
    cy0 = (uint32_t)wy1;
    cy1 = (uint32_t)wy2;
}

// Primitives whose full-row bbox holds at most this many pixels are walked
// once in k_setup; when none of those pixels is inside, they get no rows.
constexpr uint32_t kTinyPixels = 4;

// ---------------------------------------------------------------------------
// The strip path.  A target's rows are cut into strips of strip_h rows that
// span its whole width, so that no row walk is ever split (a row's weights
// come from euc's serial additions from its start).  k_strip keeps a strip's
// visibility keys in shared memory, where a reduction costs little, and
// walks the strip's (primitive, row) items there.  That pays where many
// fragments land on each pixel, and each strip entry brings enough of them,
// so k_bin_count sends a scene's primitives to the strips when its
// triangles' screen areas add up to kStripOverdraw times its covered
// rectangle and to kStripTriFrags per triangle or more (or always, when
// forced), while the entry list has room; kRowsBinned marks them in rows[].  A strip is worked in
// units of at most kStripUnit entries, one block each: the unit reduces its
// fragments in shared memory, then merges every key it lowered into the keys
// k_init seeded with one 64-bit min per pixel.  The other primitives, and the
// scenes the path does not take (lines, ordered blends, targets too wide for
// a strip), go through k_raster's item queue after the strips.  Which way a
// primitive goes changes no result: the keys are order-free reductions.
// ---------------------------------------------------------------------------
constexpr int kStripThreads = 512;            // threads of a k_strip block
constexpr int kStripBlocksPerSm = 2;          // k_strip blocks resident per SM (its grid)
constexpr uint32_t kStripMaxRows = 16;        // rows of a strip at most
constexpr size_t kStripKeyBytes = 96 * 1024;  // a strip's keys in shared memory at most
constexpr uint32_t kRowsBinned = 0x80000000u; // rows[t]: the primitive went to the strips
constexpr uint32_t kStripUnit = 1024;         // entries of one strip a k_strip block takes at once at most
constexpr uint32_t kStripClaim = 32;          // items a k_strip warp claims at a time
constexpr uint64_t kStripOverdraw = 4;        // fragments per covered pixel that route a scene to the strips ...
constexpr uint64_t kStripTriFrags = 16;       // ... when its triangles make this many fragments each on average
constexpr uint64_t kStripMinPixels = 64;      // target pixels per primitive above which a scene stays off them
constexpr uint32_t kBinHist = 1024;           // strips of a scene the binning kernels count in shared memory

// Keys per row of a strip w pixels wide in shared memory: an odd count, so
// that the same column of different rows falls in different banks.
__host__ __device__ inline uint32_t strip_pitch(uint32_t w) { return w | 1u; }

// Rows per strip for a W x H target; 0 when the strip path cannot take it.
__host__ __device__ inline uint32_t strip_rows(uint32_t W, uint32_t H) {
    if (W == 0 || H == 0 || H >= (1u << 24) || 8ull * strip_pitch(W) > kStripKeyBytes) return 0;
    const uint64_t r = kStripKeyBytes / (8ull * strip_pitch(W));
    return (uint32_t)(r < kStripMaxRows ? r : kStripMaxRows);
}

// Width bucket of a k_strip entry (the span w of its middle row in the
// strip): exact below 32, then 16 pixels wide; entries are walked bucket by
// bucket, widest first.
constexpr uint32_t kWidthBuckets = 64;
__host__ __device__ inline uint32_t width_bucket(uint32_t w) {
    return w < 32u ? w : (32u + ((w - 32u) >> 4) < kWidthBuckets - 1 ? 32u + ((w - 32u) >> 4) : kWidthBuckets - 1);
}

// ---------------------------------------------------------------------------
// k_setup: triangles.rs:55-199, once per primitive (euc repeats it per band;
// only the bbox clamp depends on the band and that is applied per row).
// Block b sets up primitives [b * kBlock, (b + 1) * kBlock), all of scene
// chunk_scene[b] (null: scene 0); chunk_sums must be zero at launch.  bbox
// (null when the batch has no strips) receives the bbox of every triangle
// with rows: the binning reads those 16 bytes instead of the record's line.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_setup(const SceneDev *__restrict__ sc,
                                                  const uint32_t *__restrict__ chunk_scene,
                                                  const float4 *__restrict__ clip, TriRec *__restrict__ recs,
                                                  uint32_t *__restrict__ rows, uint2 *__restrict__ chunk_sums,
                                                  int *__restrict__ err, SceneStats *__restrict__ stats,
                                                  uint4 *__restrict__ cov, const uint8_t *__restrict__ galive,
                                                  uint4 *__restrict__ bbox) {
    // a warp's 32 records, staged so that they leave as 512-byte stores;
    // 16-byte word k of lane l's record sits at l * 8 + (k ^ (l & 7)), which
    // keeps both the staging and the copy-out at the minimum four wavefronts
    __shared__ uint4 s_rec[kBlock / 32][32 * 8];
    const int lane = threadIdx.x & 31;
    uint4 *stage = s_rec[threadIdx.x >> 5];
    bool staged = false;
    const uint64_t t = (uint64_t)blockIdx.x * kBlock + threadIdx.x;
    const int si = chunk_scene ? (int)chunk_scene[blockIdx.x] : 0;
    const SceneDev &s = sc[si];
    const uint64_t lt = t - s.tri_base;
    uint32_t nrows = 0, culled = 0;
    float frag_est = 0.0f;  // the primitive's screen area in pixels, at most its bbox (the strip routing)
    // pixels this primitive may touch: x in [cx0, cx1), y in [cy0, cy1)
    uint32_t cx0 = 0xFFFFFFFFu, cy0 = 0xFFFFFFFFu, cx1 = 0, cy1 = 0;
    if (s.prim != EUC_PRIM_TRIANGLE_LIST) {  // uniform: a block holds one scene
        if (lt < s.ngroups) setup_line(s, si, lt, t, clip, recs, err, nrows, cx0, cy0, cx1, cy1);
    } else if (lt < s.ngroups) {
        uint32_t vid[3] = {0, 0, 0};
        bool ok = true;
        if (s.geom) {  // the geometry stage's output slot: checked and written by k_geometry
            ok = galive[t] != 0;
#pragma unroll
            for (int k = 0; k < 3; ++k) vid[k] = (uint32_t)(3 * lt + k);
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const uint64_t e = 3 * lt + k;
                if (e < s.nstream) {
                    const uint64_t id = s.idx ? (uint64_t)__ldg(s.idx + e) : e;
                    if (id >= s.nverts) ok = false;  // index.rs:53 panics on this
                    vid[k] = (uint32_t)id;
                }
            }
            if (!ok) atomicCAS(err + si, 0, EUC_ERR_INDEX_OOB);
        }
        const uint64_t cbase = s.geom ? s.gvtx_base : s.vtx_base;
        if (ok && lt < s.ntris) {
            float h[3][4], e3[3][3];
            const float flip1 = s.yflip ? -1.0f : 1.0f;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float4 c = clip[cbase + vid[k]];
                h[k][0] = c.x * 1.0f;
                h[k][1] = c.y * flip1;
                h[k][2] = c.z;
                h[k][3] = c.w;
                e3[k][0] = h[k][0] / h[k][3];
                e3[k][1] = h[k][1] / h[k][3];
                e3[k][2] = h[k][2] / h[k][3];
            }
            // winding = cross(e1 - e0, e2 - e0).z   (triangles.rs:67-70)
            const float ax = e3[1][0] - e3[0][0], ay = e3[1][1] - e3[0][1];
            const float bx = e3[2][0] - e3[0][0], by = e3[2][1] - e3[0][1];
            const float winding = ax * by - ay * bx;
            bool cull = false;
            if (s.cull != EUC_CULL_NONE) {
                const float dir = s.cull == EUC_CULL_BACK ? 1.0f : -1.0f;
                cull = winding * dir < 0.0f;
            }
            if (cull) {
                culled = 1;
            } else {
                if (winding >= 0.0f) {  // reverse vertex order (triangles.rs:78-80)
#pragma unroll
                    for (int k = 0; k < 4; ++k) { float tmp = h[0][k]; h[0][k] = h[2][k]; h[2][k] = tmp; }
#pragma unroll
                    for (int k = 0; k < 3; ++k) { float tmp = e3[0][k]; e3[0][k] = e3[2][k]; e3[2][k] = tmp; }
                    uint32_t tv = vid[0]; vid[0] = vid[2]; vid[2] = tv;
                }
                const float size_x = (float)s.W, size_y = (float)s.H;
                const float nd[3][3] = {{s.ndc_x, 0.0f, -1.0f}, {0.0f, s.ndc_y, 1.0f}, {0.0f, 0.0f, 1.0f}};
                // coords_to_weights (triangles.rs:86-102)
                const float A[3] = {h[0][0], h[0][1], h[0][3]};
                const float B[3] = {h[1][0], h[1][1], h[1][3]};
                const float Cc[3] = {h[2][0], h[2][1], h[2][3]};
                const float ca[3] = {A[0] - Cc[0], A[1] - Cc[1], A[2] - Cc[2]};
                const float cb[3] = {B[0] - Cc[0], B[1] - Cc[1], B[2] - Cc[2]};
                const float n[3] = {ca[1] * cb[2] - ca[2] * cb[1], ca[2] * cb[0] - ca[0] * cb[2],
                                    ca[0] * cb[1] - ca[1] * cb[0]};
                const float m2 = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
                const float rec_det =
                    m2 > 0.0f ? 1.0f / rmin(n[0] * Cc[0] + n[1] * Cc[1] + n[2] * Cc[2], -1.1920928955078125e-07f) : 1.0f;
                float R[3][3] = {{cb[1] * Cc[2] - cb[2] * Cc[1], cb[2] * Cc[0] - cb[0] * Cc[2], cb[0] * Cc[1] - cb[1] * Cc[0]},
                                 {Cc[1] * ca[2] - Cc[2] * ca[1], Cc[2] * ca[0] - Cc[0] * ca[2], Cc[0] * ca[1] - Cc[1] * ca[0]},
                                 {n[0], n[1], n[2]}};
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j) R[i][j] = R[i][j] * rec_det;
                float M[3][3];
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j) M[i][j] = R[i][0] * nd[0][j] + R[i][1] * nd[1][j] + R[i][2] * nd[2][j];
                // screen coordinates and bbox (triangles.rs:110-139)
                float scr[3][2];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    scr[k][0] = size_x * (e3[k][0] * 0.5f + 0.5f);
                    scr[k][1] = size_y * (e3[k][1] * -0.5f + 0.5f);
                }
                const float mnx = rmin(rmin(scr[0][0], scr[1][0]), scr[2][0]);
                const float mny = rmin(rmin(scr[0][1], scr[1][1]), scr[2][1]);
                const float mxx = rmax(rmax(scr[0][0], scr[1][0]), scr[2][0]);
                const float mxy = rmax(rmax(scr[0][1], scr[1][1]), scr[2][1]);
                const uint32_t bx0 = min(sat_u32(mnx + 0.0f), s.W), bx1 = min(sat_u32(mxx + 1.0f), s.W);
                const uint32_t by0 = min(sat_u32(mny + 0.0f), s.H), by1 = min(sat_u32(mxy + 1.0f), s.H);
                // weights at the origin and per pixel (triangles.rs:142-145)
                float o[3], dxw[3], dyw[3];
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    o[i] = M[i][0] * 0.0f + M[i][1] * 0.0f + M[i][2] * 1.0f;
                    const float wx = M[i][0] * 1000.0f + M[i][1] * 0.0f + M[i][2] * 1.0f;
                    const float wy = M[i][0] * 0.0f + M[i][1] * 1000.0f + M[i][2] * 1.0f;
                    dxw[i] = (wx - o[i]) * (1.0f / 1000.0f);
                    dyw[i] = (wy - o[i]) * (1.0f / 1000.0f);
                }
                // vertices by height (triangles.rs:148-171)
                // (selects, not an index table: the vertices stay in registers)
                int oy[3];
                if (scr[0][1] == mny) {
                    oy[0] = 0; oy[1] = scr[1][1] < scr[2][1] ? 1 : 2; oy[2] = 3 - oy[1];
                } else if (scr[1][1] == mny) {
                    oy[0] = 1; oy[1] = scr[0][1] < scr[2][1] ? 0 : 2; oy[2] = 2 - oy[1];
                } else {
                    oy[0] = 2; oy[1] = scr[0][1] < scr[1][1] ? 0 : 1; oy[2] = 1 - oy[1];
                }
                // z-clip class (triangles.rs:173)
                bool noclip = true;
                if (s.zclip) {
#pragma unroll
                    for (int k = 0; k < 3; ++k) noclip = noclip && (s.zmin <= e3[k][2] && e3[k][2] <= s.zmax);
                }
                TriRec r;
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    r.o[i] = o[i];
                    r.dx[i] = dxw[i];
                    r.dy[i] = dyw[i];
                    r.zc[i] = h[i][2];
                }
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    r.vby[2 * k] = oy[k] == 0 ? scr[0][0] : oy[k] == 1 ? scr[1][0] : scr[2][0];
                    r.vby[2 * k + 1] = oy[k] == 0 ? scr[0][1] : oy[k] == 1 ? scr[1][1] : scr[2][1];
                }
                r.bx0 = bx0; r.bx1 = bx1; r.by0 = by0; r.by1 = by1;
                r.v[0] = vid[0]; r.v[1] = vid[1]; r.v[2] = vid[2];
                r.scene = (uint32_t)si;
                // bit 1: every row lies in one render_par band and the bbox
                // extent is below 128, so every row spans the whole bbox
                // (triangles.rs:224-226) and k_raster skips the band and edge
                // arithmetic
                // bit 2: every row lies in one band (the band clamp is the
                // bbox itself), so bit 1 alone decides the row kind
                const bool one_band = by1 > by0 && by0 / s.gr == (by1 - 1) / s.gr;
                const bool full_rows = one_band && (unsigned long long)(bx1 - bx0) * (by1 - by0) < 128ull;
                r.flags = (noclip ? 1u : 0u) | (full_rows ? 2u : 0u) | (one_band ? 4u : 0u);
#pragma unroll
                for (int k = 0; k < 5; ++k) r.pad[k] = 0;
                nrows = bx1 > bx0 ? by1 - by0 : 0u;
                // NDC area |winding| / 2 is (W / 2) x (H / 2) pixels per unit
                frag_est = fminf(fabsf(winding) * (size_x * size_y * 0.125f), (float)(bx1 - bx0) * (float)(by1 - by0));
                if (full_rows && (bx1 - bx0) * (by1 - by0) <= kTinyPixels) {
                    // a tiny primitive: walk its few pixels here exactly as
                    // k_raster would (full-bbox rows, triangles.rs:257-301);
                    // one that covers none of them needs no raster work
                    bool any = false;
                    for (uint32_t y = by0; y < by1 && !any; ++y) {
                        const float yf = (float)y, xsf = (float)bx0;
                        float w0 = (o[0] + dyw[0] * yf) + dxw[0] * xsf;
                        float w1 = (o[1] + dyw[1] * yf) + dxw[1] * xsf;
                        float w2 = (o[2] + dyw[2] * yf) + dxw[2] * xsf;
                        for (uint32_t x = bx0; x < bx1; ++x) {
                            const float wu2 = (w2 - w0) - w1;
                            any = any || (w0 >= 0.0f && w1 >= 0.0f && wu2 >= 0.0f);
                            w0 = w0 + dxw[0];
                            w1 = w1 + dxw[1];
                            w2 = w2 + dxw[2];
                        }
                    }
                    if (!any) nrows = 0;
                }
                if (nrows) {
                    // only a primitive with rows is ever read again (the scan
                    // keeps exactly those)
                    const uint4 *src = reinterpret_cast<const uint4 *>(&r);
#pragma unroll
                    for (int k = 0; k < 8; ++k) stage[lane * 8 + (k ^ (lane & 7))] = src[k];
                    staged = true;
                    if (bbox) bbox[t] = make_uint4(bx0, bx1, by0, by1);  // the binning's copy
                    cx0 = bx0;
                    cx1 = bx1;
                    cy0 = by0;
                    cy1 = by1;
                }
            }
        }
    }
    {  // the warp's staged records, 16-byte word c of the warp's 4 KB per lane and pass
        const uint32_t live = __ballot_sync(0xFFFFFFFFu, staged);
        __syncwarp();
        if (live) {
            uint4 *dst = reinterpret_cast<uint4 *>(recs + (t - (uint64_t)lane));
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int c = k * 32 + lane, owner = c >> 3;
                if ((live >> owner) & 1u) dst[c] = stage[owner * 8 + ((c & 7) ^ (owner & 7))];
            }
        }
    }
    rows[t] = nrows;
    // the scene's covered rectangle: min of (x0, y0, ~x1, ~y1) over its primitives
    {
        const uint32_t m0 = __reduce_min_sync(0xFFFFFFFFu, cx0), m1 = __reduce_min_sync(0xFFFFFFFFu, cy0);
        const uint32_t m2 = __reduce_min_sync(0xFFFFFFFFu, ~cx1), m3 = __reduce_min_sync(0xFFFFFFFFu, ~cy1);
        if ((threadIdx.x & 31) == 0 && m0 != 0xFFFFFFFFu) {
            atomicMin(&cov[si].x, m0);
            atomicMin(&cov[si].y, m1);
            atomicMin(&cov[si].z, m2);
            atomicMin(&cov[si].w, m3);
        }
    }
    // per-block sums for the scan (zeroed before the launch; each warp adds
    // its own, no block barrier), the culled count of this scene, and the
    // pixels its rows may walk (the strip path's routing)
    const uint32_t live = nrows ? 1u : 0u;
    uint32_t wl = warp_sum(live), wr = warp_sum(nrows), wc = warp_sum(culled);
    const unsigned long long ww = warp_sum(nrows ? (unsigned long long)frag_est : 0ull);
    if ((threadIdx.x & 31) == 0) {
        if (wl) atomicAdd(&chunk_sums[blockIdx.x].x, wl);
        if (wr) atomicAdd(&chunk_sums[blockIdx.x].y, wr);
        if (wc) atomicAdd(&stats[si].culled, (unsigned long long)wc);
        if (ww) atomicAdd(&stats[si].walked, ww);
        if (wl) atomicAdd(&stats[si].live, (unsigned long long)wl);
    }
}

// ---------------------------------------------------------------------------
// scan_block (in k_scan_plan): stable compaction of the primitives that
// cover at least one row (submission order kept) and the exclusive scan of
// their row counts.  Block b covers primitives [b*kScanBlock,
// (b+1)*kScanBlock), i.e. the setup chunks [b*kScanPer, (b+1)*kScanPer).
// totals[0] = live primitives, totals[1] = rows, totals[2] = k_raster's work
// counter (reset here, so that no separate memset is needed).
// ---------------------------------------------------------------------------
EUC_DEV void scan_block(const uint32_t *__restrict__ rows, const uint2 *__restrict__ chunk_sums, uint64_t ntri,
                        uint32_t *__restrict__ live_tri, uint64_t *__restrict__ live_rowoff,
                        unsigned long long *__restrict__ totals, uint32_t nscan) {
    __shared__ unsigned long long s_a[kBlock / 32 + 1];
    __shared__ unsigned long long s_pre[2];
    // prefix of all earlier chunks
    const uint64_t nchunk_before = (uint64_t)blockIdx.x * kScanPer;
    unsigned long long pl = 0, pr = 0;
    for (uint64_t j = threadIdx.x; j < nchunk_before; j += kBlock) {
        const uint2 c = chunk_sums[j];
        pl += c.x;
        pr += c.y;
    }
    unsigned long long tl, tr;
    block_excl_scan<unsigned long long>(pl, s_a, &tl);
    block_excl_scan<unsigned long long>(pr, s_a, &tr);
    if (threadIdx.x == 0) { s_pre[0] = tl; s_pre[1] = tr; }
    __syncthreads();
    const unsigned long long base_l = s_pre[0], base_r = s_pre[1];
    // this thread's kScanPer consecutive primitives
    const uint64_t t0 = (uint64_t)blockIdx.x * kScanBlock + (uint64_t)threadIdx.x * kScanPer;
    uint32_t r[kScanPer];
    unsigned long long my_l = 0, my_r = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        r[k] = t0 + k < ntri ? rows[t0 + k] : 0u;
        if (r[k] & kRowsBinned) r[k] = 0;  // walked by k_strip
        my_l += r[k] ? 1 : 0;
        my_r += r[k];
    }
    unsigned long long bl, br;
    unsigned long long ol = base_l + block_excl_scan<unsigned long long>(my_l, s_a, &bl);
    unsigned long long orr = base_r + block_excl_scan<unsigned long long>(my_r, s_a, &br);
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        if (r[k]) {
            live_tri[ol] = (uint32_t)(t0 + k);
            live_rowoff[ol] = orr;
            ++ol;
            orr += r[k];
        }
    }
    if (blockIdx.x == nscan - 1 && threadIdx.x == kBlock - 1) {
        totals[0] = base_l + bl;
        totals[1] = base_r + br;
        totals[2] = 0;  // work counter of k_raster, phase 0
        totals[3] = 0;  // work counter of k_raster, phase 1 (ordered scenes)
    }
}

// ---------------------------------------------------------------------------
// k_init: visibility key of every pixel that a primitive may touch (the
// scene's covered rectangle); pixels outside it are never read or written.
// ---------------------------------------------------------------------------
EUC_DEV bool covered(const uint4 &c, uint32_t x, uint32_t y) {
    return x >= c.x && y >= c.y && x < ~c.z && y < ~c.w;
}

// Pixels of the covered rectangle [c.x, ~c.z) x [c.y, ~c.w); 0 when empty.
__host__ __device__ inline uint64_t rect_area(const uint4 &c) {
    const uint32_t x1 = ~c.z, y1 = ~c.w;
    return (c.x < x1 && c.y < y1) ? (uint64_t)(x1 - c.x) * (y1 - c.y) : 0ull;
}

// Blocks of k_init / k_resolve walk groups of `group` consecutive chunks,
// grid-strided, so the scene table is searched once per group rather than
// once per chunk (the host picks group = 1 for small launches, up to
// kChunkGroup for large batches).  The chunks of every scene are counted on
// the device by plan_chunks, from the covered rectangle k_setup found, so no block
// is spent on pixels that no primitive reaches.
constexpr int kChunkGroup = 16;

// Entries i0, i0 + kBlock, i0 + 2 kBlock, ... of a row-major rectangle rw
// wide, as (column, row): one division for the first entry and one for the
// step, then a fixed quotient and remainder per step (the column wraps at
// most once, since both it and the remainder are below rw).
struct RectWalk {
    uint32_t rx, ry, qs, rs, rw;
    EUC_DEV RectWalk(uint32_t i0, uint32_t w) : rw(w) {
        ry = i0 / w;
        rx = i0 - ry * w;
        qs = (uint32_t)kBlock / w;
        rs = (uint32_t)kBlock - qs * w;
    }
    EUC_DEV void next() {
        rx += rs;
        ry += qs;
        if (rx >= rw) {
            rx -= rw;
            ++ry;
        }
    }
};

// Each thread of k_init initialises kInitPer entries of the covered rectangle,
// kBlock apart, so that every load and store instruction of a warp covers 32
// consecutive entries and the kInitPer depth loads are in flight together; a
// chunk is kBlock * kInitPer entries.
constexpr int kInitPer = 8;
constexpr int kInitChunk = kBlock * kInitPer;

// Scene of chunk `c` given the scene of an earlier chunk of the same group.
EUC_DEV int advance_scene(const uint64_t *base, int nsc, int si, uint64_t c) {
    while (si + 1 < nsc && base[si + 1] <= c) ++si;
    return si;
}

// ibase: the first k_init chunk of every scene (nsc + 1 entries, plan_chunks).
__global__ void __launch_bounds__(kBlock) k_init(const SceneDev *__restrict__ sc, const uint64_t *__restrict__ ibase,
                                                 int nsc, const uint4 *__restrict__ cov,
                                                 unsigned long long *__restrict__ vbuf, uint32_t group) {
    __shared__ int s_scene;
    const uint64_t nchunks = ibase[nsc];
    for (uint64_t g = blockIdx.x; g * group < nchunks; g += gridDim.x) {
        const uint64_t c0 = g * group;
        __syncthreads();
        if (threadIdx.x == 0) s_scene = find_scene(ibase, nsc, c0);
        __syncthreads();
        int si = s_scene;
        for (uint64_t c = c0; c < c0 + group && c < nchunks; ++c) {
            si = advance_scene(ibase, nsc, si, c);
            const SceneDev &s = sc[si];
            // pixel and entry indices within a scene fit 32 bits (plan_scene)
            const uint32_t i0 = (uint32_t)(c - ibase[si]) * kInitChunk + threadIdx.x;
            unsigned long long *row0 = vbuf + s.pix_base;
            if (s.keytype == KEY_ORDERED) {
                // every entry, padding included (the pixel scan sums them all):
                // no fragment yet, cursor 0
                const uint32_t lim = (s.W * s.H + kBlock - 1) / kBlock * kBlock;
#pragma unroll
                for (int k = 0; k < kInitPer; ++k)
                    if (i0 + k * kBlock < lim) row0[i0 + k * kBlock] = 0ull;
                continue;
            }
            // entries i0, i0 + kBlock, ... of the covered rectangle, row by row
            const uint4 cv = cov[si];
            const uint32_t area = (uint32_t)rect_area(cv);
            if (i0 >= area) continue;
            RectWalk rk(i0, ~cv.z - cv.x);
            uint32_t px[kInitPer];
            float d[kInitPer];
#pragma unroll
            for (int k = 0; k < kInitPer; ++k, rk.next()) {
                const uint32_t i = i0 + k * kBlock;
                const bool live = i < area;
                const uint32_t x = cv.x + rk.rx, y = cv.y + rk.ry;
                px[k] = live ? y * s.W + x : 0xFFFFFFFFu;
                d[k] = (live && s.keytype == KEY_MIN)
                           ? *reinterpret_cast<const float *>(s.depth + (uint64_t)y * s.dpitch + 4ull * x)
                           : 0.0f;
            }
#pragma unroll
            for (int k = 0; k < kInitPer; ++k)
                if (px[k] != 0xFFFFFFFFu)
                    row0[px[k]] = s.keytype == KEY_MIN ? init_key_min(d[k], s.depth_test == EUC_TEST_GREATER) : ~0ull;
        }
    }
}

// ---------------------------------------------------------------------------
// k_raster: one (primitive, row) at a time per thread, warp-scheduled.
// ---------------------------------------------------------------------------
// Step k (in the window's major range) of line t: its pixel, then the same
// candidate handling as a triangle's pixel (lines.rs:79-97).
EUC_DEV void raster_line_step(const SceneDev &s, const TriRec &r, uint32_t t, uint32_t k,
                              unsigned long long *__restrict__ vbuf, uint32_t &cnt, int phase,
                              uint2 *__restrict__ frags, bool probe) {
    const uint64_t i = (uint64_t)r.pad[4] + k;
    const uint64_t amaj = r.pad[2], amin = r.pad[3];
    // |dmajor|, |dminor| < 2^31: the numerator stays below 2^64
    const uint64_t m = amaj ? (2 * amin * i + amaj - 1) / (2 * amaj) : 0;
    const long long a = (long long)(int32_t)r.pad[0] + ((r.flags & kLineNegMaj) ? -(long long)i : (long long)i);
    const long long b = (long long)(int32_t)r.pad[1] + ((r.flags & kLineNegMin) ? -(long long)m : (long long)m);
    if (b < (long long)r.bx0 || b > (long long)r.bx1) return;  // outside the window's minor range
    const uint32_t x = (uint32_t)((r.flags & kLineXMajor) ? a : b), y = (uint32_t)((r.flags & kLineXMajor) ? b : a);
    const float frac = ((r.flags & kLineUseX) ? (float)x - r.o[0] : (float)y - r.o[1]) * r.o[2];
    const float z = r.zc[0] + frac * (r.zc[1] - r.zc[0]);
    if (s.zclip && !(s.zmin <= z && z <= s.zmax)) return;  // CoordinateMode::passes_z_clip
    unsigned long long *key = vbuf + s.pix_base + (uint64_t)y * s.W + x;
    if (s.keytype == KEY_ORDERED) {
        unsigned int *e = reinterpret_cast<unsigned int *>(key);
        if (phase == 0) {
            ++cnt;
            atomicAdd(e, 1u);
        } else {
            const unsigned int slot = __ldcg(e) + atomicAdd(e + 1, 1u);
            frags[slot] = make_uint2(t, __float_as_uint(z));
        }
        return;
    }
    ++cnt;
    bool pass;
    unsigned long long kv;
    if (s.keytype == KEY_MIN) {
        pass = !isnan(z);
        const float zc = z == 0.0f ? 0.0f : z;
        const uint32_t o = s.depth_test == EUC_TEST_GREATER ? ~ord_f32(zc) : ord_f32(zc);
        kv = ((unsigned long long)o << 32) | (((t + 1u) << 1) | ((z == 0.0f && signbit(z)) ? 1u : 0u));
    } else {
        pass = true;
        if (s.depth_test != EUC_TEST_NONE) {
            const float old = *reinterpret_cast<const float *>(s.depth + (uint64_t)y * s.dpitch + 4ull * x);
            if (s.depth_test == EUC_TEST_LESS) pass = z < old;
            else if (s.depth_test == EUC_TEST_EQUAL) pass = z == old;
            else pass = z > old;
        }
        kv = ((unsigned long long)(~t) << 32) | __float_as_uint(z);
    }
    if (!pass) return;
    if (!probe || kv < __ldcg(key)) atomicMin(key, kv);
}

// The pixel span [xs, xe) of row y of triangle r: the whole band-clamped
// bbox row when the extent is below 128, else the edge intersections
// (triangles.rs:219-253).  False when it is empty.
EUC_DEV bool row_span(const SceneDev &s, const TriRec &r, uint32_t y, uint32_t &xs, uint32_t &xe) {
    const float yf = (float)y;
    bool full = r.flags & 2u;  // one band, extent < 128 (k_setup)
    if (!full && !(r.flags & 4u)) {  // rows in several bands
        // band of this row and the band-clamped bbox (pipeline.rs:341-360, triangles.rs:114-139)
        const uint32_t lo = (y / s.gr) * s.gr;
        const uint32_t hi = min(lo + s.gr, s.H);
        const uint32_t by0c = max(r.by0, lo), by1c = min(r.by1, hi);
        full = (unsigned long long)(r.bx1 - r.bx0) * (unsigned long long)(by1c - by0c) < 128ull;
    }
    if (full) {  // triangles.rs:224-226
        xs = r.bx0;
        xe = r.bx1;
    } else {     // triangles.rs:228-253
        const float ax = r.vby[0], ay = r.vby[1], bxv = r.vby[2], byv = r.vby[3], cx = r.vby[4], cy = r.vby[5];
        const float ac = ax + ((yf - ay) / (cy - ay)) * (cx - ax);
        float lo_f, hi_f;
        if (yf < byv) {
            const float ab = ax + ((yf - ay) / (byv - ay)) * (bxv - ax);
            lo_f = rmin(ab, ac);
            hi_f = rmax(ab, ac);
        } else {
            const float bc = bxv + ((yf - byv) / (cy - byv)) * (cx - bxv);
            lo_f = rmin(bc, ac);
            hi_f = rmax(bc, ac);
        }
        const float fx0 = (float)r.bx0, fx1 = (float)r.bx1;
        const float fl = floorf(lo_f), ce = ceilf(hi_f);
        xs = (fl >= fx0 && fl < fx1) ? sat_u32(fl) : r.bx0;
        xe = (ce >= fx0 && ce < fx1) ? sat_u32(ce) : r.bx1;
    }
    return xs < xe;
}

EUC_DEV void raster_row(const SceneDev &s, const TriRec &r, uint32_t t, uint32_t y,
                        unsigned long long *__restrict__ vbuf, uint32_t &cnt, int phase, uint2 *__restrict__ frags,
                        bool probe) {
    if (s.prim != EUC_PRIM_TRIANGLE_LIST) {  // lines: `y` is the step within the window
        raster_line_step(s, r, t, y, vbuf, cnt, phase, frags, probe);
        return;
    }
    uint32_t xs, xe;
    if (!row_span(s, r, y, xs, xe)) return;
    // row-start weights, then the serial walk (triangles.rs:257-301)
    const float yf = (float)y;
    const float xsf = (float)xs;
    float w0 = (r.o[0] + r.dy[0] * yf) + r.dx[0] * xsf;
    float w1 = (r.o[1] + r.dy[1] * yf) + r.dx[1] * xsf;
    float w2 = (r.o[2] + r.dy[2] * yf) + r.dx[2] * xsf;
    const float d0 = r.dx[0], d1 = r.dx[1], d2 = r.dx[2];
    const float z0 = r.zc[0], z1 = r.zc[1], z2 = r.zc[2];
    const bool noclip = r.flags & 1u;
    unsigned long long *row_keys = vbuf + s.pix_base + (uint64_t)y * s.W;
    const float *row_depth = s.depth ? reinterpret_cast<const float *>(s.depth + (uint64_t)y * s.dpitch) : nullptr;
    const bool kmin = s.keytype == KEY_MIN, greater = s.depth_test == EUC_TEST_GREATER;
    const uint32_t tmin = (t + 1u) << 1;
    const unsigned long long tlast = (unsigned long long)(~t) << 32;
    if (kmin && !probe) {
        // Less / Greater with depth writes, fire-and-forget reductions: each
        // candidate is keyed and reduced where the walk finds it
        const uint32_t flip = greater ? 0xFFFFFFFFu : 0u;
#pragma unroll 4
        for (uint32_t x = xs; x < xe; ++x) {
            const float wu2 = (w2 - w0) - w1;
            if (w0 >= 0.0f && w1 >= 0.0f && wu2 >= 0.0f) {
                const float z = (z0 * w0 + z1 * w1) + z2 * wu2;
                if (noclip || (s.zmin <= z && z <= s.zmax)) {
                    ++cnt;
                    if (z == z) {  // a NaN depth fails every test (partial_cmp is None)
                        const uint32_t b = __float_as_uint(z + 0.0f);  // -0 and +0 compare equal
                        const uint32_t o = (b ^ ((uint32_t)((int32_t)b >> 31) | 0x80000000u)) ^ flip;
                        const uint32_t neg0 = __float_as_uint(z) == 0x80000000u ? 1u : 0u;
                        atomicMin(row_keys + x, ((unsigned long long)o << 32) | (tmin | neg0));
                    }
                }
            }
            w0 = w0 + d0;
            w1 = w1 + d1;
            w2 = w2 + d2;
        }
        return;
    }
    // The walk advances pixel by pixel exactly as euc's loop does; candidates
    // are gathered kWalk at a time so that their key loads are in flight
    // together instead of one L2 round trip per pixel.
    constexpr int kWalk = 4;
    static_assert(kWalk == 4, "the empty-group test below names four candidates");
    for (uint32_t x = xs; x < xe; x += kWalk) {
        float zz[kWalk];
        bool cand[kWalk];
#pragma unroll
        for (int k = 0; k < kWalk; ++k) {
            cand[k] = false;
            zz[k] = 0.0f;
            if (x + k < xe) {
                const float wu2 = (w2 - w0) - w1;
                if (w0 >= 0.0f && w1 >= 0.0f && wu2 >= 0.0f) {
                    const float z = (z0 * w0 + z1 * w1) + z2 * wu2;
                    if (noclip || (s.zmin <= z && z <= s.zmax)) {
                        cand[k] = true;
                        zz[k] = z;
                    }
                }
                w0 = w0 + d0;
                w1 = w1 + d1;
                w2 = w2 + d2;
            }
        }
        // most groups of a full-bbox row (extent < 128) hold no candidate:
        // only the weight additions above are needed there
        if (!(cand[0] | cand[1] | cand[2] | cand[3])) continue;
        if (s.keytype == KEY_ORDERED) {
            // phase 0 counts each pixel's candidates (low word of its entry);
            // phase 1 appends (primitive, z) at offset (low word, set by the
            // pixel scan) + cursor (high word)
#pragma unroll
            for (int k = 0; k < kWalk; ++k) {
                if (!cand[k]) continue;
                unsigned int *e = reinterpret_cast<unsigned int *>(row_keys + x + k);
                if (phase == 0) {
                    ++cnt;
                    atomicAdd(e, 1u);
                } else {
                    const unsigned int slot = __ldcg(e) + atomicAdd(e + 1, 1u);
                    frags[slot] = make_uint2(t, __float_as_uint(zz[k]));
                }
            }
            continue;
        }
        unsigned long long key[kWalk];
        bool pass[kWalk];
        float old[kWalk];
        if (!kmin && s.depth_test != EUC_TEST_NONE) {
#pragma unroll
            for (int k = 0; k < kWalk; ++k) old[k] = cand[k] ? row_depth[x + k] : 0.0f;
        }
#pragma unroll
        for (int k = 0; k < kWalk; ++k) {
            cnt += cand[k] ? 1u : 0u;
            const float z = zz[k];
            if (kmin) {
                pass[k] = cand[k] && !isnan(z);
                const float zc = z == 0.0f ? 0.0f : z;
                const uint32_t o = greater ? ~ord_f32(zc) : ord_f32(zc);
                const uint32_t neg0 = (z == 0.0f && signbit(z)) ? 1u : 0u;
                key[k] = ((unsigned long long)o << 32) | (tmin | neg0);
            } else {
                bool p = cand[k];
                if (s.depth_test == EUC_TEST_LESS) p = p && z < old[k];
                else if (s.depth_test == EUC_TEST_EQUAL) p = p && z == old[k];
                else if (s.depth_test == EUC_TEST_GREATER) p = p && z > old[k];
                pass[k] = p;
                key[k] = tlast | __float_as_uint(z);
            }
        }
        if (probe) {
            // read the keys first and skip the atomics that cannot win (high
            // depth complexity: most candidates lose)
            unsigned long long cur[kWalk];
#pragma unroll
            for (int k = 0; k < kWalk; ++k) cur[k] = pass[k] ? __ldcg(row_keys + x + k) : 0ull;
#pragma unroll
            for (int k = 0; k < kWalk; ++k)
                if (pass[k] && key[k] < cur[k]) atomicMin(row_keys + x + k, key[k]);
        } else {
            // fire-and-forget reductions: the walk never waits on memory
#pragma unroll
            for (int k = 0; k < kWalk; ++k)
                if (pass[k]) atomicMin(row_keys + x + k, key[k]);
        }
    }
}

// Warps are scheduled independently: a warp claims the next `witems`
// (primitive, row) items from a global counter, finds the first primitive of
// its range with a 32-way search of the row offsets, copies the offsets of
// the (at most `witems`) primitives that the range can touch into shared
// memory and maps each lane's items with a binary search there.  Rows of one
// large primitive spread over many warps; no block barrier couples a warp to
// the slowest row of another warp.  witems: a multiple of 32, at most
// kWarpItems (a launch-shape choice; results do not depend on it).
constexpr int kWarpItems = 256;

__global__ void __launch_bounds__(kBlock, 4) k_raster(const SceneDev *__restrict__ sc, const TriRec *__restrict__ recs,
                                                   const uint32_t *__restrict__ live_tri,
                                                   const uint64_t *__restrict__ live_rowoff,
                                                   unsigned long long *__restrict__ totals,
                                                   const int *__restrict__ err, unsigned long long *__restrict__ vbuf,
                                                   SceneStats *__restrict__ stats, int phase,
                                                   uint2 *__restrict__ frags, int witems, bool probe) {
    __shared__ uint64_t s_off[kBlock / 32][kWarpItems];
    const int lane = threadIdx.x & 31;
    uint64_t *off = s_off[threadIdx.x >> 5];
    const uint64_t nlive = totals[0], nitems = totals[1];
    // Few items for the grid (a small scene): smaller claims, down to one
    // step, so that every warp gets some instead of a few warps walking
    // many steps each (uniform over the grid: it depends on nitems alone)
    {
        const uint64_t nwarps = (uint64_t)gridDim.x * (kBlock / 32);
        const uint64_t fair = (nitems + nwarps - 1) / nwarps;
        if (fair < (uint64_t)witems) witems = (int)max((uint64_t)32, (fair + 31) / 32 * 32);
    }
    // Warps beyond the number of chunks would only find the counter exhausted;
    // they leave at once instead of queueing on its atomic.
    const uint64_t gwarp = (uint64_t)blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5);
    if (gwarp * witems >= nitems) return;
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(totals + 2 + phase, (unsigned long long)witems);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= nitems) break;
        // largest l with live_rowoff[l] <= base; invariant off(lo) <= base < off(hi)
        uint64_t lo = 0, hi = nlive;
        while (hi - lo > 32) {
            const uint64_t step = (hi - lo + 31) / 32;
            const uint64_t at = lo + lane * step;
            const bool le = at < hi && live_rowoff[at] <= base;
            const int k = 31 - __clz(__ballot_sync(0xFFFFFFFFu, le));  // lane 0 always qualifies
            lo = lo + (uint64_t)k * step;
            hi = min(lo + step, hi);
        }
        {
            const bool le = lo + lane < hi && live_rowoff[lo + lane] <= base;
            lo += 31 - __clz(__ballot_sync(0xFFFFFFFFu, le));
        }
        const uint64_t l0 = lo;
        for (int j = lane; j < witems; j += 32) off[j] = l0 + j < nlive ? live_rowoff[l0 + j] : ~0ull;
        __syncwarp();
        uint32_t scene0 = 0xFFFFFFFFu, cnt0 = 0;
        // The 32 items of a step are consecutive, so their primitives are a
        // run of the window from a0 (the primitive of the step's first item):
        // lane j marks where primitive a0 + 1 + j starts within the step, and
        // each lane counts the starts at or before its own item.
        int a0 = 0;  // window entry 0 is the primitive of item `base`
        for (int s = 0; s < witems / 32; ++s) {
            const uint64_t i0 = base + (uint64_t)s * 32;
            if (i0 >= nitems) break;
            const int c = a0 + 1 + lane;
            uint32_t bit = 0;
            if (lane < 31 && c < witems) {
                const uint64_t o = off[c];
                if (o > i0 && o < i0 + 32) bit = 1u << (uint32_t)(o - i0);
            }
            const uint32_t starts = __reduce_or_sync(0xFFFFFFFFu, bit);
            const int a = a0 + __popc(starts & ((2u << lane) - 1u));
            const int alast = a0 + __popc(starts);  // the primitive of the step's last item
            a0 = (alast + 1 < witems && off[alast + 1] == i0 + 32) ? alast + 1 : alast;
            const uint64_t i = i0 + lane;
            if (i >= nitems) continue;
            const uint32_t t = live_tri[l0 + a];
            TriRec r = load_rec(recs + t, kRecRaster);
            const uint32_t scene = r.scene;
            if (err[scene]) continue;
            if (sc[scene].prim != EUC_PRIM_TRIANGLE_LIST) r = load_rec(recs + t, kRecAll);  // a line's walk state
            if (phase == 1 && sc[scene].keytype != KEY_ORDERED) continue;  // the fill pass is for ordered scenes
            uint32_t cnt = 0;
            raster_row(sc[scene], r, t, r.by0 + (uint32_t)(i - off[a]), vbuf, cnt, phase, frags, probe);
            if (scene0 == 0xFFFFFFFFu) scene0 = scene;
            if (scene == scene0) cnt0 += cnt;
            else if (cnt) atomicAdd(&stats[scene].candidates, (unsigned long long)cnt);
        }
        // per-lane counts for each lane's first scene; most warps hold one scene
        const uint32_t s0 = __shfl_sync(0xFFFFFFFFu, scene0, 0);
        if (__all_sync(0xFFFFFFFFu, scene0 == s0 || cnt0 == 0)) {
            const uint32_t sum = warp_sum(cnt0);
            if (lane == 0 && sum) atomicAdd(&stats[s0].candidates, (unsigned long long)sum);
        } else if (cnt0) {
            atomicAdd(&stats[scene0].candidates, (unsigned long long)cnt0);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// k_bin_count: the strip path's routing and entry counts, after k_setup (a
// scene's fragment estimate and covered rectangle are complete by then).
// Blocks stride the setup chunks (each one scene); a chunk of a scene the
// path does not take costs one check.  A primitive of a scene that the path
// takes is admitted while the entry list has room: its rows are marked
// kRowsBinned (the item queue skips it, and its chunk's sums drop it), and
// each strip it overlaps counts one entry, first in the block's shared
// memory, then with one global atomic per strip.
// strip_mode: 0 route by overdraw, 2 every scene the path can take.
// ---------------------------------------------------------------------------
EUC_DEV bool strip_routed(const SceneDev &s, const SceneStats &st, const uint4 &cv, uint32_t strip_mode) {
    return s.strip_h && (strip_mode == 2 || (st.walked >= kStripOverdraw * rect_area(cv) &&
                                             st.walked >= kStripTriFrags * st.live));
}

__global__ void __launch_bounds__(kBlock) k_bin_count(const SceneDev *__restrict__ sc,
                                                      const uint32_t *__restrict__ chunk_scene, uint64_t nchunks,
                                                      uint32_t *__restrict__ rows, const uint4 *__restrict__ bbox,
                                                      const uint4 *__restrict__ cov,
                                                      const SceneStats *__restrict__ stats,
                                                      uint2 *__restrict__ chunk_sums, uint32_t *__restrict__ strip_cnt,
                                                      unsigned long long *__restrict__ nentries, uint64_t entry_cap,
                                                      uint32_t strip_mode) {
    __shared__ uint32_t s_hist[kBinHist];
    const int lane = threadIdx.x & 31;
    for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {  // uniform over the block
        const int si = chunk_scene ? (int)chunk_scene[c] : 0;
        const SceneDev &s = sc[si];
        if (!strip_routed(s, stats[si], cov[si], strip_mode)) continue;
        const uint64_t t = c * kBlock + threadIdx.x;
        const bool local = s.nstrips <= kBinHist;
        __syncthreads();  // the previous chunk's flush is done with the histogram
        for (uint32_t q = threadIdx.x; local && q < s.nstrips; q += kBlock) s_hist[q] = 0;
        const uint32_t nr = rows[t];
        uint32_t q0 = 0, nst = 0;
        if (nr) {
            const uint4 w3 = __ldg(bbox + t);  // bx0, bx1, by0, by1
            q0 = w3.z / s.strip_h;
            nst = (w3.w - 1) / s.strip_h - q0 + 1;
        }
        // admission, in warp order while the entry list has room
        const uint32_t inc = warp_incl_scan(nst), tot = __shfl_sync(0xFFFFFFFFu, inc, 31);
        unsigned long long at = 0;
        if (lane == 31 && tot) at = atomicAdd(nentries, (unsigned long long)tot);
        at = __shfl_sync(0xFFFFFFFFu, at, 31);
        const bool binned = nst && at + inc <= entry_cap;
        __syncthreads();  // the histogram is clear
        if (binned) {
            rows[t] = nr | kRowsBinned;
            for (uint32_t k = 0; k < nst; ++k) {
                if (local) atomicAdd(s_hist + q0 + k, 1u);
                else atomicAdd(strip_cnt + s.strip_base + q0 + k, 1u);
            }
        }
        const uint32_t bl = warp_sum(binned ? 1u : 0u), br = warp_sum(binned ? nr : 0u);
        if (lane == 0 && bl) {
            atomicSub(&chunk_sums[c].x, bl);
            atomicSub(&chunk_sums[c].y, br);
        }
        __syncthreads();
        for (uint32_t q = threadIdx.x; local && q < s.nstrips; q += kBlock)
            if (s_hist[q]) atomicAdd(strip_cnt + s.strip_base + q, s_hist[q]);
    }
}

// ---------------------------------------------------------------------------
// k_bin: the strip lists.  Every admitted primitive (kRowsBinned) adds one
// entry {primitive, first row << 16 | end row} (rows relative to the strip)
// to each strip it overlaps; the order within a list does not matter.
// Blocks stride the setup chunks (each one scene): a chunk counts its entries
// per strip in shared memory, reserves each strip's range with one global
// atomic, then writes the entries.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_bin(const SceneDev *__restrict__ sc, const uint32_t *__restrict__ chunk_scene,
                                                uint64_t nchunks, const uint32_t *__restrict__ rows,
                                                const uint4 *__restrict__ bbox, const uint4 *__restrict__ cov,
                                                const SceneStats *__restrict__ stats,
                                                const uint32_t *__restrict__ strip_off, uint32_t *__restrict__ strip_fill,
                                                uint2 *__restrict__ entries, uint32_t strip_mode) {
    __shared__ uint32_t s_cnt[kBinHist], s_base[kBinHist];
    for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {  // uniform over the block
        const int si = chunk_scene ? (int)chunk_scene[c] : 0;
        const SceneDev &s = sc[si];
        if (!strip_routed(s, stats[si], cov[si], strip_mode)) continue;
        const uint64_t t = c * kBlock + threadIdx.x;
        const bool local = s.nstrips <= kBinHist;
        __syncthreads();  // the previous chunk is done with the counts
        for (uint32_t q = threadIdx.x; local && q < s.nstrips; q += kBlock) s_cnt[q] = 0;
        const uint32_t h = s.strip_h;
        uint32_t by0 = 0, by1 = 0, q0 = 0, nst = 0;
        if (rows[t] & kRowsBinned) {
            const uint4 w3 = __ldg(bbox + t);  // bx0, bx1, by0, by1
            by0 = w3.z;
            by1 = w3.w;
            q0 = by0 / h;
            nst = (by1 - 1) / h - q0 + 1;
        }
        __syncthreads();
        if (local) {
            for (uint32_t k = 0; k < nst; ++k) atomicAdd(s_cnt + q0 + k, 1u);
            __syncthreads();
            for (uint32_t q = threadIdx.x; q < s.nstrips; q += kBlock) {
                const uint32_t n = s_cnt[q];
                if (n) s_base[q] = strip_off[s.strip_base + q] + atomicAdd(strip_fill + s.strip_base + q, n);
                s_cnt[q] = 0;
            }
            __syncthreads();
        }
        for (uint32_t k = 0; k < nst; ++k) {
            const uint32_t q = q0 + k, g = s.strip_base + q, s0 = q * h;
            const uint32_t pos = local ? s_base[q] + atomicAdd(s_cnt + q, 1u) : strip_off[g] + atomicAdd(strip_fill + g, 1u);
            const uint32_t ya = max(by0, s0) - s0, yb = min(by1, s0 + h) - s0;
            entries[pos] = make_uint2((uint32_t)t, (ya << 16) | yb);
        }
    }
}

// Shared-memory 64-bit min reduction (no value returned).
EUC_DEV void smem_min_u64(uint32_t saddr, unsigned long long v) {
    asm volatile("red.shared.min.u64 [%0], %1;" ::"r"(saddr), "l"(v) : "memory");
}

// The KEY_MIN walk of strip_walk_row, with the clip-range test compiled in
// or out (a record's flag bit 0: the whole triangle lies inside [zmin, zmax]).
template <bool kClip>
EUC_DEV void strip_walk_min(float w0, float w1, float w2, float d0, float d1, float d2, float z0, float z1, float z2,
                            float zmin, float zmax, uint32_t flip, uint32_t tmin, uint32_t xs, uint32_t xe,
                            uint32_t srow, uint32_t &cnt) {
#pragma unroll 4
    for (uint32_t x = xs; x < xe; ++x) {
        const float wu2 = (w2 - w0) - w1;
        if (w0 >= 0.0f && w1 >= 0.0f && wu2 >= 0.0f) {
            const float z = (z0 * w0 + z1 * w1) + z2 * wu2;
            if (!kClip || (zmin <= z && z <= zmax)) {
                ++cnt;
                if (z == z) {  // a NaN depth fails every test (partial_cmp is None)
                    const uint32_t b = __float_as_uint(z + 0.0f);  // -0 and +0 compare equal
                    const uint32_t o = (b ^ ((uint32_t)((int32_t)b >> 31) | 0x80000000u)) ^ flip;
                    const uint32_t neg0 = __float_as_uint(z) == 0x80000000u ? 1u : 0u;
                    smem_min_u64(srow + 8u * x, ((unsigned long long)o << 32) | (tmin | neg0));
                }
            }
        }
        w0 = w0 + d0;
        w1 = w1 + d1;
        w2 = w2 + d2;
    }
}

// walk_row for a strip: the same serial walk (triangles.rs:257-301), with
// the keys in shared memory; `srow` is the shared address of the row's key
// for x = 0 (8 bytes per pixel).  KEY_MIN or KEY_LAST scenes.
EUC_DEV void strip_walk_row(const SceneDev &s, const TriRec &r, uint32_t t, uint32_t y, uint32_t xs, uint32_t xe,
                            uint32_t srow, uint32_t &cnt) {
    const float yf = (float)y;
    const float xsf = (float)xs;
    float w0 = (r.o[0] + r.dy[0] * yf) + r.dx[0] * xsf;
    float w1 = (r.o[1] + r.dy[1] * yf) + r.dx[1] * xsf;
    float w2 = (r.o[2] + r.dy[2] * yf) + r.dx[2] * xsf;
    const float d0 = r.dx[0], d1 = r.dx[1], d2 = r.dx[2];
    const float z0 = r.zc[0], z1 = r.zc[1], z2 = r.zc[2];
    const bool noclip = r.flags & 1u;
    const float zmin = s.zmin, zmax = s.zmax;
    if (s.keytype == KEY_MIN) {
        const uint32_t flip = s.depth_test == EUC_TEST_GREATER ? 0xFFFFFFFFu : 0u;
        const uint32_t tmin = (t + 1u) << 1;
        if (noclip)
            strip_walk_min<false>(w0, w1, w2, d0, d1, d2, z0, z1, z2, zmin, zmax, flip, tmin, xs, xe, srow, cnt);
        else
            strip_walk_min<true>(w0, w1, w2, d0, d1, d2, z0, z1, z2, zmin, zmax, flip, tmin, xs, xe, srow, cnt);
        return;
    }
    // KEY_LAST: every fragment against the unchanged initial depth
    const float *row_depth = s.depth ? reinterpret_cast<const float *>(s.depth + (uint64_t)y * s.dpitch) : nullptr;
    const unsigned long long tlast = (unsigned long long)(~t) << 32;
    for (uint32_t x = xs; x < xe; ++x) {
        const float wu2 = (w2 - w0) - w1;
        if (w0 >= 0.0f && w1 >= 0.0f && wu2 >= 0.0f) {
            const float z = (z0 * w0 + z1 * w1) + z2 * wu2;
            if (noclip || (zmin <= z && z <= zmax)) {
                ++cnt;
                bool pass = true;
                if (s.depth_test != EUC_TEST_NONE) {
                    const float old = row_depth[x];
                    if (s.depth_test == EUC_TEST_LESS) pass = z < old;
                    else if (s.depth_test == EUC_TEST_EQUAL) pass = z == old;
                    else pass = z > old;
                }
                if (pass) smem_min_u64(srow + 8u * x, tlast | __float_as_uint(z));
            }
        }
        w0 = w0 + d0;
        w1 = w1 + d1;
        w2 = w2 + d2;
    }
}

// Block-wide exclusive scan over kStripThreads threads (k_strip).
EUC_DEV uint32_t strip_block_scan(uint32_t v, uint32_t *smem /* >= kStripThreads/32 + 1 */, uint32_t *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t inc = warp_incl_scan(v);
    if (lane == 31) smem[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint32_t x = lane < kStripThreads / 32 ? smem[lane] : 0u;
        const uint32_t xi = warp_incl_scan(x);
        if (lane < kStripThreads / 32) smem[lane] = xi - x;
        if (lane == kStripThreads / 32 - 1) smem[kStripThreads / 32] = xi;
    }
    __syncthreads();
    const uint32_t r = smem[warp] + inc - v;
    *total = smem[kStripThreads / 32];
    __syncthreads();
    return r;
}

// ---------------------------------------------------------------------------
// k_strip: one unit (up to kStripUnit entries of one strip) at a time per
// block, claimed from a work counter (totals[7]).  sbase: the first strip of
// each scene (nsc + 1 entries).  The unit's keys over the strip's rows inside
// the scene's covered rectangle start at ~0 in shared memory; the warps
// claim runs of kStripClaim items of its entries from a shared counter and
// walk them with shared-memory reductions; every key the unit lowered is
// then merged into vbuf (which k_init seeded) with one 64-bit min and put
// back to ~0 for the next unit.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kStripThreads, kStripBlocksPerSm) k_strip(const SceneDev *__restrict__ sc,
                                                            const uint64_t *__restrict__ sbase, int nsc,
                                                            const uint4 *__restrict__ cov,
                                                            const uint32_t *__restrict__ strip_off,
                                                            const uint32_t *__restrict__ strip_uoff,
                                                            const uint32_t *__restrict__ unit_strip,
                                                            const uint2 *__restrict__ entries,
                                                            const TriRec *__restrict__ recs,
                                                            const int *__restrict__ err,
                                                            unsigned long long *__restrict__ vbuf,
                                                            SceneStats *__restrict__ stats,
                                                            unsigned long long *__restrict__ totals) {
    extern __shared__ unsigned long long s_keys[];  // rows [r0, r1) x columns [cx0, cx1) of the strip
    __shared__ uint32_t s_pref[kStripUnit];         // first item of each entry of the unit (in width order)
    __shared__ uint32_t s_t[kStripUnit];            // its primitive
    __shared__ uint8_t s_ya[kStripUnit];            // its first row within the strip
    __shared__ uint8_t s_nr[kStripUnit];            // its rows within the strip
    __shared__ uint32_t s_bkt[kWidthBuckets];       // entries per width bucket, then the bucket's first position
    __shared__ uint32_t s_scan[kStripThreads / 32 + 1];
    __shared__ uint16_t s_first[kStripUnit * kStripMaxRows / 32];  // entry holding item 32k of the unit
    __shared__ uint32_t s_u, s_next;
    static_assert(2 * kStripThreads == kStripUnit && kStripMaxRows <= 255, "two entries per thread, rows in 8 bits");
    static_assert(kStripMaxRows < 32 && kStripClaim % 32 == 0 && kStripUnit <= 65536,
                  "one table slot per entry at most, claims start at a slot, entries in 16 bits");
    static_assert(offsetof(TriRec, bx0) == 48, "k_strip reads the bbox width from 8-byte word 6 of a record");
    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t nstrips = (uint32_t)sbase[nsc];
    const uint32_t nunits = strip_uoff[nstrips];
    const uint32_t keys_saddr = (uint32_t)__cvta_generic_to_shared(s_keys);
    uint32_t key_bytes;  // the launch's dynamic shared memory
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(key_bytes));
    for (uint32_t i = tid; i < key_bytes / 8; i += kStripThreads) s_keys[i] = ~0ull;
    for (;;) {
        if (tid == 0) {
            s_u = (uint32_t)atomicAdd(totals + 7, 1ull);
            s_next = 0;
        }
        __syncthreads();
        const uint32_t u = s_u;
        if (u >= nunits) break;
        const uint32_t g = unit_strip[u];
        const int si = find_scene(sbase, nsc, g);
        const SceneDev &s = sc[si];
        const uint4 cv = cov[si];
        const uint32_t s0 = (g - s.strip_base) * s.strip_h;
        // every entry's rows lie in the strip and in the covered rectangle
        const uint32_t r0 = max(s0, cv.y), r1 = min(min(s0 + s.strip_h, s.H), ~cv.w);
        const uint32_t cx0 = cv.x, cx1 = ~cv.z;
        const bool empty = r0 >= r1 || cx0 >= cx1;  // never for a strip with entries
        const uint32_t wc = empty ? 0u : cx1 - cx0, area = empty ? 0u : (r1 - r0) * strip_pitch(wc);
        const uint32_t pitch = strip_pitch(wc);
        const uint32_t e_begin = strip_off[g] + (u - strip_uoff[g]) * kStripUnit;
        const int nload = (int)(min(e_begin + kStripUnit, strip_off[g + 1]) - e_begin);
        // the unit's entries, two per thread, ordered by the span of their
        // middle row in the strip, widest first (a counting sort over
        // kWidthBuckets): the rows a warp walks together have about the same
        // length, and the short ones come last, so that the warps reach the
        // unit's closing barrier together
        if (tid < (int)kWidthBuckets) s_bkt[tid] = 0;
        uint2 ev[2];
        uint32_t bk[2], rk[2];
        __syncthreads();
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = 2 * tid + h;
            ev[h] = make_uint2(0u, 0u);
            bk[h] = 0xFFFFFFFFu;
            if (k < nload) {
                ev[h] = entries[e_begin + k];
                // the span of the entry's middle row in this strip: the bbox
                // width where every row spans it, else the edge intersections
                TriRec rs = load_rec(recs + ev[h].x, 0x38u);  // words 3-5
                uint32_t xs = rs.bx0, xe = rs.bx1;
                if (!(rs.flags & 2u)) {
                    const uint32_t ya = ev[h].y >> 16, yb = ev[h].y & 0xFFFFu;
                    if (!row_span(s, rs, s0 + ((ya + yb) >> 1), xs, xe)) xe = xs;
                }
                bk[h] = kWidthBuckets - 1u - width_bucket(xe - xs);  // widest first
            }
            const uint32_t m = __match_any_sync(0xFFFFFFFFu, bk[h]);
            const int leader = __ffs(m) - 1;
            uint32_t base = 0;
            if (bk[h] != 0xFFFFFFFFu && lane == leader) base = atomicAdd(s_bkt + bk[h], (uint32_t)__popc(m));
            rk[h] = __shfl_sync(0xFFFFFFFFu, base, leader) + __popc(m & ((1u << lane) - 1u));
        }
        __syncthreads();
        if (tid < 32) {  // bucket sizes -> first positions
            static_assert(kWidthBuckets == 64, "two buckets per lane");
            const uint32_t c0 = s_bkt[2 * lane], c1 = s_bkt[2 * lane + 1];
            const uint32_t inc = warp_incl_scan(c0 + c1);
            s_bkt[2 * lane] = inc - c0 - c1;
            s_bkt[2 * lane + 1] = inc - c1;
        }
        __syncthreads();
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (bk[h] == 0xFFFFFFFFu) continue;
            const uint32_t d = s_bkt[bk[h]] + rk[h];
            s_t[d] = ev[h].x;
            s_ya[d] = (uint8_t)(ev[h].y >> 16);
            s_nr[d] = (uint8_t)((ev[h].y & 0xFFFFu) - (ev[h].y >> 16));
        }
        __syncthreads();
        const uint32_t n0 = 2 * tid < nload ? s_nr[2 * tid] : 0u, n1 = 2 * tid + 1 < nload ? s_nr[2 * tid + 1] : 0u;
        uint32_t total;
        const uint32_t pre = strip_block_scan(n0 + n1, s_scan, &total);
        s_pref[2 * tid] = pre;
        s_pref[2 * tid + 1] = pre + n0;
        // an entry has at most kStripMaxRows < 32 items, so at most one
        // multiple of 32 falls in its range
        if (n0 && ((pre + 31u) & ~31u) < pre + n0) s_first[(pre + 31u) >> 5] = (uint16_t)(2 * tid);
        if (n1 && ((pre + n0 + 31u) & ~31u) < pre + n0 + n1) s_first[(pre + n0 + 31u) >> 5] = (uint16_t)(2 * tid + 1);
        __syncthreads();
        uint32_t cnt = 0;
        if (!err[si] && !empty) {  // a scene with a bad index draws nothing
            for (;;) {
                uint32_t i0 = 0;
                if (lane == 0) i0 = atomicAdd(&s_next, kStripClaim);
                i0 = __shfl_sync(0xFFFFFFFFu, i0, 0);
                if (i0 >= total) break;
                int a0 = s_first[i0 >> 5];  // the entry of item i0 (a multiple of kStripClaim)
                const uint32_t iend = min(total, i0 + kStripClaim);
                // 32 consecutive items at a time: their entries are a run from
                // a0 (every entry has at least one row)
                for (uint32_t j0 = i0; j0 < iend; j0 += 32) {
                    const int c = a0 + 1 + lane;
                    uint32_t bit = 0;
                    if (lane < 31 && c < nload) {
                        const uint32_t o = s_pref[c];
                        if (o > j0 && o < j0 + 32) bit = 1u << (o - j0);
                    }
                    const uint32_t starts = __reduce_or_sync(0xFFFFFFFFu, bit);
                    const int a = a0 + __popc(starts & ((2u << lane) - 1u));
                    const int alast = a0 + __popc(starts);
                    a0 = (alast + 1 < nload && s_pref[alast + 1] == j0 + 32) ? alast + 1 : alast;
                    const uint32_t i = j0 + lane;
                    if (i >= iend) continue;
                    const uint32_t t = s_t[a];
                    const uint32_t y = s0 + s_ya[a] + (i - s_pref[a]);
                    const TriRec r = load_rec(recs + t, kRecRaster);
                    uint32_t xs, xe;
                    if (!row_span(s, r, y, xs, xe)) continue;
                    strip_walk_row(s, r, t, y, xs, xe, keys_saddr + 8u * ((y - r0) * pitch) - 8u * cx0, cnt);
                }
            }
        }
        __syncthreads();
        // merge the keys this unit lowered (the padding column is never
        // written) and put them back to ~0; key i is at row i / pitch, column
        // i % pitch, stepped by kStripThreads without a division
        if (area) {
            const uint32_t qs = kStripThreads / pitch, rs = kStripThreads - qs * pitch;
            uint32_t ry = tid / pitch, rx = tid - ry * pitch;
            unsigned long long *drow = vbuf + s.pix_base + (uint64_t)(r0 + ry) * s.W + cx0;
            for (uint32_t i = tid; i < area; i += kStripThreads) {
                const unsigned long long k = s_keys[i];
                if (k != ~0ull) {
                    atomicMin(drow + rx, k);
                    s_keys[i] = ~0ull;
                }
                rx += rs;
                const uint32_t wrap = rx >= pitch ? 1u : 0u;
                rx -= wrap * pitch;
                drow += (uint64_t)(qs + wrap) * s.W;
            }
        }
        const uint32_t wsum = warp_sum(cnt);
        if (lane == 0 && wsum) atomicAdd(&stats[si].candidates, (unsigned long long)wsum);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// k_resolve<F>: shade the winner of every pixel and write colour / depth.
// ---------------------------------------------------------------------------
template <class F>
EUC_DEV void get_v_data(const TriRec &r, const float *__restrict__ vd0, const float *__restrict__ vd1,
                        const float *__restrict__ vd2, float xf, float yf, float *out) {  // triangles.rs:274-294
    float w[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) w[c] = (r.o[c] + r.dy[c] * yf) + r.dx[c] * xf;
    const float wu2 = (w[2] - w[0]) - w[1];
    const float rr = 1.0f / w[2];
    const float p0 = w[0] * rr, p1 = w[1] * rr, p2 = wu2 * rr;
#pragma unroll
    for (int i = 0; i < F::NV; ++i) out[i] = (vd0[i] * p0 + vd1[i] * p1) + vd2[i] * p2;
}

// The winner's vertex outputs at (xf, yf): get_v_data for a triangle,
// weighted_sum2 of the two ends for a line (lines.rs:98-110).
template <class F>
EUC_DEV void vdata_at(const SceneDev &s, const TriRec &r, const float *__restrict__ vb, float xf, float yf,
                      float *out) {
    constexpr int S = vd_stride(F::NV);
    float a0[S], a1[S];
    load_vd<F>(vb + (uint64_t)r.v[0] * S, a0);
    load_vd<F>(vb + (uint64_t)r.v[1] * S, a1);
    if (s.prim != EUC_PRIM_TRIANGLE_LIST) {
        const float frac = ((r.flags & kLineUseX) ? xf - r.o[0] : yf - r.o[1]) * r.o[2];
#pragma unroll
        for (int i = 0; i < F::NV; ++i) out[i] = a0[i] * (1.0f - frac) + a1[i] * frac;
        return;
    }
    float a2[S];
    load_vd<F>(vb + (uint64_t)r.v[2] * S, a2);
    get_v_data<F>(r, a0, a1, a2, xf, yf, out);
}

// Decodes a visibility key; false when no fragment passed at this pixel.
EUC_DEV bool decode_key(const SceneDev &s, unsigned long long key, uint32_t &t, float &z) {
    if (s.keytype == KEY_MIN) {
        const uint32_t low = (uint32_t)key;
        if (low == 0) return false;
        t = (low >> 1) - 1u;
        uint32_t o = (uint32_t)(key >> 32);
        if (s.depth_test == EUC_TEST_GREATER) o = ~o;
        z = (low & 1u) ? -0.0f : unord_f32(o);
        return true;
    }
    if (key == ~0ull) return false;
    t = ~(uint32_t)(key >> 32);
    z = __uint_as_float((uint32_t)key);
    return true;
}

template <class F>
EUC_DEV void store_pixel(const SceneDev &s, uint32_t x, uint32_t y, const float *frag) {
    const float c0 = frag[0], c1 = F::NF > 1 ? frag[F::NF > 1 ? 1 : 0] : 0.0f;
    const float c2 = F::NF > 2 ? frag[F::NF > 2 ? 2 : 0] : 0.0f, c3 = F::NF > 3 ? frag[F::NF > 3 ? 3 : 0] : 0.0f;
    uint8_t *p = s.pixel + (uint64_t)y * s.ppitch;
    if (s.pfmt == EUC_FMT_RGBA32F) {  // the fragment as it is (no pack)
        float *q = reinterpret_cast<float *>(p) + 4ull * x;
        q[0] = c0;
        q[1] = c1;
        q[2] = c2;
        q[3] = c3;
        return;
    }
    const uint32_t r8 = sat_u8(F::pack(c0)), g8 = sat_u8(F::pack(c1)), b8 = sat_u8(F::pack(c2)), a8 = sat_u8(F::pack(c3));
    if (s.pfmt == EUC_FMT_RGBA8) {
        reinterpret_cast<uint32_t *>(p)[x] = r8 | (g8 << 8) | (b8 << 16) | (a8 << 24);
    } else if (s.pfmt == EUC_FMT_BGRA8) {
        reinterpret_cast<uint32_t *>(p)[x] = b8 | (g8 << 8) | (r8 << 16) | (a8 << 24);
    } else {  // RGB8: two stores, the 2-byte one on its even address
        p += 3ull * x;
        if (((uintptr_t)p & 1u) == 0) {
            *reinterpret_cast<uint16_t *>(p) = (uint16_t)(r8 | (g8 << 8));
            p[2] = (uint8_t)b8;
        } else {
            p[0] = (uint8_t)r8;
            *reinterpret_cast<uint16_t *>(p + 1) = (uint16_t)(g8 | (b8 << 8));
        }
    }
}

// Level-1 MSAA scenes are resolved by warps of 16x2 pixels that cover whole
// 2x2 cells of the band-relative coarse grid: row pair p = b * ppb + k is rows
// b*gr + 2k and b*gr + 2k + 1 of band b (a band of odd height ends with a
// single row), ppb = ceil(gr / 2).
__host__ __device__ inline uint32_t pair_of_row(uint32_t y, uint32_t gr) {
    return (y / gr) * ((gr + 1) >> 1) + ((y % gr) >> 1);
}

__host__ __device__ inline bool resolve_by_quads(const SceneDev &s) {
    return s.level == 1 && s.pixel_write && s.keytype != KEY_ORDERED;
}

// Shaders cheap enough to be evaluated where their pixel is (no job list).
constexpr uint32_t kDirectShaders = (FlatFn::kDirect ? 1u << EUC_SHADER_FLAT : 0u) |
                                    (VColorFn::kDirect ? 1u << EUC_SHADER_VCOLOR : 0u) |
                                    (GouraudFn::kDirect ? 1u << EUC_SHADER_GOURAUD : 0u) |
                                    (TexturedFn::kDirect ? 1u << EUC_SHADER_TEXTURED : 0u) |
                                    (PhongFn::kDirect ? 1u << EUC_SHADER_PHONG : 0u) |
                                    (ShadowFn::kDirect ? 1u << EUC_SHADER_SHADOW : 0u);

// Scenes resolved kDirectPer pixels per thread with no shared memory: depth
// only, or a cheap shader without MSAA.
constexpr int kDirectPer = 4;
__host__ __device__ inline bool resolve_direct(const SceneDev &s) {
    return s.keytype != KEY_ORDERED &&
           (!s.pixel_write || (s.level == 0 && ((kDirectShaders >> s.shader) & 1u)));
}

// k_resolve chunks (blocks of work) of a scene: kBlock pixels of the covered
// rectangle, or kBlock/32 warp tiles of 16x2 pixels over the row pairs and
// 16-pixel columns that meet it.
__host__ __device__ inline uint64_t resolve_chunks(const SceneDev &s, const uint4 &cv) {
    const uint64_t area = rect_area(cv);
    if (area == 0) return 0;
    if (resolve_direct(s)) return (area + kBlock * kDirectPer - 1) / (kBlock * kDirectPer);
    if (resolve_by_quads(s)) {
        const uint64_t pairs = pair_of_row(~cv.w - 1, s.gr) - pair_of_row(cv.y, s.gr) + 1;
        const uint64_t cols = ((~cv.z - 1) >> 4) - (cv.x >> 4) + 1;
        return (pairs * cols + kBlock / 32 - 1) / (kBlock / 32);
    }
    return (area + kBlock - 1) / kBlock;
}

// Upper bound of resolve_chunks over every rectangle (the whole target), for
// sizing launches on the host.
__host__ __device__ inline uint64_t resolve_blocks(const SceneDev &s) {
    uint4 full;
    full.x = 0;
    full.y = 0;
    full.z = ~s.W;
    full.w = ~s.H;
    return resolve_chunks(s, full);
}

// Chunk bases of k_init and k_resolve per scene, from the covered rectangles
// (exclusive prefix sums, nsc + 1 entries each).  One block, any nsc.
EUC_DEV void plan_chunks(const SceneDev *__restrict__ sc, int nsc, const uint4 *__restrict__ cov,
                         uint64_t *__restrict__ ibase, uint64_t *__restrict__ rbase) {
    __shared__ uint64_t s_a[kBlock / 32 + 1];
    uint64_t ci = 0, cr = 0;
    for (int s0 = 0; s0 < nsc; s0 += kBlock) {
        const int si = s0 + (int)threadIdx.x;
        uint64_t ni = 0, nr = 0;
        if (si < nsc) {
            const SceneDev &s = sc[si];
            const uint4 cv = cov[si];
            if (s.keytype == KEY_ORDERED) {  // every entry; k_resolve_ordered sizes itself
                const uint64_t lim = ((uint64_t)s.W * s.H + kBlock - 1) / kBlock * kBlock;
                ni = (lim + kInitChunk - 1) / kInitChunk;
            } else {
                ni = (rect_area(cv) + kInitChunk - 1) / kInitChunk;
                nr = resolve_chunks(s, cv);
            }
        }
        uint64_t ti, tr;
        const uint64_t ei = block_excl_scan<uint64_t>(ni, s_a, &ti);
        const uint64_t er = block_excl_scan<uint64_t>(nr, s_a, &tr);
        if (si < nsc) {
            ibase[si] = ci + ei;
            rbase[si] = cr + er;
        }
        ci += ti;
        cr += tr;
    }
    if (threadIdx.x == 0) {
        ibase[nsc] = ci;
        rbase[nsc] = cr;
    }
}

// Exclusive scans of the strips' entry counts into their list offsets, and
// of their units (ceil(count / kStripUnit)) into unit offsets (nstrips + 1
// entries each), and the strip of every unit.  Block b covers strips
// [b*kScanBlock, (b+1)*kScanBlock) and sums the strips before them itself.
EUC_DEV void strip_scan_block(uint32_t b, const uint32_t *__restrict__ cnt, uint32_t nstrips,
                              uint32_t *__restrict__ off, uint32_t *__restrict__ uoff,
                              uint32_t *__restrict__ unit_strip) {
    __shared__ uint32_t s_a[kBlock / 32 + 1];
    __shared__ uint32_t s_pre[2];
    const uint64_t g0 = (uint64_t)b * kScanBlock;
    uint32_t pre = 0, preu = 0;
    for (uint64_t j = threadIdx.x; j < g0; j += kBlock) {
        pre += cnt[j];
        preu += (cnt[j] + kStripUnit - 1) / kStripUnit;
    }
    uint32_t tp, tu;
    block_excl_scan<uint32_t>(pre, s_a, &tp);
    block_excl_scan<uint32_t>(preu, s_a, &tu);
    if (threadIdx.x == 0) {
        s_pre[0] = tp;
        s_pre[1] = tu;
    }
    __syncthreads();
    const uint64_t q0 = g0 + (uint64_t)threadIdx.x * kScanPer;
    uint32_t c[kScanPer], mine = 0, mineu = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        c[k] = q0 + k < nstrips ? cnt[q0 + k] : 0u;
        mine += c[k];
        mineu += (c[k] + kStripUnit - 1) / kStripUnit;
    }
    uint32_t bt, btu;
    uint32_t o = s_pre[0] + block_excl_scan<uint32_t>(mine, s_a, &bt);
    uint32_t ou = s_pre[1] + block_excl_scan<uint32_t>(mineu, s_a, &btu);
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        const uint32_t nu = (c[k] + kStripUnit - 1) / kStripUnit;
        if (q0 + k < nstrips) {
            off[q0 + k] = o;
            uoff[q0 + k] = ou;
            for (uint32_t u = 0; u < nu; ++u) unit_strip[ou + u] = (uint32_t)(q0 + k);
        }
        o += c[k];
        ou += nu;
    }
    if (g0 + kScanBlock >= nstrips && threadIdx.x == kBlock - 1) {
        off[nstrips] = s_pre[0] + bt;
        uoff[nstrips] = s_pre[1] + btu;
    }
}

// The scan of the setup's row counts (blocks 0 .. nscan - 1, scan_block), the
// chunk plan of init / resolve (block nscan, plan_chunks) and the scans of
// the strips (the blocks after, strip_scan_block): independent work after
// k_setup, in one launch.
__global__ void __launch_bounds__(kBlock) k_scan_plan(const uint32_t *__restrict__ rows,
                                                      const uint2 *__restrict__ chunk_sums, uint64_t ntri,
                                                      uint32_t *__restrict__ live_tri,
                                                      uint64_t *__restrict__ live_rowoff,
                                                      unsigned long long *__restrict__ totals, uint32_t nscan,
                                                      const SceneDev *__restrict__ sc, int nsc,
                                                      const uint4 *__restrict__ cov, uint64_t *__restrict__ ibase,
                                                      uint64_t *__restrict__ rbase, const uint32_t *__restrict__ strip_cnt,
                                                      uint32_t nstrips, uint32_t *__restrict__ strip_off,
                                                      uint32_t *__restrict__ strip_uoff, uint32_t *__restrict__ unit_strip) {
    if (blockIdx.x == nscan) plan_chunks(sc, nsc, cov, ibase, rbase);
    else if (blockIdx.x > nscan)
        strip_scan_block(blockIdx.x - nscan - 1, strip_cnt, nstrips, strip_off, strip_uoff, unit_strip);
    else scan_block(rows, chunk_sums, ntri, live_tri, live_rowoff, totals, nscan);
}

// The clears of prep_clear as a launch of their own (n threads).
__global__ void __launch_bounds__(kBlock) k_prep(const PrepArgs prep) {
    const uint64_t i = (uint64_t)blockIdx.x * kBlock + threadIdx.x;
    if (i < prep.n) prep_clear(prep, i);
}

// The per-scene part of chunk_pixel's mapping (what it divides by the band
// height), computed when a block's chunks reach a new scene.
struct ChunkGeom {
    bool quads;                  // resolve_by_quads: 16x2-pixel tiles
    uint32_t p0, a0, cols, ppb;  // first row pair and tile column, tile columns, row pairs per band
    uint64_t ntiles;             // tiles of the covered rectangle
};

// One warp's job list in k_resolve: its 32 pixels' winners and positions,
// their fragment evaluations and the results.
template <class F>
struct ResolveSmem {
    ChunkGeom geo;  // of the warp's current scene (kept here, not in registers)
    uint32_t t[32];
    uint32_t xy[32][3];
    uint16_t job[4 * 32];
    float frag[32][4][F::NF];
};

// Chunk `lb` of a resolve_direct scene: kBlock * kDirectPer pixels of the
// covered rectangle, each thread taking kDirectPer of them kBlock apart (the
// key loads of a thread are in flight together).
template <class F>
EUC_DEV void resolve_direct_chunk(const SceneDev &s, const uint4 &cv, uint64_t lb, const TriRec *__restrict__ recs,
                                  const float *__restrict__ vdata, const unsigned long long *__restrict__ vbuf) {
    const uint32_t area = (uint32_t)rect_area(cv);  // pixel indices fit 32 bits
    const uint32_t i0 = (uint32_t)lb * (kBlock * kDirectPer) + threadIdx.x;
    RectWalk rk(i0, ~cv.z - cv.x);
    uint32_t px[kDirectPer], py[kDirectPer];
    unsigned long long key[kDirectPer];
#pragma unroll
    for (int k = 0; k < kDirectPer; ++k, rk.next()) {
        const uint32_t i = i0 + k * kBlock;
        px[k] = cv.x + rk.rx;
        py[k] = i < area ? cv.y + rk.ry : 0xFFFFFFFFu;
        key[k] = i < area ? vbuf[s.pix_base + (uint64_t)py[k] * s.W + px[k]] : 0ull;
    }
    // unrolled: the record and varyings gathers of the pixels overlap
#pragma unroll
    for (int k = 0; k < kDirectPer; ++k) {
        uint32_t t;
        float z;
        if (py[k] == 0xFFFFFFFFu || !decode_key(s, key[k], t, z)) continue;
        const uint32_t x = px[k], y = py[k];
        if (s.depth_write) *reinterpret_cast<float *>(s.depth + (uint64_t)y * s.dpitch + 4ull * x) = z;
        if (!s.pixel_write) continue;
        if constexpr (F::kDirect) {
            const typename F::U &u = *reinterpret_cast<const typename F::U *>(s.uniforms);
            const float *vb = vdata + (s.geom ? s.gvd_base : s.vd_base);
            const TriRec r = load_rec(recs + t, s.prim == EUC_PRIM_TRIANGLE_LIST ? kRecShade : kRecAll);
            float vd[F::NV], frag[F::NF];
            vdata_at<F>(s, r, vb, (float)x, (float)y, vd);
            F::fragment(u, vd, frag);
            store_pixel<F>(s, x, y, frag);
        }
    }
}

// This thread's pixel in chunk lb of a scene's covered rectangle (which is
// not empty, or the scene would have no chunks) and the first row of its band.
EUC_DEV ChunkGeom chunk_geom(const SceneDev &s, const uint4 &cv) {
    ChunkGeom g;
    g.quads = resolve_by_quads(s);
    g.ppb = (s.gr + 1) >> 1;
    g.a0 = cv.x >> 4;
    g.cols = ((~cv.z - 1) >> 4) - g.a0 + 1;
    g.p0 = g.quads ? pair_of_row(cv.y, s.gr) : 0u;
    g.ntiles = g.quads ? (uint64_t)(pair_of_row(~cv.w - 1, s.gr) - g.p0 + 1) * g.cols : 0ull;
    return g;
}

EUC_DEV bool chunk_pixel(const SceneDev &s, const uint4 &cv, const ChunkGeom &g, uint64_t lb, uint32_t &x,
                         uint32_t &y, uint32_t &lo) {
    const int tid = threadIdx.x, lane = tid & 31;
    x = y = lo = 0;
    if (g.quads) {  // warp = 16x2 pixels on whole 2x2 cells of the band-relative grid
        const uint64_t w64 = lb * (kBlock / 32) + (tid >> 5);
        if (w64 >= g.ntiles) return false;
        // a scene has fewer than 2^32 / 32 tiles (its pixel indices fit 32
        // bits): a 32-bit division, not a 64-bit one
        const uint32_t w = (uint32_t)w64, wr = w / g.cols;
        const uint32_t p = g.p0 + wr, a = g.a0 + (w - wr * g.cols);
        const uint32_t b = p / g.ppb, k = p - b * g.ppb;
        lo = b * s.gr;
        x = a * 16 + (lane & 15);
        y = lo + 2 * k + (lane >> 4);
        return x < s.W && y < min(lo + s.gr, s.H) && covered(cv, x, y);
    }
    const uint32_t rw = ~cv.z - cv.x;
    const uint32_t i = (uint32_t)lb * kBlock + tid;  // pixel indices fit 32 bits (plan_scene)
    if (i >= (uint32_t)rect_area(cv)) return false;
    const uint32_t ry = i / rw;
    y = cv.y + ry;
    x = cv.x + (i - ry * rw);
    lo = (y / s.gr) * s.gr;
    return true;
}

// One 256-pixel chunk `lb` of scene `s`; every thread of the block calls it.
template <class F>
EUC_DEV void resolve_chunk(const SceneDev &s, const uint4 &cv, const ChunkGeom &geo, uint64_t lb,
                           const TriRec *__restrict__ recs,
                           const float *__restrict__ vdata, const unsigned long long *__restrict__ vbuf,
                           ResolveSmem<F> &sm) {
    const int lane = threadIdx.x & 31;
    // 1. this thread's pixel
    uint32_t x, y, lo;
    const bool quads = geo.quads;
    const bool inside = chunk_pixel(s, cv, geo, lb, x, y, lo);
    uint32_t t = 0xFFFFFFFFu;
    float z = 0.0f;
    const bool win = inside && decode_key(s, vbuf[s.pix_base + (uint64_t)y * s.W + x], t, z);
    if (win && s.depth_write) *reinterpret_cast<float *>(s.depth + (uint64_t)y * s.dpitch + 4ull * x) = z;
    if (!s.pixel_write) return;  // uniform over the block (one scene)

    // 2. the fragment evaluations this chunk needs, compacted into a job list.
    // A job is (pixel slot, corner); corner 0 is the pixel itself when there
    // is no MSAA.  With level-1 MSAA each pixel shades the corner of its 2x2
    // cell at its own offset and reuses the other three from the cell's other
    // pixels when they have the same winner.  A coarse fragment is a pure
    // function of (primitive, grid point), so sharing changes no bits (euc's
    // own coarse cache, pipeline.rs:477-494, is transparent the same way).
    uint32_t *s_t = sm.t;
    uint32_t(*s_xy)[3] = sm.xy;
    uint16_t *s_job = sm.job;
    float(*s_frag)[4][F::NF] = sm.frag;
    const uint32_t tw = win ? t : 0xFFFFFFFFu;
    if (!__any_sync(0xFFFFFFFFu, win)) return;  // nothing to shade in this warp's pixels
    s_t[lane] = tw;
    s_xy[lane][0] = x;
    s_xy[lane][1] = y;
    s_xy[lane][2] = lo;
    const int own_c = (lane & 1) | ((lane >> 4) << 1);
    // the winners of this pixel's 2x2 cell: a cell never leaves its warp's 16x2 tile
    uint32_t nb[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) nb[c] = __shfl_sync(0xFFFFFFFFu, tw, (lane & ~17) | (c & 1) | ((c >> 1) << 4));
    uint32_t need = 0;  // bit c: this pixel evaluates corner c itself
    if (win) {
        if (s.level == 0) {
            need = 1u;
        } else if (quads) {
#pragma unroll
            for (int c = 0; c < 4; ++c)
                if (c == own_c || nb[c] != t) need |= 1u << c;
        } else {
            need = 0xFu;
        }
    }
    // the warp's job list
    const uint32_t cnt = __popc(need), inc = warp_incl_scan(cnt);
    uint32_t off = inc - cnt;
    const uint32_t njobs = __shfl_sync(0xFFFFFFFFu, inc, 31);
#pragma unroll
    for (int c = 0; c < 4; ++c)
        if (need & (1u << c)) s_job[off++] = (uint16_t)((lane << 2) | c);
    __syncwarp();

    // 3. every thread evaluates jobs until the list is done
    const typename F::U &u = *reinterpret_cast<const typename F::U *>(s.uniforms);
    const float *vb = vdata + (s.geom ? s.gvd_base : s.vd_base);
    const uint32_t L = s.level;
    for (uint32_t j = lane; j < njobs; j += 32) {
        const int slot = s_job[j] >> 2, c = s_job[j] & 3;
        const TriRec &r = recs[s_t[slot]];  // (field loads here: the vector copy costs this path registers)
        float xf, yf;
        if (L == 0) {
            xf = (float)s_xy[slot][0];
            yf = (float)s_xy[slot][1];
        } else {
            const uint32_t sx = s_xy[slot][0], sy = s_xy[slot][1], slo = s_xy[slot][2];
            xf = (float)(((sx >> L) + (uint32_t)(c & 1)) << L);
            yf = (float)(slo + ((((sy - slo) >> L) + (uint32_t)(c >> 1)) << L));
        }
        float vd[F::NV];
        vdata_at<F>(s, r, vb, xf, yf, vd);
        F::fragment(u, vd, s_frag[slot][c]);
    }
    __syncwarp();

    // 4. combine (pipeline.rs:541-573) and store
    if (!win) return;
    float frag[F::NF];
    if (L == 0) {
#pragma unroll
        for (int i = 0; i < F::NF; ++i) frag[i] = s_frag[lane][0][i];
    } else {
        int src[4];
#pragma unroll
        for (int c = 0; c < 4; ++c)
            src[c] = (need & (1u << c)) ? lane : ((lane & ~17) | (c & 1) | ((c >> 1) << 4));
        const float div = 1.0f / (float)(1u << L);
        const float fx = rfract((float)x * div);
        const float fy = rfract((float)(y - lo) * div);
#pragma unroll
        for (int i = 0; i < F::NF; ++i) {
            const float a0 = s_frag[src[0]][0][i] * (1.0f - fy) + s_frag[src[2]][2][i] * fy;
            const float a1 = s_frag[src[1]][1][i] * (1.0f - fy) + s_frag[src[3]][3][i] * fy;
            frag[i] = a0 * (1.0f - fx) + a1 * fx;
        }
    }
    store_pixel<F>(s, x, y, frag);
}

// Blocks walk groups of `group` chunks (grid-strided) of the scenes
// [s_begin, s_end); rbase (global scene index, from plan_chunks) holds the first
// chunk of each.
template <class F>
__global__ void __launch_bounds__(kBlock, F::kResolveBlocks) k_resolve(const SceneDev *__restrict__ sc,
                                                                    const uint64_t *__restrict__ rbase,
                                                    int s_begin, int s_end, uint32_t group,
                                                    const TriRec *__restrict__ recs, const float *__restrict__ vdata,
                                                    const unsigned long long *__restrict__ vbuf,
                                                    const uint4 *__restrict__ cov) {
    // warps work independently: each has its own job list and no block barrier
    __shared__ ResolveSmem<F> s_warp[kBlock / 32];
    ResolveSmem<F> &sm = s_warp[threadIdx.x >> 5];
    const uint64_t *base = rbase + s_begin;
    const int n = s_end - s_begin;
    const uint64_t c_begin = base[0], c_end = base[n];
    for (uint64_t g = blockIdx.x; c_begin + g * group < c_end; g += gridDim.x) {
        const uint64_t c0 = c_begin + g * group;
        int si = find_scene(base, n, c0), gsi = -1;
        const ChunkGeom &geo = sm.geo;
        for (uint64_t c = c0; c < c0 + group && c < c_end; ++c) {
            si = advance_scene(base, n, si, c);
            const SceneDev &s = sc[s_begin + si];
            if (resolve_direct(s)) {  // uniform: one scene per chunk
                resolve_direct_chunk<F>(s, cov[s_begin + si], c - base[si], recs, vdata, vbuf);
            } else {
                const uint4 cv = cov[s_begin + si];
                if (si != gsi) {  // the block's chunks reached a new scene
                    if ((threadIdx.x & 31) == 0) sm.geo = chunk_geom(s, cv);
                    __syncwarp();
                    gsi = si;
                }
                // the keys of this block's next chunk in the same scene start
                // on their way to L2 (the keys of a large batch outgrow it)
                const uint64_t nc = c + 1 < c0 + group ? c + 1 : c_begin + (g + gridDim.x) * group;
                if (nc < base[si + 1]) {
                    uint32_t px, py, plo;
                    if (chunk_pixel(s, cv, geo, nc - base[si], px, py, plo))
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(vbuf + s.pix_base + (uint64_t)py * s.W + px));
                }
                resolve_chunk<F>(s, cv, geo, c - base[si], recs, vdata, vbuf, sm);
                __syncwarp();  // the next chunk reuses the warp's shared memory
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Host-buffer renders on a device that reads pageable host memory: blocks
// take pieces of the regions in turn; 16-byte words with four loads in
// flight per thread (the link's latency is microseconds), 4-byte or
// single-byte words where a piece's ends are not aligned that far.
// ---------------------------------------------------------------------------
struct CopyPiece {
    const uint8_t *src;
    uint8_t *dst;
    uint64_t bytes;
};

EUC_DEV void copy_piece(const CopyPiece &p) {
    const uint64_t n = p.bytes;
    const uintptr_t al = (uintptr_t)p.src | (uintptr_t)p.dst | (uintptr_t)n;
    if ((al & 15) == 0) {
        const uint4 *s = (const uint4 *)p.src;
        uint4 *d = (uint4 *)p.dst;
        const uint64_t n16 = n / 16;
        uint64_t i = threadIdx.x;
        for (; i + 3 * kBlock < n16; i += 4 * kBlock) {
            const uint4 a = s[i], b = s[i + kBlock], c = s[i + 2 * kBlock], e = s[i + 3 * kBlock];
            d[i] = a;
            d[i + kBlock] = b;
            d[i + 2 * kBlock] = c;
            d[i + 3 * kBlock] = e;
        }
        for (; i < n16; i += kBlock) d[i] = s[i];
    } else if ((al & 3) == 0) {
        const uint32_t *s = (const uint32_t *)p.src;
        uint32_t *d = (uint32_t *)p.dst;
        for (uint64_t i = threadIdx.x; i < n / 4; i += kBlock) d[i] = s[i];
    } else {
        for (uint64_t i = threadIdx.x; i < n; i += kBlock) p.dst[i] = p.src[i];
    }
}

__global__ void __launch_bounds__(kBlock) k_copy_pieces(const CopyPiece *__restrict__ pieces, uint32_t npieces) {
    for (uint32_t i = blockIdx.x; i < npieces; i += gridDim.x) copy_piece(pieces[i]);
}

// ---------------------------------------------------------------------------
// Texture ingest: one thread per texel, image-crate layouts -> sampler layouts.
// ---------------------------------------------------------------------------
__host__ __device__ inline uint32_t src_bpp(uint32_t f) {
    switch (f) {
    case EUC_SRC_RGBA8: case EUC_SRC_BGRA8: case EUC_SRC_R32F: return 4;
    case EUC_SRC_RGB8: return 3;
    case EUC_SRC_LUMA8: return 1;
    default: return 2;  // EUC_SRC_LUMA_ALPHA8
    }
}

// Block (32, 8): x runs along a row; blocks stride the rows.
__global__ void __launch_bounds__(256) k_ingest(const uint8_t *__restrict__ src, uint64_t spitch, uint32_t fmt,
                                                uint8_t *__restrict__ dst, uint64_t dpitch, uint32_t W, uint32_t H) {
    const uint32_t x = blockIdx.x * 32 + threadIdx.x;
    if (x >= W) return;
    const uint32_t bpp = src_bpp(fmt);
    for (uint32_t y = blockIdx.y * 8 + threadIdx.y; y < H; y += gridDim.y * 8) {
        const uint8_t *p = src + (uint64_t)y * spitch + (uint64_t)x * bpp;
        uint32_t *q = reinterpret_cast<uint32_t *>(dst + (uint64_t)y * dpitch) + x;
        uint32_t r, g, b, a;
        switch (fmt) {
        case EUC_SRC_R32F: *q = *reinterpret_cast<const uint32_t *>(p); continue;  // f32 bits as they are
        case EUC_SRC_RGBA8: r = p[0]; g = p[1]; b = p[2]; a = p[3]; break;
        case EUC_SRC_BGRA8: r = p[2]; g = p[1]; b = p[0]; a = p[3]; break;
        case EUC_SRC_RGB8: r = p[0]; g = p[1]; b = p[2]; a = 255; break;
        case EUC_SRC_LUMA8: r = g = b = p[0]; a = 255; break;
        default: r = g = b = p[0]; a = p[1]; break;  // luma + alpha
        }
        *q = r | (g << 8) | (b << 16) | (a << 24);
    }
}

// ---------------------------------------------------------------------------
// N-dimensional nearest sampling: Nearest::sample (sampler/nearest.rs:27-33)
// after the wrap of sampler/mod.rs:100-179, Denormalize per axis
// (math.rs:40-60) and Buffer<T, N>'s linear index (buffer.rs:85-100, axis 0
// fastest).  One thread per query; texels are copied byte for byte.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_sample_nearest(const uint8_t *__restrict__ tex, uint32_t ndim, uint4 size,
                                                           uint32_t tb, uint32_t wrap, const float *__restrict__ q,
                                                           uint64_t count, uint8_t *__restrict__ out) {
    const uint32_t sz[4] = {size.x, size.y, size.z, size.w};
    for (uint64_t i = (uint64_t)blockIdx.x * kBlock + threadIdx.x; i < count; i += (uint64_t)gridDim.x * kBlock) {
        uint64_t lin = 0, factor = 1;
        for (uint32_t a = 0; a < ndim; ++a) {
            const float e = wrap_coord(wrap, q[i * ndim + a]);
            uint32_t idx = sat_u32(rmax(e * (float)sz[a], 0.0f));  // `(e * s as f32).max(0.0) as usize`
            idx = idx < sz[a] - 1u ? idx : sz[a] - 1u;             // `.min(s - 1)`
            lin += (uint64_t)idx * factor;
            factor *= sz[a];
        }
        const uint8_t *src = tex + lin * tb;
        uint8_t *dst = out + i * tb;
        for (uint32_t b = 0; b < tb; ++b) dst[b] = src[b];
    }
}

// ---------------------------------------------------------------------------
// Ordered path (KEY_ORDERED): per-pixel fragment lists replayed in order.
// ---------------------------------------------------------------------------
constexpr int kOScanPer = 8;
constexpr int kOScanBlock = kBlock * kOScanPer;

// Sum of the per-pixel candidate counts (low words of vbuf) of each block of
// kOScanBlock entries in [p0, p1).
__global__ void __launch_bounds__(kBlock) k_oscan_reduce(const unsigned long long *__restrict__ vbuf, uint64_t p0,
                                                         uint64_t p1, unsigned long long *__restrict__ bsum) {
    __shared__ unsigned long long s_a[kBlock / 32 + 1];
    const uint64_t q0 = p0 + (uint64_t)blockIdx.x * kOScanBlock + (uint64_t)threadIdx.x * kOScanPer;
    unsigned long long v = 0;
#pragma unroll
    for (int k = 0; k < kOScanPer; ++k)
        if (q0 + k < p1) v += (uint32_t)vbuf[q0 + k];
    unsigned long long tot;
    block_excl_scan<unsigned long long>(v, s_a, &tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

// Exclusive scan of the counts: the low word of each entry becomes the offset
// of its pixel's list, the high word (the fill cursor) 0.  total[0] = number
// of fragments.
__global__ void __launch_bounds__(kBlock) k_oscan_apply(unsigned long long *__restrict__ vbuf, uint64_t p0, uint64_t p1,
                                                        const unsigned long long *__restrict__ bsum,
                                                        unsigned long long *__restrict__ total) {
    __shared__ unsigned long long s_a[kBlock / 32 + 1];
    __shared__ unsigned long long s_pre;
    unsigned long long pre = 0;
    for (uint64_t j = threadIdx.x; j < blockIdx.x; j += kBlock) pre += bsum[j];
    unsigned long long tp;
    block_excl_scan<unsigned long long>(pre, s_a, &tp);
    if (threadIdx.x == 0) s_pre = tp;
    __syncthreads();
    const uint64_t q0 = p0 + (uint64_t)blockIdx.x * kOScanBlock + (uint64_t)threadIdx.x * kOScanPer;
    uint32_t c[kOScanPer];
    unsigned long long mine = 0;
#pragma unroll
    for (int k = 0; k < kOScanPer; ++k) {
        c[k] = q0 + k < p1 ? (uint32_t)vbuf[q0 + k] : 0u;
        mine += c[k];
    }
    unsigned long long bt;
    unsigned long long o = s_pre + block_excl_scan<unsigned long long>(mine, s_a, &bt);
#pragma unroll
    for (int k = 0; k < kOScanPer; ++k) {
        if (q0 + k < p1) vbuf[q0 + k] = (unsigned long long)(uint32_t)o;  // offsets beyond 2^32 are refused by the host
        o += c[k];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == kBlock - 1) total[0] = s_pre + bt;
}

// Fragment of primitive `r` at pixel (x, y): plain or coarse-grid MSAA.
template <class F>
EUC_DEV void shade_at(const SceneDev &s, const typename F::U &u, const TriRec &r, const float *__restrict__ vb,
                      uint32_t x, uint32_t y, float *frag) {
    float vd[F::NV];
    if (s.level == 0) {
        vdata_at<F>(s, r, vb, (float)x, (float)y, vd);
        F::fragment(u, vd, frag);
        return;
    }
    const uint32_t L = s.level, lo = (y / s.gr) * s.gr;  // pipeline.rs:541-573
    const float div = 1.0f / (float)(1u << L);
    const float fx = rfract((float)x * div), fy = rfract((float)(y - lo) * div);
    const uint32_t px = x >> L, py = (y - lo) >> L;
    float t[4][F::NF];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        vdata_at<F>(s, r, vb, (float)((px + (uint32_t)(c & 1)) << L), (float)(lo + ((py + (uint32_t)(c >> 1)) << L)),
                    vd);
        F::fragment(u, vd, t[c]);
    }
#pragma unroll
    for (int i = 0; i < F::NF; ++i) {
        const float a0 = t[0][i] * (1.0f - fy) + t[2][i] * fy;
        const float a1 = t[1][i] * (1.0f - fy) + t[3][i] * fy;
        frag[i] = a0 * (1.0f - fx) + a1 * fx;
    }
}

// Replays each pixel's fragments in submission order with euc's sequential
// depth test (pipeline.rs:519-526) and blend-into-the-current-pixel
// (pipeline.rs:574-576).  Lists are short in practice; the next fragment is
// found by a linear scan for the smallest primitive id above the last one.
template <class F>
__global__ void __launch_bounds__(kBlock) k_resolve_ordered(const SceneDev *__restrict__ sc,
                                                            const uint64_t *__restrict__ res_base, int s_begin,
                                                            int s_end, uint64_t blk_begin,
                                                            const TriRec *__restrict__ recs,
                                                            const float *__restrict__ vdata,
                                                            const unsigned long long *__restrict__ vbuf,
                                                            const uint2 *__restrict__ frags,
                                                            const uint4 *__restrict__ cov) {
    __shared__ int s_scene;
    const uint64_t blk = blk_begin + blockIdx.x;
    if (threadIdx.x == 0) s_scene = s_begin + find_scene(res_base + s_begin, s_end - s_begin, blk);
    __syncthreads();
    const SceneDev &s = sc[s_scene];
    const uint64_t q = (blk - res_base[s_scene]) * kBlock + threadIdx.x;
    if (q >= (uint64_t)s.W * s.H) return;
    const uint32_t y = (uint32_t)q / s.W, x = (uint32_t)q - y * s.W;
    if (!covered(cov[s_scene], x, y)) return;
    const unsigned long long e = vbuf[s.pix_base + q];
    const uint32_t off = (uint32_t)e, n = (uint32_t)(e >> 32);
    if (n == 0) return;
    float *dp = s.depth ? reinterpret_cast<float *>(s.depth + (uint64_t)y * s.dpitch + 4ull * x) : nullptr;
    const bool f32 = s.pfmt == EUC_FMT_RGBA32F;  // the pixel kept as four floats
    uint8_t *pp = s.pixel ? s.pixel + (uint64_t)y * s.ppitch +
                                (uint64_t)x * (f32 ? 16u : s.pfmt == EUC_FMT_RGB8 ? 3u : 4u)
                          : nullptr;
    const bool uses_depth = s.depth_test != EUC_TEST_NONE || s.depth_write;
    float D = uses_depth ? *dp : 0.0f;
    const int ri = s.pfmt == EUC_FMT_BGRA8 ? 2 : 0, bi = s.pfmt == EUC_FMT_BGRA8 ? 0 : 2;
    const int nch = s.pfmt == EUC_FMT_RGB8 ? 3 : 4;
    uint32_t ch[4] = {0, 0, 0, 255};
    float pf[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (s.pixel_write) {
        if (f32)
            for (int i = 0; i < 4; ++i) pf[i] = reinterpret_cast<const float *>(pp)[i];
        else
            for (int i = 0; i < nch; ++i) ch[i] = pp[i];
    }
    const typename F::U &u = *reinterpret_cast<const typename F::U *>(s.uniforms);
    const float *vb = vdata + (s.geom ? s.gvd_base : s.vd_base);
    uint32_t last = 0;  // 1 + the primitive processed last
    for (uint32_t k = 0; k < n; ++k) {
        uint32_t best = 0xFFFFFFFFu, bz = 0;
        for (uint32_t j = 0; j < n; ++j) {
            const uint2 f = frags[off + j];
            if (f.x + 1u > last && f.x < best) {
                best = f.x;
                bz = f.y;
            }
        }
        last = best + 1u;
        const float z = __uint_as_float(bz);
        bool pass = true;
        if (s.depth_test == EUC_TEST_LESS) pass = z < D;
        else if (s.depth_test == EUC_TEST_EQUAL) pass = z == D;
        else if (s.depth_test == EUC_TEST_GREATER) pass = z > D;
        if (!pass) continue;
        if (s.depth_write) D = z;
        if (!s.pixel_write) continue;
        float frag[F::NF];
        shade_at<F>(s, u, load_rec(recs + best, s.prim == EUC_PRIM_TRIANGLE_LIST ? kRecShade : kRecAll), vb, x, y,
                    frag);
        float c[4] = {frag[0], F::NF > 1 ? frag[F::NF > 1 ? 1 : 0] : 0.0f, F::NF > 2 ? frag[F::NF > 2 ? 2 : 0] : 0.0f,
                      F::NF > 3 ? frag[F::NF > 3 ? 3 : 0] : 0.0f};
        if (s.blend == EUC_BLEND_ALPHA) {  // src-over on the unpacked old pixel
            float old[4];
            if (f32) {
                for (int i = 0; i < 4; ++i) old[i] = pf[i];
            } else {
                old[0] = (float)ch[ri] / 255.0f;
                old[1] = (float)ch[1] / 255.0f;
                old[2] = (float)ch[bi] / 255.0f;
                old[3] = nch == 3 ? 1.0f : (float)ch[3] / 255.0f;
            }
            const float a = c[3];
#pragma unroll
            for (int i = 0; i < 4; ++i) c[i] = c[i] * a + old[i] * (1.0f - a);
        }
        if (f32) {
            for (int i = 0; i < 4; ++i) pf[i] = c[i];
            continue;
        }
        ch[ri] = sat_u8(F::pack(c[0]));
        ch[1] = sat_u8(F::pack(c[1]));
        ch[bi] = sat_u8(F::pack(c[2]));
        if (nch == 4) ch[3] = sat_u8(F::pack(c[3]));
    }
    if (s.depth_write) *dp = D;
    if (s.pixel_write) {
        if (f32)
            for (int i = 0; i < 4; ++i) reinterpret_cast<float *>(pp)[i] = pf[i];
        else
            for (int i = 0; i < nch; ++i) pp[i] = (uint8_t)ch[i];
    }
}

}  // namespace eucg
