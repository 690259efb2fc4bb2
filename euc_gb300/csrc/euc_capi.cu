// euc_capi.cu — host runtime and C ABI of the GB300 triangle pipeline.
//
// A render is a batch of one scene; a batch runs every scene through the same
// six launches (vertex per shader kind, setup, scan, init, raster, resolve per
// shader kind) on one stream.  Scratch buffers live in the context and grow
// on demand (euc_ctx_reserve pre-sizes them).  Scene tables and uniforms go
// up through a ring of pinned staging slots, each guarded by an event.

#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <thread>
#include <map>
#include <atomic>
#include <array>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "euc_kernels.cuh"

using namespace eucg;

namespace {

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
};

constexpr int kStageSlots = 8;

struct StageSlot {
    void *host = nullptr;
    void *dev = nullptr;
    size_t cap = 0;
    cudaEvent_t done = nullptr;
    bool pending = false;
};

}  // namespace

struct euc_ctx {
    int device = 0;
    int nsm = 0;
    DevBuf clip, vdata, recs, rows, chunk_sums, live_tri, live_rowoff, totals, vbuf, err, stats, cov;
    DevBuf obsum, frags;  // ordered path: pixel-scan block sums, fragment lists
    DevBuf plan;          // plan_chunks: k_init and k_resolve chunk bases (2 x (scenes + 1))
    DevBuf galive;        // geometry stage: 1 per output slot that holds a triangle
    // strip path: per-strip entry counts, fill cursors, list offsets, unit
    // offsets, the entry lists and the strip of each unit
    DevBuf strip_cnt, strip_fill, strip_off, strip_uoff, entries, unit_strip;
    DevBuf bbox;  // strip path: each primitive's bbox (16 B), the binning's only read of it
    int raster_blocks = 0;  // resident k_raster blocks per SM
    bool pageable = false;  // kernels may access pageable host memory (cudaDevAttrPageableMemoryAccess)
    euc_tuning tune{};      // launch-shape overrides (0 = default)
    // buffers used by euc_render_host
    DevBuf h_arena;    // host-buffer renders: inputs and targets on the device
    DevBuf h_pinned;   // ... and their page-locked staging (cudaMallocHost)
    DevBuf h_tex[1];   // texture ingest: staged host rows
    StageSlot slots[kStageSlots];
    int next_slot = 0;
    int last_nscenes = 0;
    // profiling: event pairs per stage, pooled
    bool profiling = false;
    bool capturing = false;  // a graph is being recorded: no profiling events
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_marks;
    uint64_t launches = 0;
    // euc_render's recorded shapes (render_one), and how often each shape
    // was seen before it is recorded
    std::vector<struct ShapeGraph *> shapes;
    std::map<std::vector<unsigned char>, int> sightings;
    uint64_t shape_clock = 0;
    std::mutex mu;
};

namespace {

#define CUDA_TRY(x)                                  \
    do {                                             \
        cudaError_t e_ = (x);                        \
        if (e_ != cudaSuccess) {                     \
            (void)cudaGetLastError();                \
            return e_ == cudaErrorMemoryAllocation ? EUC_ERR_OOM : EUC_ERR_CUDA; \
        }                                            \
    } while (0)

int grow(DevBuf &b, size_t bytes) {
    if (bytes <= b.cap) return EUC_OK;
    size_t ncap = std::max(bytes, b.cap + b.cap / 2);
    ncap = (ncap + 255) & ~(size_t)255;
    if (b.p) {
        CUDA_TRY(cudaDeviceSynchronize());
        CUDA_TRY(cudaFree(b.p));
        b.p = nullptr;
        b.cap = 0;
    }
    CUDA_TRY(cudaMalloc(&b.p, ncap));
    b.cap = ncap;
    return EUC_OK;
}

inline uint64_t pad_up(uint64_t v, uint64_t a) { return (v + a - 1) / a * a; }

uint32_t fmt_bpp(uint32_t f) {
    switch (f) {
    case EUC_FMT_RGBA8: case EUC_FMT_BGRA8: case EUC_FMT_R32F: return 4;
    case EUC_FMT_RGB8: return 3;
    case EUC_FMT_RGBA32F: return 16;
    default: return 0;
    }
}

size_t uniforms_size_for(uint32_t shader) {
    switch (shader) {
    case EUC_SHADER_FLAT: return sizeof(euc_flat_uniforms);
    case EUC_SHADER_VCOLOR: return sizeof(euc_vcolor_uniforms);
    case EUC_SHADER_GOURAUD: return sizeof(euc_gouraud_uniforms);
    case EUC_SHADER_TEXTURED: return sizeof(euc_textured_uniforms);
    case EUC_SHADER_PHONG: return sizeof(euc_phong_uniforms);
    case EUC_SHADER_SHADOW: return sizeof(euc_shadow_uniforms);
    default: return 0;
    }
}

int shader_nv(uint32_t shader) {
    switch (shader) {
    case EUC_SHADER_FLAT: return FlatFn::NV;
    case EUC_SHADER_VCOLOR: return VColorFn::NV;
    case EUC_SHADER_GOURAUD: return GouraudFn::NV;
    case EUC_SHADER_TEXTURED: return TexturedFn::NV;
    case EUC_SHADER_PHONG: return PhongFn::NV;
    case EUC_SHADER_SHADOW: return ShadowFn::NV;
    default: return 0;
    }
}

bool attr_ok(int32_t off, uint32_t bytes, uint32_t stride) {
    return off >= 0 && (off & 3) == 0 && (uint32_t)off + bytes <= stride;
}

int check_sampler(const euc_sampler &s) {
    if (!s.data) return EUC_OK;
    // euc's `Texture::linear()` asserts a non-empty texture (texture.rs:63-66).
    if (s.width < 1 || s.height < 1) return EUC_ERR_INVALID;
    if (s.format != EUC_FMT_RGBA8 && s.format != EUC_FMT_R32F) return EUC_ERR_INVALID;
    if (s.filter > EUC_FILTER_LINEAR || s.wrap > EUC_WRAP_MIRROR) return EUC_ERR_INVALID;
    if ((s.pitch & 3) || (s.pitch && s.pitch < s.width * 4)) return EUC_ERR_INVALID;
    if (((uintptr_t)s.data & 3) != 0) return EUC_ERR_INVALID;
    if (s.format == EUC_FMT_RGBA8 && !(s.texel_div > 0.0f)) return EUC_ERR_INVALID;
    return EUC_OK;
}

// Host-side plan of one scene.
struct Plan {
    SceneDev d;
    bool skip;       // nothing observable is drawn
    uint32_t nv;     // VertexData floats
    const void *uniforms;
    size_t usize;
};

// Validates a scene and fills its plan (everything but the batch offsets).
// Mirrors euc's panics: target sizes (pipeline.rs:256-270), band height
// (pipeline.rs:328-330).  Index bounds are checked on the device.
int plan_scene(const euc_scene &sc, Plan &p) {
    std::memset(&p, 0, sizeof(p));
    const euc_pipeline_desc &d = sc.desc;
    if (d.shader >= EUC_SHADER_COUNT) return EUC_ERR_INVALID;
    if (d.depth_test > EUC_TEST_GREATER || d.cull > EUC_CULL_FRONT || d.y_axis > EUC_Y_UP) return EUC_ERR_INVALID;
    if (d.blend > EUC_BLEND_ALPHA || d.primitives > EUC_PRIM_LINE_LIST || d.geometry > EUC_GEOM_DISCARD)
        return EUC_ERR_INVALID;
    if (d.geometry != EUC_GEOM_NONE && d.primitives != EUC_PRIM_TRIANGLE_LIST) return EUC_ERR_INVALID;
    const size_t need = uniforms_size_for(d.shader);
    if (!sc.uniforms || sc.uniforms_size < need) return EUC_ERR_INVALID;
    const euc_vertex_layout &l = sc.layout;
    if (l.stride == 0 || (l.stride & 3)) return EUC_ERR_INVALID;
    if (sc.nverts && (!sc.vertices || ((uintptr_t)sc.vertices & 3))) return EUC_ERR_INVALID;
    if (sc.indices && ((uintptr_t)sc.indices & 3)) return EUC_ERR_INVALID;
    bool ok = true;
    switch (d.shader) {
    case EUC_SHADER_VCOLOR: ok = attr_ok(l.position, 16, l.stride) && attr_ok(l.color, 4, l.stride); break;
    case EUC_SHADER_GOURAUD: ok = attr_ok(l.position, 12, l.stride) && attr_ok(l.normal, 12, l.stride); break;
    case EUC_SHADER_TEXTURED: ok = attr_ok(l.position, 12, l.stride) && attr_ok(l.uv, 8, l.stride); break;
    case EUC_SHADER_PHONG:
        ok = attr_ok(l.position, 12, l.stride) && attr_ok(l.normal, 12, l.stride) && (l.uv < 0 || attr_ok(l.uv, 8, l.stride));
        break;
    default: ok = attr_ok(l.position, 12, l.stride); break;
    }
    if (!ok) return EUC_ERR_INVALID;
    if (d.shader == EUC_SHADER_TEXTURED) {
        const euc_textured_uniforms *u = (const euc_textured_uniforms *)sc.uniforms;
        if (!u->tex.data) return EUC_ERR_INVALID;
        if (int rc = check_sampler(u->tex)) return rc;
    }
    if (d.shader == EUC_SHADER_PHONG) {
        const euc_phong_uniforms *u = (const euc_phong_uniforms *)sc.uniforms;
        if (int rc = check_sampler(u->tex)) return rc;
        if (int rc = check_sampler(u->shadow)) return rc;
    }
    const bool uses_depth = d.depth_test != EUC_TEST_NONE || d.depth_write;
    const euc_target &px = sc.pixel, &dp = sc.depth;
    const bool px_empty = px.data == nullptr, dp_empty = dp.data == nullptr;
    if (!px_empty && d.pixel_write) {
        const uint32_t bpp = fmt_bpp(px.format);
        if (bpp == 0 || px.format == EUC_FMT_R32F) return EUC_ERR_INVALID;
        const uint32_t pitch = px.pitch ? px.pitch : px.width * bpp;
        if (pitch < px.width * bpp) return EUC_ERR_INVALID;
        if (bpp % 4 == 0 && ((pitch & 3) || ((uintptr_t)px.data & 3))) return EUC_ERR_INVALID;
    }
    if (!dp_empty && uses_depth) {
        if (dp.format != EUC_FMT_R32F) return EUC_ERR_INVALID;
        const uint32_t pitch = dp.pitch ? dp.pitch : dp.width * 4;
        if (pitch < dp.width * 4 || (pitch & 3) || ((uintptr_t)dp.data & 3)) return EUC_ERR_INVALID;
    }
    const uint32_t pw = px_empty ? 0 : px.width, ph = px_empty ? 0 : px.height;
    const uint32_t dw = dp_empty ? 0 : dp.width, dh = dp_empty ? 0 : dp.height;
    p.skip = false;
    uint32_t W, H;
    if (!d.pixel_write && !uses_depth) { p.skip = true; return EUC_OK; }  // pipeline.rs:257
    if (d.pixel_write && !uses_depth) { W = pw; H = ph; }
    else if (!d.pixel_write) { W = dw; H = dh; }
    else {
        if (pw != dw || ph != dh) return EUC_ERR_SIZE_MISMATCH;
        W = pw; H = ph;
    }
    const uint32_t level = d.aa_level > 6 ? 6 : d.aa_level;
    uint64_t gr;
    if (d.band_rows == EUC_BANDS_PAR) {
        gr = 20000ull * (1ull << level) / (W > 1 ? W : 1);
        if (gr == 0) return EUC_ERR_BAND;
        if (H / gr == 0) {
            if (d.flags & EUC_FLAG_PAR_EMPTY) { p.skip = true; return EUC_OK; }
            gr = H > 0 ? H : 1;
        }
    } else {
        gr = d.band_rows;
        if (gr > H) gr = H > 0 ? H : 1;
    }
    if (W == 0 || H == 0) { p.skip = true; return EUC_OK; }
    if ((uint64_t)W * H >= 0xFFFFFF00ull) return EUC_ERR_CAPACITY;  // pixel indices are 32-bit on the device
    const uint64_t nstream = sc.indices ? sc.nindices : sc.nverts;
    if (sc.nverts >= 0xFFFFFFFFull || nstream >= 0x3FFFFFFFull) return EUC_ERR_INVALID;
    SceneDev &s = p.d;
    s.verts = (const uint8_t *)sc.vertices;
    s.idx = sc.indices;
    s.pixel = (uint8_t *)px.data;
    s.depth = (uint8_t *)dp.data;
    s.nverts = sc.nverts;
    s.nstream = nstream;
    s.lay = l;
    // primitive slots: one per triangle / line; the index checks of a
    // trailing partial primitive belong to its slot (primitives.rs:18-104)
    s.prim = d.primitives;
    if (d.primitives == EUC_PRIM_TRIANGLE_LIST) {
        s.ntris = (uint32_t)(nstream / 3);
        s.ngroups = (uint32_t)((nstream + 2) / 3);
    } else if (d.primitives == EUC_PRIM_LINE_LIST) {
        s.ntris = (uint32_t)(nstream / 2);
        s.ngroups = (uint32_t)((nstream + 1) / 2);
    } else {  // three lines per complete triangle
        s.ntris = (uint32_t)(3 * (nstream / 3));
        s.ngroups = (uint32_t)(3 * ((nstream + 2) / 3));
    }
    s.geom = d.geometry;
    s.gparam = d.geometry_param;
    if (s.geom != EUC_GEOM_NONE) {  // setup sees the geometry stage's output slots
        s.gratio = geometry_ratio(s.geom);
        s.ntin = (uint32_t)(nstream / 3);
        s.ngin = (uint32_t)((nstream + 2) / 3);
        if ((uint64_t)s.gratio * s.ntin >= 0x3FFFFFFFull) return EUC_ERR_CAPACITY;
        s.ntris = s.ngroups = s.gratio * s.ntin;
    }
    s.W = W;
    s.H = H;
    s.ndc_x = 2.0f / (float)W;
    s.ndc_y = -2.0f / (float)H;
    s.gr = (uint32_t)gr;
    s.level = level;
    s.ppitch = px_empty ? 0 : (px.pitch ? px.pitch : px.width * fmt_bpp(px.format));
    s.dpitch = dp_empty ? 0 : (dp.pitch ? dp.pitch : dp.width * 4);
    s.pfmt = px_empty ? EUC_FMT_NONE : px.format;
    s.pixel_write = d.pixel_write ? 1 : 0;
    s.depth_test = d.depth_test;
    s.depth_write = d.depth_write ? 1 : 0;
    s.yflip = d.y_axis == EUC_Y_UP ? 1 : 0;
    s.zclip = d.z_clip ? 1 : 0;
    s.zmin = d.z_clip_min;
    s.zmax = d.z_clip_max;
    s.cull = d.cull;
    s.blend = d.blend;
    s.shader = d.shader;
    if (!s.pixel_write && !s.depth_write) { p.skip = true; return EUC_OK; }  // nothing is ever written
    if (s.pixel_write && px_empty) s.pixel_write = 0;  // Empty drops writes (texture.rs:315-318)
    s.keytype = (s.depth_write && (d.depth_test == EUC_TEST_LESS || d.depth_test == EUC_TEST_GREATER)) ? KEY_MIN : KEY_LAST;
    // blends that read the old pixel depend on the order of every passing
    // fragment: those scenes (and any with EUC_FLAG_ORDERED) replay per-pixel
    // fragment lists instead of reducing visibility keys
    if ((s.pixel_write && d.blend == EUC_BLEND_ALPHA) || (d.flags & EUC_FLAG_ORDERED)) s.keytype = KEY_ORDERED;
    p.nv = (uint32_t)vd_stride(shader_nv(d.shader));  // padded VertexData floats per vertex
    p.uniforms = sc.uniforms;
    p.usize = need;
    return EUC_OK;
}

}  // namespace

namespace eucg {
// The scene checks of the render path, for the serving loop's submissions.
__attribute__((visibility("hidden"))) int check_scene(const euc_scene *s) {
    Plan p;
    return s ? plan_scene(*s, p) : EUC_ERR_INVALID;
}
}  // namespace eucg

namespace {

int acquire_slot(euc_ctx *ctx, size_t bytes, StageSlot *&out) {
    StageSlot &s = ctx->slots[ctx->next_slot];
    ctx->next_slot = (ctx->next_slot + 1) % kStageSlots;
    if (s.pending) {
        CUDA_TRY(cudaEventSynchronize(s.done));
        s.pending = false;
    }
    if (s.cap < bytes) {
        size_t ncap = std::max(bytes, (size_t)65536);
        if (s.host) CUDA_TRY(cudaFreeHost(s.host));
        if (s.dev) CUDA_TRY(cudaFree(s.dev));
        s.host = s.dev = nullptr;
        s.cap = 0;
        CUDA_TRY(cudaMallocHost(&s.host, ncap));
        CUDA_TRY(cudaMalloc(&s.dev, ncap));
        s.cap = ncap;
    }
    if (!s.done) CUDA_TRY(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
    out = &s;
    return EUC_OK;
}

// Chunks per group of the chunk-group kernels (k_init, k_resolve): 1 while
// the launch has fewer chunks than 16 blocks per SM can hold, growing to
// kChunkGroup for large batches so that the scene search is amortised.
// `group` > 0 and `per_sm` > 0 override the size and the per-SM cap.
uint32_t chunk_group(uint64_t nchunks, int nsm, uint32_t group = 0, uint32_t per_sm = 0) {
    if (group) return group;
    const uint64_t slots = (uint64_t)(nsm > 0 ? nsm : 1) * (per_sm ? per_sm : 16);
    return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(kChunkGroup, nchunks / slots));
}

// Grid of the chunk-group kernels: one block per group, at most 16 blocks per
// SM (the blocks stride the groups).
unsigned chunk_grid(uint64_t nchunks, int nsm, uint32_t group = 0, uint32_t per_sm = 0) {
    const uint32_t g = chunk_group(nchunks, nsm, group, per_sm);
    const uint64_t groups = (nchunks + g - 1) / g;
    const uint64_t cap = (uint64_t)(nsm > 0 ? nsm : 1) * (per_sm ? per_sm : 16);
    return (unsigned)std::max<uint64_t>(1, std::min(groups, cap));
}

// Resident blocks of k_raster per SM (its grid is persistent).
int raster_blocks_per_sm() {
    static int n = 0;
    if (n == 0) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_raster, kBlock, 0) != cudaSuccess || b < 1) {
            (void)cudaGetLastError();
            b = 4;
        }
        n = b;
    }
    return n;
}

// Records an event on `st` when profiling; returns nullptr otherwise.
cudaEvent_t prof_event(euc_ctx *ctx, cudaStream_t st) {
    if (!ctx->profiling || ctx->capturing) return nullptr;
    if (ctx->ev_used == ctx->ev_pool.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        ctx->ev_pool.push_back(e);
    }
    cudaEvent_t e = ctx->ev_pool[ctx->ev_used++];
    cudaEventRecord(e, st);
    return e;
}

void prof_mark(euc_ctx *ctx, int stage, cudaEvent_t a, cudaEvent_t b) {
    if (a && b) ctx->ev_marks.push_back({stage, {a, b}});
}

template <class F>
void launch_vertex(const SceneDev *sc, const uint64_t *vb, int s0, int s1, uint64_t blk0, uint64_t nblk, euc_ctx *ctx,
                   cudaStream_t st, const PrepArgs &prep) {
    if (nblk)
        k_vertex<F><<<(unsigned)nblk, kBlock, 0, st>>>(sc, vb, s0, s1, blk0, (float4 *)ctx->clip.p, (float *)ctx->vdata.p,
                                                       prep);
}

// rbase: the device chunk bases of plan_chunks; nblk: an upper bound of the
// chunks of scenes [s0, s1) (their whole targets), which sizes the grid.
template <class F>
void launch_geometry(const SceneDev *sc, const uint64_t *gb, int s0, int s1, uint64_t blk0, uint64_t nblk, euc_ctx *ctx,
                     cudaStream_t st) {
    k_geometry<F><<<(unsigned)nblk, kBlock, 0, st>>>(sc, gb, s0, s1, blk0, (float4 *)ctx->clip.p, (float *)ctx->vdata.p,
                                                     (uint8_t *)ctx->galive.p, (int *)ctx->err.p);
}

void dispatch_geometry(uint32_t shader, const SceneDev *sc, const uint64_t *gb, int s0, int s1, uint64_t blk0,
                       uint64_t nblk, euc_ctx *ctx, cudaStream_t st) {
    switch (shader) {
    case EUC_SHADER_FLAT: launch_geometry<FlatFn>(sc, gb, s0, s1, blk0, nblk, ctx, st); break;
    case EUC_SHADER_VCOLOR: launch_geometry<VColorFn>(sc, gb, s0, s1, blk0, nblk, ctx, st); break;
    case EUC_SHADER_GOURAUD: launch_geometry<GouraudFn>(sc, gb, s0, s1, blk0, nblk, ctx, st); break;
    case EUC_SHADER_TEXTURED: launch_geometry<TexturedFn>(sc, gb, s0, s1, blk0, nblk, ctx, st); break;
    case EUC_SHADER_PHONG: launch_geometry<PhongFn>(sc, gb, s0, s1, blk0, nblk, ctx, st); break;
    case EUC_SHADER_SHADOW: launch_geometry<ShadowFn>(sc, gb, s0, s1, blk0, nblk, ctx, st); break;
    }
}

template <class F>
void launch_resolve(const SceneDev *sc, const uint64_t *rbase, int s0, int s1, uint64_t nblk, euc_ctx *ctx,
                    cudaStream_t st) {
    if (!nblk) return;
    const euc_tuning &tu = ctx->tune;
    k_resolve<F><<<chunk_grid(nblk, ctx->nsm, tu.chunk_group, tu.chunk_blocks_per_sm), kBlock, 0, st>>>(
        sc, rbase, s0, s1, chunk_group(nblk, ctx->nsm, tu.chunk_group, tu.chunk_blocks_per_sm),
        (const TriRec *)ctx->recs.p, (const float *)ctx->vdata.p, (const unsigned long long *)ctx->vbuf.p,
        (const uint4 *)ctx->cov.p);
}

void dispatch_vertex(uint32_t shader, const SceneDev *sc, const uint64_t *vb, int s0, int s1, uint64_t blk0, uint64_t nblk,
                     euc_ctx *ctx, cudaStream_t st, const PrepArgs &prep) {
    switch (shader) {
    case EUC_SHADER_FLAT: launch_vertex<FlatFn>(sc, vb, s0, s1, blk0, nblk, ctx, st, prep); break;
    case EUC_SHADER_VCOLOR: launch_vertex<VColorFn>(sc, vb, s0, s1, blk0, nblk, ctx, st, prep); break;
    case EUC_SHADER_GOURAUD: launch_vertex<GouraudFn>(sc, vb, s0, s1, blk0, nblk, ctx, st, prep); break;
    case EUC_SHADER_TEXTURED: launch_vertex<TexturedFn>(sc, vb, s0, s1, blk0, nblk, ctx, st, prep); break;
    case EUC_SHADER_PHONG: launch_vertex<PhongFn>(sc, vb, s0, s1, blk0, nblk, ctx, st, prep); break;
    case EUC_SHADER_SHADOW: launch_vertex<ShadowFn>(sc, vb, s0, s1, blk0, nblk, ctx, st, prep); break;
    }
}

void dispatch_resolve(uint32_t shader, const SceneDev *sc, const uint64_t *rbase, int s0, int s1, uint64_t nblk,
                      euc_ctx *ctx, cudaStream_t st) {
    switch (shader) {
    case EUC_SHADER_FLAT: launch_resolve<FlatFn>(sc, rbase, s0, s1, nblk, ctx, st); break;
    case EUC_SHADER_VCOLOR: launch_resolve<VColorFn>(sc, rbase, s0, s1, nblk, ctx, st); break;
    case EUC_SHADER_GOURAUD: launch_resolve<GouraudFn>(sc, rbase, s0, s1, nblk, ctx, st); break;
    case EUC_SHADER_TEXTURED: launch_resolve<TexturedFn>(sc, rbase, s0, s1, nblk, ctx, st); break;
    case EUC_SHADER_PHONG: launch_resolve<PhongFn>(sc, rbase, s0, s1, nblk, ctx, st); break;
    case EUC_SHADER_SHADOW: launch_resolve<ShadowFn>(sc, rbase, s0, s1, nblk, ctx, st); break;
    }
}

template <class F>
void launch_resolve_ordered(const SceneDev *sc, const uint64_t *pb, int s0, int s1, uint64_t blk0, uint64_t nblk,
                            euc_ctx *ctx, cudaStream_t st) {
    if (nblk)
        k_resolve_ordered<F><<<(unsigned)nblk, kBlock, 0, st>>>(sc, pb, s0, s1, blk0, (const TriRec *)ctx->recs.p,
                                                                (const float *)ctx->vdata.p,
                                                                (const unsigned long long *)ctx->vbuf.p,
                                                                (const uint2 *)ctx->frags.p, (const uint4 *)ctx->cov.p);
}

void dispatch_resolve_ordered(uint32_t shader, const SceneDev *sc, const uint64_t *pb, int s0, int s1, uint64_t blk0,
                              uint64_t nblk, euc_ctx *ctx, cudaStream_t st) {
    switch (shader) {
    case EUC_SHADER_FLAT: launch_resolve_ordered<FlatFn>(sc, pb, s0, s1, blk0, nblk, ctx, st); break;
    case EUC_SHADER_VCOLOR: launch_resolve_ordered<VColorFn>(sc, pb, s0, s1, blk0, nblk, ctx, st); break;
    case EUC_SHADER_GOURAUD: launch_resolve_ordered<GouraudFn>(sc, pb, s0, s1, blk0, nblk, ctx, st); break;
    case EUC_SHADER_TEXTURED: launch_resolve_ordered<TexturedFn>(sc, pb, s0, s1, blk0, nblk, ctx, st); break;
    case EUC_SHADER_PHONG: launch_resolve_ordered<PhongFn>(sc, pb, s0, s1, blk0, nblk, ctx, st); break;
    case EUC_SHADER_SHADOW: launch_resolve_ordered<ShadowFn>(sc, pb, s0, s1, blk0, nblk, ctx, st); break;
    }
}

// Runs a batch of scenes.  All pointers inside `scenes` are device pointers.
// Staging supplied by a CUDA graph instead of the context's ring.  With
// `dry` the batch is planned and the scratch buffers are sized, nothing is
// enqueued, and `need` returns the staging bytes.  Otherwise `host` / `dev`
// (at least `need` bytes, owned by the graph) carry the scene tables, no
// stream is synchronised and the ordered path (which synchronises) is refused.
struct StageOverride {
    bool dry = false;
    bool fill = false;     // fill `host` with the scene tables and return: nothing is enqueued
    bool no_copy = false;  // enqueue the launches without the copy of `host` to `dev`
    void *host = nullptr;
    void *dev = nullptr;
    size_t need = 0;
};

int run_batch(euc_ctx *ctx, const euc_scene *scenes, size_t n, cudaStream_t st, StageOverride *so = nullptr) {
    std::vector<Plan> plans;
    plans.reserve(n);
    for (size_t i = 0; i < n; ++i) {
        Plan p;
        if (int rc = plan_scene(scenes[i], p)) return rc;
        if (!p.skip) plans.push_back(p);
    }
    ctx->last_nscenes = (int)plans.size();
    if (plans.empty()) return EUC_OK;
    // group scenes by shader kind so that each kind owns contiguous ranges
    // group scenes by (ordered path, shader kind): each group owns contiguous
    // vertex / pixel / resolve ranges, and ordered scenes come last so that
    // their pixels form one range for the pixel scan
    auto group_of = [](const Plan &p) { return (p.d.keytype == KEY_ORDERED ? 64u : 0u) + p.d.shader; };
    std::stable_sort(plans.begin(), plans.end(),
                     [&](const Plan &a, const Plan &b) { return group_of(a) < group_of(b); });
    const int ns = (int)plans.size();
    uint64_t vtx = 0, vd = 0, tri = 0, pix = 0, res = 0;
    std::vector<uint64_t> res_base(ns);
    for (int i = 0; i < ns; ++i) {
        Plan &p = plans[i];
        p.d.vtx_base = vtx;
        p.d.vd_base = vd;
        p.d.tri_base = tri;
        p.d.pix_base = pix;
        res_base[i] = res;
        vtx += pad_up(p.d.nverts, kBlock);
        vd += pad_up(p.d.nverts * p.nv, 4);  // 16-byte aligned regions: vector gathers
        tri += pad_up(std::max<uint64_t>(p.d.ngroups, 1), kBlock);
        pix += pad_up((uint64_t)p.d.W * p.d.H, kBlock);
        res += resolve_blocks(p.d);
    }
    // strip path: the scenes it may take, their strips, and the widest
    // strip's keys (k_strip's dynamic shared memory).  In the default mode a
    // scene with fewer than one primitive per kStripMinPixels target pixels
    // cannot be overdrawn enough to pay for the strip launches; k_bin_count
    // decides for the others on the device.
    std::vector<uint64_t> strip_first(ns + 1);
    uint64_t nstrips = 0;
    size_t strip_smem = 0;
    const uint32_t strip_mode = ctx->tune.strip_path;
    for (int i = 0; i < ns; ++i) {
        Plan &p = plans[i];
        strip_first[i] = nstrips;
        const bool can = p.d.prim == EUC_PRIM_TRIANGLE_LIST && p.d.keytype != KEY_ORDERED &&
                         (strip_mode == 2 ||
                          (strip_mode == 0 && (uint64_t)p.d.ntris * kStripMinPixels >= (uint64_t)p.d.W * p.d.H));
        const uint32_t h = can ? strip_rows(p.d.W, p.d.H) : 0u;
        p.d.strip_h = h;
        p.d.strip_base = (uint32_t)nstrips;
        p.d.nstrips = h ? (p.d.H + h - 1) / h : 0u;
        nstrips += p.d.nstrips;
        if (h) strip_smem = std::max(strip_smem, (size_t)h * strip_pitch(p.d.W) * sizeof(unsigned long long));
    }
    strip_first[ns] = nstrips;
    if (nstrips >= 0x7FFFFFFFull) return EUC_ERR_CAPACITY;
    // geometry stage: its input threads, and its output vertices after every
    // scene's vertex-stage outputs (the vertex launches cover only those)
    const uint64_t vtx_stage = vtx;  // the vertex launches end here
    std::vector<uint64_t> gin_base(ns);
    uint64_t gin = 0;
    for (int i = 0; i < ns; ++i) {
        Plan &p = plans[i];
        gin_base[i] = gin;
        if (!p.d.geom) continue;
        gin += pad_up(p.d.ngin, kBlock);
        p.d.gvtx_base = vtx;
        p.d.gvd_base = vd;
        vtx += 3ull * p.d.ntris;
        vd += pad_up(3ull * p.d.ntris * p.nv, 4);
    }
    if (tri >= 0x7FFFFFF0ull) return EUC_ERR_CAPACITY;  // visibility keys hold a 31-bit primitive id
    const uint64_t nchunks = tri / kBlock;
    const uint64_t nscan = (tri + kScanBlock - 1) / kScanBlock;
    int rc;
    if ((rc = grow(ctx->clip, std::max<uint64_t>(vtx, 1) * sizeof(float4)))) return rc;
    if ((rc = grow(ctx->vdata, std::max<uint64_t>(vd, 1) * sizeof(float)))) return rc;
    if ((rc = grow(ctx->recs, tri * sizeof(TriRec)))) return rc;
    if ((rc = grow(ctx->rows, tri * sizeof(uint32_t)))) return rc;
    if ((rc = grow(ctx->chunk_sums, nchunks * sizeof(uint2)))) return rc;
    if ((rc = grow(ctx->live_tri, tri * sizeof(uint32_t)))) return rc;
    if ((rc = grow(ctx->live_rowoff, tri * sizeof(uint64_t)))) return rc;
    if ((rc = grow(ctx->totals, 8 * sizeof(unsigned long long)))) return rc;
    if ((rc = grow(ctx->vbuf, pix * sizeof(unsigned long long)))) return rc;
    if ((rc = grow(ctx->err, ns * sizeof(int)))) return rc;
    if ((rc = grow(ctx->stats, ns * sizeof(SceneStats)))) return rc;
    if ((rc = grow(ctx->cov, ns * sizeof(uint4)))) return rc;
    if ((rc = grow(ctx->plan, 2 * (ns + 1) * sizeof(uint64_t)))) return rc;
    if (gin && (rc = grow(ctx->galive, tri))) return rc;
    // strip lists: an admitted primitive has one entry per strip it overlaps;
    // k_bin_count admits primitives while the list has room
    const uint64_t entry_cap = nstrips ? 2 * tri + (1ull << 21) : 0;
    if (nstrips) {
        if ((rc = grow(ctx->strip_cnt, nstrips * sizeof(uint32_t)))) return rc;
        if ((rc = grow(ctx->strip_fill, nstrips * sizeof(uint32_t)))) return rc;
        if ((rc = grow(ctx->strip_off, (nstrips + 1) * sizeof(uint32_t)))) return rc;
        if ((rc = grow(ctx->strip_uoff, (nstrips + 1) * sizeof(uint32_t)))) return rc;
        if ((rc = grow(ctx->entries, entry_cap * sizeof(uint2)))) return rc;
        if ((rc = grow(ctx->unit_strip, (nstrips + entry_cap / kStripUnit + 1) * sizeof(uint32_t)))) return rc;
        if ((rc = grow(ctx->bbox, tri * sizeof(uint4)))) return rc;
    }
    // staging: scene table | vtx bases | resolve bases | geometry bases |
    // first strip of each scene | scene of each setup chunk | uniforms
    const size_t off_sc = 0;
    const size_t off_vb = pad_up(ns * sizeof(SceneDev), 16);
    const size_t off_rb = off_vb + pad_up(ns * sizeof(uint64_t), 16);
    const size_t off_gb = off_rb + pad_up(ns * sizeof(uint64_t), 16);
    const size_t off_sb = off_gb + pad_up(ns * sizeof(uint64_t), 16);
    const size_t off_cs = off_sb + pad_up((ns + 1) * sizeof(uint64_t), 16);
    // one scene needs no chunk -> scene table (the kernels read a null one as scene 0)
    const bool one_scene = ns == 1;
    size_t off_u = off_cs + (one_scene ? 0 : pad_up(nchunks * sizeof(uint32_t), 16));
    std::vector<size_t> uoff(ns);
    for (int i = 0; i < ns; ++i) {
        uoff[i] = off_u;
        off_u += pad_up(plans[i].usize, 16);
    }
    if (so) {
        if (plans.back().d.keytype == KEY_ORDERED) return EUC_ERR_INVALID;  // a graph cannot synchronise
        if (so->dry) {
            so->need = off_u;
            return EUC_OK;
        }
        if (off_u > so->need) return EUC_ERR_INVALID;
    }
    StageSlot *slot = nullptr;
    if (!so && (rc = acquire_slot(ctx, off_u, slot))) return rc;
    uint8_t *h = (uint8_t *)(so ? so->host : slot->host);
    uint8_t *dv = (uint8_t *)(so ? so->dev : slot->dev);
    SceneDev *hsc = (SceneDev *)(h + off_sc);
    uint64_t *hvb = (uint64_t *)(h + off_vb), *hrb = (uint64_t *)(h + off_rb), *hgb = (uint64_t *)(h + off_gb);
    std::memcpy(h + off_sb, strip_first.data(), (ns + 1) * sizeof(uint64_t));
    uint32_t *hcs = (uint32_t *)(h + off_cs);
    for (int i = 0; i < ns && !one_scene; ++i) {  // scene ranges of primitives are padded to whole setup chunks
        const uint64_t c0 = plans[i].d.tri_base / kBlock, c1 = (i + 1 < ns ? plans[i + 1].d.tri_base : tri) / kBlock;
        for (uint64_t c = c0; c < c1; ++c) hcs[c] = (uint32_t)i;
    }
    for (int i = 0; i < ns; ++i) {
        std::memcpy(h + uoff[i], plans[i].uniforms, plans[i].usize);
        plans[i].d.uniforms = dv + uoff[i];
        hsc[i] = plans[i].d;
        hvb[i] = plans[i].d.vtx_base;
        hrb[i] = res_base[i];
        hgb[i] = gin_base[i];
    }
    if (so && so->fill) return EUC_OK;
    if (!so || !so->no_copy) CUDA_TRY(cudaMemcpyAsync(dv, h, off_u, cudaMemcpyHostToDevice, st));
    const SceneDev *dsc = (const SceneDev *)(dv + off_sc);
    const uint64_t *dvb = (const uint64_t *)(dv + off_vb), *drb = (const uint64_t *)(dv + off_rb),
                   *dgb = (const uint64_t *)(dv + off_gb), *dsb = (const uint64_t *)(dv + off_sb);
    const uint32_t *dcs = one_scene ? nullptr : (const uint32_t *)(dv + off_cs);
    PrepArgs prep = {};
    prep.err = (int *)ctx->err.p;
    prep.stats = (SceneStats *)ctx->stats.p;
    prep.cov = (uint4 *)ctx->cov.p;
    prep.chunk_sums = (uint2 *)ctx->chunk_sums.p;
    prep.strip_cnt = (uint32_t *)ctx->strip_cnt.p;
    prep.strip_fill = (uint32_t *)ctx->strip_fill.p;
    prep.totals = (unsigned long long *)ctx->totals.p;
    prep.nchunks = nchunks;
    prep.n = std::max<uint64_t>(std::max<uint64_t>((uint64_t)ns, nchunks), std::max<uint64_t>(nstrips, 2));
    prep.nsc = (uint32_t)ns;
    prep.nstrips = (uint32_t)nstrips;
    // vertex stage, one launch per shader kind; the first also does the clears
    cudaEvent_t e0 = prof_event(ctx, st);
    const PrepArgs no_prep = {};
    bool prepped = false;
    for (int a = 0; a < ns;) {
        int b = a;
        while (b < ns && plans[b].d.shader == plans[a].d.shader) ++b;
        const uint64_t blk0 = plans[a].d.vtx_base / kBlock;
        const uint64_t blk1 = (b < ns ? plans[b].d.vtx_base : vtx_stage) / kBlock;
        dispatch_vertex(plans[a].d.shader, dsc, dvb, a, b, blk0, blk1 - blk0, ctx, st, prepped ? no_prep : prep);
        prepped = prepped || blk1 > blk0;
        ctx->launches += blk1 > blk0;
        a = b;
    }
    if (!prepped) {
        k_prep<<<(unsigned)((prep.n + kBlock - 1) / kBlock), kBlock, 0, st>>>(prep);
        ctx->launches += 1;
    }
    // geometry stage, one launch per shader kind that has one
    for (int a = 0; a < ns && gin;) {
        int b = a;
        while (b < ns && plans[b].d.shader == plans[a].d.shader) ++b;
        const uint64_t blk0 = gin_base[a] / kBlock, blk1 = (b < ns ? gin_base[b] : gin) / kBlock;
        if (blk1 > blk0) {
            dispatch_geometry(plans[a].d.shader, dsc, dgb, a, b, blk0, blk1 - blk0, ctx, st);
            ctx->launches += 1;
        }
        a = b;
    }
    cudaEvent_t e1 = prof_event(ctx, st);
    k_setup<<<(unsigned)nchunks, kBlock, 0, st>>>(dsc, dcs, (const float4 *)ctx->clip.p,
                                                   (TriRec *)ctx->recs.p, (uint32_t *)ctx->rows.p,
                                                   (uint2 *)ctx->chunk_sums.p, (int *)ctx->err.p,
                                                   (SceneStats *)ctx->stats.p, (uint4 *)ctx->cov.p,
                                                   (const uint8_t *)ctx->galive.p,
                                                   nstrips ? (uint4 *)ctx->bbox.p : nullptr);
    // binning blocks stride the setup chunks
    const unsigned bin_grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(nchunks, (uint64_t)ctx->nsm * 8));
    if (nstrips) {  // the strip path's routing and counts
        k_bin_count<<<bin_grid, kBlock, 0, st>>>(
            dsc, dcs, nchunks, (uint32_t *)ctx->rows.p, (const uint4 *)ctx->bbox.p, (const uint4 *)ctx->cov.p,
            (const SceneStats *)ctx->stats.p, (uint2 *)ctx->chunk_sums.p, (uint32_t *)ctx->strip_cnt.p,
            (unsigned long long *)ctx->totals.p + 6, entry_cap, strip_mode);
        ctx->launches += 1;
    }
    cudaEvent_t e2 = prof_event(ctx, st);
    uint64_t *const ibase = (uint64_t *)ctx->plan.p, *const rbase = ibase + ns + 1;
    const uint64_t nsblk = (nstrips + kScanBlock - 1) / kScanBlock;
    k_scan_plan<<<(unsigned)(nscan + 1 + nsblk), kBlock, 0, st>>>(
        (const uint32_t *)ctx->rows.p, (const uint2 *)ctx->chunk_sums.p, tri, (uint32_t *)ctx->live_tri.p,
        (uint64_t *)ctx->live_rowoff.p, (unsigned long long *)ctx->totals.p, (uint32_t)nscan, dsc, ns,
        (const uint4 *)ctx->cov.p, ibase, rbase, (const uint32_t *)ctx->strip_cnt.p, (uint32_t)nstrips,
        (uint32_t *)ctx->strip_off.p, (uint32_t *)ctx->strip_uoff.p, (uint32_t *)ctx->unit_strip.p);
    cudaEvent_t e3 = prof_event(ctx, st);
    const euc_tuning &tu = ctx->tune;
    const uint64_t ichunks = (pix + kInitChunk - 1) / kInitChunk + ns;  // bounds the chunks plan_chunks counts
    k_init<<<chunk_grid(ichunks, ctx->nsm, tu.chunk_group, tu.chunk_blocks_per_sm), kBlock, 0, st>>>(
        dsc, ibase, ns, (const uint4 *)ctx->cov.p, (unsigned long long *)ctx->vbuf.p,
        chunk_group(ichunks, ctx->nsm, tu.chunk_group, tu.chunk_blocks_per_sm));
    cudaEvent_t e4 = prof_event(ctx, st);
    if (nstrips) {  // the strip lists, then the strips (after k_init, before the item queue)
        k_bin<<<bin_grid, kBlock, 0, st>>>(dsc, dcs, nchunks, (const uint32_t *)ctx->rows.p, (const uint4 *)ctx->bbox.p,
                                           (const uint4 *)ctx->cov.p, (const SceneStats *)ctx->stats.p,
                                           (const uint32_t *)ctx->strip_off.p, (uint32_t *)ctx->strip_fill.p,
                                           (uint2 *)ctx->entries.p, strip_mode);
        k_strip<<<(unsigned)ctx->nsm * kStripBlocksPerSm, kStripThreads, strip_smem, st>>>(
            dsc, dsb, ns, (const uint4 *)ctx->cov.p, (const uint32_t *)ctx->strip_off.p,
            (const uint32_t *)ctx->strip_uoff.p, (const uint32_t *)ctx->unit_strip.p, (const uint2 *)ctx->entries.p,
            (const TriRec *)ctx->recs.p, (const int *)ctx->err.p, (unsigned long long *)ctx->vbuf.p,
            (SceneStats *)ctx->stats.p, (unsigned long long *)ctx->totals.p);
        ctx->launches += 2;
    }
    const int witems = tu.raster_warp_rows ? (int)tu.raster_warp_rows : kWarpItems;
    // persistent blocks, but no more than the items can keep busy: a
    // primitive slot has at most max(W, H) + 2 items (rows, or line steps)
    uint64_t item_bound = 0;
    for (int i = 0; i < ns; ++i) {
        const uint64_t slots = (i + 1 < ns ? plans[i + 1].d.tri_base : tri) - plans[i].d.tri_base;
        item_bound += slots * ((uint64_t)std::max(plans[i].d.W, plans[i].d.H) + 2);
    }
    const uint64_t busy = (item_bound + (uint64_t)witems * (kBlock / 32) - 1) / ((uint64_t)witems * (kBlock / 32));
    const unsigned rgrid = (unsigned)std::max<uint64_t>(
        1, std::min<uint64_t>(busy, (uint64_t)ctx->nsm * (tu.raster_blocks_per_sm ? tu.raster_blocks_per_sm
                                                                                   : (uint32_t)ctx->raster_blocks)));
    const bool probe = tu.raster_probe == 1;
    k_raster<<<rgrid, kBlock, 0, st>>>(dsc, (const TriRec *)ctx->recs.p, (const uint32_t *)ctx->live_tri.p,
                                       (const uint64_t *)ctx->live_rowoff.p, (unsigned long long *)ctx->totals.p,
                                       (const int *)ctx->err.p, (unsigned long long *)ctx->vbuf.p,
                                       (SceneStats *)ctx->stats.p, 0, nullptr, witems, probe);
    ctx->launches += 4;
    // ordered scenes: scan the per-pixel counts, size the fragment buffer
    // (one stream synchronisation), fill the lists in a second raster pass
    int first_ordered = ns;
    while (first_ordered > 0 && plans[first_ordered - 1].d.keytype == KEY_ORDERED) --first_ordered;
    if (first_ordered < ns) {
        const uint64_t p0 = plans[first_ordered].d.pix_base, p1 = pix;
        const uint64_t nb = (p1 - p0 + kOScanBlock - 1) / kOScanBlock;
        if ((rc = grow(ctx->obsum, nb * sizeof(unsigned long long)))) return rc;
        unsigned long long *totals = (unsigned long long *)ctx->totals.p;
        k_oscan_reduce<<<(unsigned)nb, kBlock, 0, st>>>((const unsigned long long *)ctx->vbuf.p, p0, p1,
                                                        (unsigned long long *)ctx->obsum.p);
        k_oscan_apply<<<(unsigned)nb, kBlock, 0, st>>>((unsigned long long *)ctx->vbuf.p, p0, p1,
                                                       (const unsigned long long *)ctx->obsum.p, totals + 4);
        unsigned long long nfrag = 0;
        CUDA_TRY(cudaMemcpyAsync(&nfrag, totals + 4, sizeof(nfrag), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        if (nfrag >= 0xFFFFFFFFull) return EUC_ERR_CAPACITY;  // list offsets are 32-bit
        if ((rc = grow(ctx->frags, std::max<uint64_t>(nfrag, 1) * sizeof(uint2)))) return rc;
        k_raster<<<rgrid, kBlock, 0, st>>>(dsc, (const TriRec *)ctx->recs.p, (const uint32_t *)ctx->live_tri.p,
                                           (const uint64_t *)ctx->live_rowoff.p, (unsigned long long *)ctx->totals.p,
                                           (const int *)ctx->err.p, (unsigned long long *)ctx->vbuf.p,
                                           (SceneStats *)ctx->stats.p, 1, (uint2 *)ctx->frags.p, witems, probe);
        ctx->launches += 3;
    }
    cudaEvent_t e5 = prof_event(ctx, st);
    for (int a = 0; a < ns;) {
        int b = a;
        while (b < ns && group_of(plans[b]) == group_of(plans[a])) ++b;
        const uint64_t blk0 = res_base[a];
        const uint64_t blk1 = b < ns ? res_base[b] : res;
        if (plans[a].d.keytype == KEY_ORDERED)
            dispatch_resolve_ordered(plans[a].d.shader, dsc, drb, a, b, blk0, blk1 - blk0, ctx, st);
        else
            dispatch_resolve(plans[a].d.shader, dsc, rbase, a, b, blk1 - blk0, ctx, st);
        ctx->launches += blk1 > blk0;
        a = b;
    }
    cudaEvent_t e6 = prof_event(ctx, st);
    prof_mark(ctx, EUC_STAGE_VERTEX, e0, e1);
    prof_mark(ctx, EUC_STAGE_SETUP, e1, e2);
    prof_mark(ctx, EUC_STAGE_SCAN, e2, e3);
    prof_mark(ctx, EUC_STAGE_INIT, e3, e4);
    prof_mark(ctx, EUC_STAGE_RASTER, e4, e5);
    prof_mark(ctx, EUC_STAGE_RESOLVE, e5, e6);
    CUDA_TRY(cudaGetLastError());
    if (slot) {
        CUDA_TRY(cudaEventRecord(slot->done, st));
        slot->pending = true;
    }
    return EUC_OK;
}

}  // namespace

namespace {
int render_one(euc_ctx *ctx, const euc_scene &s, cudaStream_t st);
void free_shapes(euc_ctx *ctx);
}  // namespace

extern "C" {

int euc_abi_version(void) { return EUC_ABI_VERSION; }

const char *euc_status_string(int status) {
    switch (status) {
    case EUC_OK: return "ok";
    case EUC_ERR_INVALID: return "invalid argument";
    case EUC_ERR_SIZE_MISMATCH: return "pixel target size is not compatible with depth target size";
    case EUC_ERR_INDEX_OOB: return "index out of bounds of the vertex slice";
    case EUC_ERR_OOM: return "out of device memory";
    case EUC_ERR_CUDA: return "CUDA error";
    case EUC_ERR_BAND: return "band height is zero (target wider than 20000 << msaa level)";
    case EUC_ERR_TIMEOUT: return "bounded device wait timed out";
    case EUC_ERR_BUDGET: return "request exceeds the framebuffer budget";
    case EUC_ERR_CAPACITY: return "input exceeds a fixed capacity";
    case EUC_ERR_STALE: return "graph recorded against context scratch that has since moved";
    default: return "unknown status";
    }
}

int euc_ctx_create(int device, euc_ctx **out) {
    if (!out) return EUC_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return EUC_ERR_INVALID;
    CUDA_TRY(cudaSetDevice(device));
    euc_ctx *c = new (std::nothrow) euc_ctx();
    if (!c) return EUC_ERR_OOM;
    c->device = device;
    c->raster_blocks = raster_blocks_per_sm();
    int pageable = 0;
    if (cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) {
        delete c;
        return EUC_ERR_CUDA;
    }
    c->pageable = pageable != 0;
    // k_strip's keys: up to kStripKeyBytes of dynamic shared memory
    if (cudaFuncSetAttribute(k_strip, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStripKeyBytes) != cudaSuccess) {
        (void)cudaGetLastError();
        delete c;
        return EUC_ERR_CUDA;
    }
    *out = c;
    return EUC_OK;
}

int euc_ctx_destroy(euc_ctx *ctx) {
    if (!ctx) return EUC_ERR_INVALID;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    free_shapes(ctx);
    DevBuf *bufs[] = {&ctx->clip, &ctx->vdata, &ctx->recs, &ctx->rows, &ctx->chunk_sums, &ctx->live_tri, &ctx->live_rowoff,
                      &ctx->totals, &ctx->vbuf, &ctx->err, &ctx->stats, &ctx->cov, &ctx->obsum, &ctx->frags,
                      &ctx->plan, &ctx->galive, &ctx->h_arena, &ctx->h_tex[0], &ctx->strip_cnt, &ctx->strip_fill,
                      &ctx->strip_off, &ctx->strip_uoff, &ctx->entries, &ctx->unit_strip, &ctx->bbox};
    for (DevBuf *b : bufs)
        if (b->p) cudaFree(b->p);
    if (ctx->h_pinned.p) cudaFreeHost(ctx->h_pinned.p);
    for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
    for (auto &s : ctx->slots) {
        if (s.host) cudaFreeHost(s.host);
        if (s.dev) cudaFree(s.dev);
        if (s.done) cudaEventDestroy(s.done);
    }
    delete ctx;
    return EUC_OK;
}

int euc_ctx_reserve(euc_ctx *ctx, uint64_t max_verts, uint64_t max_tris, uint64_t max_pixels, uint64_t max_scenes) {
    if (!ctx) return EUC_ERR_INVALID;
    std::lock_guard<std::mutex> g(ctx->mu);
    CUDA_TRY(cudaSetDevice(ctx->device));
    const uint64_t ns = std::max<uint64_t>(max_scenes, 1);
    const uint64_t vtx = max_verts + ns * kBlock, tri = max_tris + ns * kBlock, pix = max_pixels + ns * kBlock;
    int rc;
    if ((rc = grow(ctx->clip, vtx * sizeof(float4)))) return rc;
    if ((rc = grow(ctx->vdata, (vtx * vd_stride(11) + 4 * ns) * sizeof(float)))) return rc;
    if ((rc = grow(ctx->recs, tri * sizeof(TriRec)))) return rc;
    if ((rc = grow(ctx->rows, tri * sizeof(uint32_t)))) return rc;
    if ((rc = grow(ctx->chunk_sums, (tri / kBlock + 1) * sizeof(uint2)))) return rc;
    if ((rc = grow(ctx->live_tri, tri * sizeof(uint32_t)))) return rc;
    if ((rc = grow(ctx->live_rowoff, tri * sizeof(uint64_t)))) return rc;
    if ((rc = grow(ctx->totals, 8 * sizeof(unsigned long long)))) return rc;
    if ((rc = grow(ctx->vbuf, pix * sizeof(unsigned long long)))) return rc;
    if ((rc = grow(ctx->err, ns * sizeof(int)))) return rc;
    if ((rc = grow(ctx->stats, ns * sizeof(SceneStats)))) return rc;
    if ((rc = grow(ctx->cov, ns * sizeof(uint4)))) return rc;
    if ((rc = grow(ctx->plan, 2 * (ns + 1) * sizeof(uint64_t)))) return rc;
    return EUC_OK;
}

int euc_ctx_set_tuning(euc_ctx *ctx, const euc_tuning *t) {
    if (!ctx) return EUC_ERR_INVALID;
    euc_tuning v{};
    if (t) {
        v = *t;
        if (v.raster_warp_rows && (v.raster_warp_rows % 32 || v.raster_warp_rows > (uint32_t)kWarpItems))
            return EUC_ERR_INVALID;
        if (v.raster_blocks_per_sm > 64 || v.chunk_group > 1024 || v.chunk_blocks_per_sm > 64 || v.raster_probe > 2 ||
            v.strip_path > 2)
            return EUC_ERR_INVALID;
        if (v.host_copy > EUC_HOST_COPY_DIRECT || (v.host_copy == EUC_HOST_COPY_DIRECT && !ctx->pageable))
            return EUC_ERR_INVALID;
    }
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->tune = v;
    return EUC_OK;
}

int euc_ctx_get_tuning(euc_ctx *ctx, euc_tuning *t) {
    if (!ctx || !t) return EUC_ERR_INVALID;
    std::lock_guard<std::mutex> g(ctx->mu);
    *t = ctx->tune;
    return EUC_OK;
}

int euc_ctx_set_profiling(euc_ctx *ctx, int enable) {
    if (!ctx) return EUC_ERR_INVALID;
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->profiling = enable != 0;
    return EUC_OK;
}

int euc_ctx_profile(euc_ctx *ctx, double ms[EUC_STAGE_COUNT], uint64_t *launches) {
    if (!ctx) return EUC_ERR_INVALID;
    std::lock_guard<std::mutex> g(ctx->mu);
    CUDA_TRY(cudaSetDevice(ctx->device));
    double acc[EUC_STAGE_COUNT] = {0, 0, 0, 0, 0, 0};
    for (auto &m : ctx->ev_marks) {
        CUDA_TRY(cudaEventSynchronize(m.second.second));
        float t = 0.0f;
        CUDA_TRY(cudaEventElapsedTime(&t, m.second.first, m.second.second));
        acc[m.first] += t;
    }
    ctx->ev_marks.clear();
    ctx->ev_used = 0;
    if (ms)
        for (int i = 0; i < EUC_STAGE_COUNT; ++i) ms[i] = acc[i];
    if (launches) *launches = ctx->launches;
    ctx->launches = 0;
    return EUC_OK;
}

int euc_ctx_sync(euc_ctx *ctx, void *stream) {
    if (!ctx) return EUC_ERR_INVALID;
    std::lock_guard<std::mutex> g(ctx->mu);
    CUDA_TRY(cudaSetDevice(ctx->device));
    CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    if (ctx->last_nscenes == 0 || !ctx->err.p) return EUC_OK;
    std::vector<int> e(ctx->last_nscenes);
    CUDA_TRY(cudaMemcpy(e.data(), ctx->err.p, e.size() * sizeof(int), cudaMemcpyDeviceToHost));
    for (int v : e)
        if (v) {
            CUDA_TRY(cudaMemset(ctx->err.p, 0, e.size() * sizeof(int)));
            return v;
        }
    return EUC_OK;
}

int euc_ctx_stats(euc_ctx *ctx, void *stream, euc_stats *out) {
    if (!ctx || !out) return EUC_ERR_INVALID;
    std::lock_guard<std::mutex> g(ctx->mu);
    CUDA_TRY(cudaSetDevice(ctx->device));
    CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    std::memset(out, 0, sizeof(*out));
    if (ctx->last_nscenes == 0 || !ctx->stats.p) return EUC_OK;
    std::vector<SceneStats> s(ctx->last_nscenes);
    CUDA_TRY(cudaMemcpy(s.data(), ctx->stats.p, s.size() * sizeof(SceneStats), cudaMemcpyDeviceToHost));
    for (auto &x : s) {
        out->culled += x.culled;
        out->candidates += x.candidates;
    }
    return EUC_OK;
}

int euc_render(euc_ctx *ctx, const euc_pipeline_desc *desc, const void *uniforms, size_t uniforms_size,
               const euc_vertex_layout *layout, const void *vertices, size_t nverts, const uint32_t *indices,
               size_t nindices, const euc_target *pixel, const euc_target *depth, void *stream) {
    if (!ctx || !desc || !layout) return EUC_ERR_INVALID;
    euc_scene s;
    std::memset(&s, 0, sizeof(s));
    s.desc = *desc;
    s.layout = *layout;
    s.vertices = vertices;
    s.nverts = nverts;
    s.indices = indices;
    s.nindices = nindices;
    if (pixel) s.pixel = *pixel;
    if (depth) s.depth = *depth;
    s.uniforms = uniforms;
    s.uniforms_size = uniforms_size;
    std::lock_guard<std::mutex> g(ctx->mu);
    CUDA_TRY(cudaSetDevice(ctx->device));
    return render_one(ctx, s, (cudaStream_t)stream);
}

int euc_render_batch(euc_ctx *ctx, const euc_scene *scenes, size_t n, void *stream) {
    if (!ctx || (n && !scenes)) return EUC_ERR_INVALID;
    std::lock_guard<std::mutex> g(ctx->mu);
    CUDA_TRY(cudaSetDevice(ctx->device));
    return run_batch(ctx, scenes, n, (cudaStream_t)stream);
}

}  // extern "C"

// The scratch buffers a recorded batch reads and writes (scratch_ptrs).
constexpr int kScratchBufs = 21;

struct euc_graph {
    euc_ctx *ctx = nullptr;
    void *host = nullptr;  // staging owned by the graph: read by every replay
    void *dev = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int nscenes = 0;
    uint64_t launches = 0;   // kernels in the recorded batch
    void *scratch[kScratchBufs] = {};  // the context's scratch pointers the graph was recorded with
};

namespace {

// The scratch buffers a recorded batch reads and writes.  A later render that
// grows one of them moves it, and the graph may then no longer be launched.
void scratch_ptrs(const euc_ctx *c, void *out[kScratchBufs]) {
    const DevBuf *b[kScratchBufs] = {&c->clip,       &c->vdata,      &c->recs,      &c->rows,       &c->chunk_sums,
                                     &c->live_tri,   &c->live_rowoff, &c->totals,   &c->vbuf,       &c->err,
                                     &c->stats,      &c->cov,        &c->plan,      &c->galive,     &c->strip_cnt,
                                     &c->strip_fill, &c->strip_off,  &c->strip_uoff, &c->entries,  &c->unit_strip,
                                     &c->bbox};
    for (int i = 0; i < kScratchBufs; ++i) out[i] = b[i]->p;
}

void graph_free(euc_graph *g) {
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    if (g->host) cudaFreeHost(g->host);
    if (g->dev) cudaFree(g->dev);
    delete g;
}

}  // namespace

// ---------------------------------------------------------------------------
// euc_render's recorded shapes.  A plain render is eight dependent stream
// operations (the scene-table copy and seven launches), and for a small
// scene their latencies, not the kernels, set the time per call.  So
// euc_render records the launches of a scene shape as a CUDA graph the
// second time it sees that shape, and from then on a call of the same shape
// fills the scene table and uniforms into the parameter of the graph's first
// kernel (k_stage_param, which writes them to the shape's device staging)
// and replays the graph: one parameter update and one graph launch.  The
// staging travels with the launch, so the host keeps no ring of page-locked
// slots and never waits for one; on GB300 the former copy of a page-locked
// slot ahead of each replay took 32.5 us of device time per 640x480 sphere
// frame, the parameter 28.7 us.  A shape is
// everything that decides the launches and their arguments: the scene record
// without its buffer pointers, the uniform size, the launch shape
// (euc_tuning), and the context's scratch buffers (a render that moved them
// retires the shape's graph).  Ordered-path scenes (which synchronise),
// profiled renders and scenes whose staging exceeds the parameter stay on the
// plain path.
// ---------------------------------------------------------------------------
constexpr size_t kShapeCap = 512;  // recorded shapes of a context at most (least recently used go)
constexpr size_t kSightCap = 4096; // shapes counted before the count starts over
constexpr size_t kStageParamBytes = 1008;  // one scene's table, bases and uniforms (at most 256 + 64 + 512)

struct alignas(16) StageParam {
    uint32_t n, pad[3];                  // bytes of b to write (a multiple of 16)
    unsigned char b[kStageParamBytes];  // the staging, laid out as run_batch reads it
};

// The first node of a recorded shape: writes its parameter's staging bytes
// to the shape's device staging.
__global__ void __launch_bounds__(64) k_stage_param(const __grid_constant__ StageParam p, unsigned char *__restrict__ dst) {
    for (uint32_t i = threadIdx.x * 16u; i < p.n; i += blockDim.x * 16u)
        *reinterpret_cast<uint4 *>(dst + i) = *reinterpret_cast<const uint4 *>(p.b + i);
}

struct ShapeGraph {
    std::vector<unsigned char> key;
    void *scratch[kScratchBufs] = {};
    StageParam param;               // the next replay's staging
    void *dev = nullptr;            // the staging the graph's kernels read
    size_t need = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t stage_node = nullptr;  // the k_stage_param node
    cudaKernelNodeParams stage_kp = {};
    cudaEvent_t done = nullptr;  // after the last replay
    bool launched = false;
    uint64_t launches = 0, last_use = 0;
};

namespace {

void shape_free(ShapeGraph *g) {
    if (g->launched) cudaEventSynchronize(g->done);
    if (g->done) cudaEventDestroy(g->done);
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    if (g->dev) cudaFree(g->dev);
    delete g;
}

void free_shapes(euc_ctx *ctx) {
    for (ShapeGraph *g : ctx->shapes) shape_free(g);
    ctx->shapes.clear();
    ctx->sightings.clear();
}

std::vector<unsigned char> shape_key(const euc_ctx *ctx, const Plan &p) {
    SceneDev d = p.d;  // plan_scene zeroed the padding
    d.verts = nullptr;
    d.idx = nullptr;
    d.uniforms = nullptr;
    d.pixel = nullptr;
    d.depth = nullptr;
    std::vector<unsigned char> k(sizeof(d) + sizeof(p.usize) + sizeof(euc_tuning));
    std::memcpy(k.data(), &d, sizeof(d));
    std::memcpy(k.data() + sizeof(d), &p.usize, sizeof(p.usize));
    std::memcpy(k.data() + sizeof(d) + sizeof(p.usize), &ctx->tune, sizeof(euc_tuning));
    return k;
}

// Records the launches of scene `s` as a new shape; nullptr when it cannot.
ShapeGraph *shape_record(euc_ctx *ctx, const euc_scene &s, std::vector<unsigned char> key) {
    StageOverride so;
    so.dry = true;
    if (run_batch(ctx, &s, 1, nullptr, &so)) return nullptr;  // validates, sizes the scratch
    if (so.need > kStageParamBytes) return nullptr;  // too large for the parameter: plain path
    ShapeGraph *g = new (std::nothrow) ShapeGraph();
    if (!g) return nullptr;
    g->key = std::move(key);
    g->need = so.need;
    g->param.n = (uint32_t)so.need;
    bool ok = cudaMalloc(&g->dev, std::max<size_t>(g->need, 16)) == cudaSuccess &&
              cudaEventCreateWithFlags(&g->done, cudaEventDisableTiming) == cudaSuccess;
    cudaStream_t cs = nullptr;
    ok = ok && cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess;
    if (ok && cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        so.dry = false;
        so.no_copy = true;
        so.host = g->param.b;
        so.dev = g->dev;
        so.need = g->need;
        ctx->capturing = true;
        const uint64_t l0 = ctx->launches;
        k_stage_param<<<1, 64, 0, cs>>>(g->param, (unsigned char *)g->dev);
        const int rc = run_batch(ctx, &s, 1, cs, &so);
        g->launches = ctx->launches - l0 + 1;
        ctx->launches = l0;
        ctx->capturing = false;
        cudaGraph_t graph = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(cs, &graph);
        g->graph = graph;
        // the staging node is the graph's only root
        size_t nroot = 1;
        ok = rc == EUC_OK && ec == cudaSuccess && graph &&
             cudaGraphGetRootNodes(graph, &g->stage_node, &nroot) == cudaSuccess && nroot == 1 &&
             cudaGraphKernelNodeGetParams(g->stage_node, &g->stage_kp) == cudaSuccess &&
             g->stage_kp.func == (void *)k_stage_param &&
             cudaGraphInstantiate(&g->exec, g->graph, 0) == cudaSuccess;
    } else {
        ok = false;
    }
    if (cs) cudaStreamDestroy(cs);
    (void)cudaGetLastError();
    if (!ok) {
        shape_free(g);
        return nullptr;
    }
    scratch_ptrs(ctx, g->scratch);
    return g;
}

int render_one(euc_ctx *ctx, const euc_scene &s, cudaStream_t st) {
    Plan p;
    if (int rc = plan_scene(s, p)) return rc;
    if (ctx->profiling || p.skip || p.d.keytype == KEY_ORDERED) return run_batch(ctx, &s, 1, st);
    std::vector<unsigned char> key = shape_key(ctx, p);
    ShapeGraph *g = nullptr;
    size_t at = 0;
    for (; at < ctx->shapes.size(); ++at)
        if (ctx->shapes[at]->key == key) {
            g = ctx->shapes[at];
            break;
        }
    if (g) {
        void *now[kScratchBufs];
        scratch_ptrs(ctx, now);
        if (std::memcmp(now, g->scratch, sizeof(now)) != 0) {  // the scratch moved: record again
            shape_free(g);
            ctx->shapes.erase(ctx->shapes.begin() + (long)at);
            g = nullptr;
        }
    }
    if (!g) {
        if (ctx->sightings.size() >= kSightCap) ctx->sightings.clear();
        if (++ctx->sightings[key] < 2) return run_batch(ctx, &s, 1, st);  // seen once: plain
        if (ctx->shapes.size() >= kShapeCap) {  // make room: the least recently used goes
            size_t lru = 0;
            for (size_t i = 1; i < ctx->shapes.size(); ++i)
                if (ctx->shapes[i]->last_use < ctx->shapes[lru]->last_use) lru = i;
            shape_free(ctx->shapes[lru]);
            ctx->shapes.erase(ctx->shapes.begin() + (long)lru);
        }
        g = shape_record(ctx, s, key);
        if (!g) return run_batch(ctx, &s, 1, st);
        ctx->shapes.push_back(g);
    }
    g->last_use = ++ctx->shape_clock;
    StageOverride so;
    so.fill = true;
    so.host = g->param.b;
    so.dev = g->dev;
    so.need = g->need;
    if (int rc = run_batch(ctx, &s, 1, st, &so)) return rc;
    // the parameter is copied here; replays already enqueued keep theirs
    void *args[2] = {&g->param, &g->dev};
    cudaKernelNodeParams kp = g->stage_kp;
    kp.kernelParams = args;
    kp.extra = nullptr;
    CUDA_TRY(cudaGraphExecKernelNodeSetParams(g->exec, g->stage_node, &kp));
    if (g->launched) CUDA_TRY(cudaStreamWaitEvent(st, g->done, 0));  // a replay on another stream has finished
    CUDA_TRY(cudaGraphLaunch(g->exec, st));
    CUDA_TRY(cudaEventRecord(g->done, st));
    g->launched = true;
    ctx->launches += g->launches;
    return EUC_OK;
}

}  // namespace

extern "C" {

int euc_graph_create(euc_ctx *ctx, const euc_scene *scenes, size_t n, euc_graph **out) {
    if (!ctx || !out || (n && !scenes)) return EUC_ERR_INVALID;
    *out = nullptr;
    std::lock_guard<std::mutex> lk(ctx->mu);
    CUDA_TRY(cudaSetDevice(ctx->device));
    StageOverride so;
    so.dry = true;
    int rc = run_batch(ctx, scenes, n, nullptr, &so);  // validates, sizes the scratch
    if (rc) return rc;
    euc_graph *g = new (std::nothrow) euc_graph();
    if (!g) return EUC_ERR_OOM;
    g->ctx = ctx;
    const size_t bytes = std::max<size_t>(so.need, 256);
    if (cudaMallocHost(&g->host, bytes) != cudaSuccess || cudaMalloc(&g->dev, bytes) != cudaSuccess) {
        (void)cudaGetLastError();
        graph_free(g);
        return EUC_ERR_OOM;
    }
    cudaStream_t cs = nullptr;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) {
        (void)cudaGetLastError();
        graph_free(g);
        return EUC_ERR_CUDA;
    }
    so.dry = false;
    so.host = g->host;
    so.dev = g->dev;
    so.need = bytes;
    rc = EUC_ERR_CUDA;
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        ctx->capturing = true;
        const uint64_t l0 = ctx->launches;
        rc = run_batch(ctx, scenes, n, cs, &so);
        g->launches = ctx->launches - l0;
        ctx->launches = l0;
        ctx->capturing = false;
        cudaGraph_t graph = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(cs, &graph);
        g->graph = graph;
        if (rc == EUC_OK && (ec != cudaSuccess || !graph)) rc = EUC_ERR_CUDA;
    }
    if (rc == EUC_OK && cudaGraphInstantiate(&g->exec, g->graph, 0) != cudaSuccess) rc = EUC_ERR_CUDA;
    (void)cudaGetLastError();
    cudaStreamDestroy(cs);
    if (rc) {
        graph_free(g);
        return rc;
    }
    g->nscenes = ctx->last_nscenes;
    scratch_ptrs(ctx, g->scratch);
    *out = g;
    return EUC_OK;
}

int euc_graph_launch(euc_graph *g, void *stream) {
    if (!g || !g->exec) return EUC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(g->ctx->mu);
    void *now[kScratchBufs];
    scratch_ptrs(g->ctx, now);
    if (memcmp(now, g->scratch, sizeof(now)) != 0) return EUC_ERR_STALE;
    CUDA_TRY(cudaSetDevice(g->ctx->device));
    CUDA_TRY(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
    g->ctx->last_nscenes = g->nscenes;
    g->ctx->launches += g->launches;
    return EUC_OK;
}

int euc_graph_destroy(euc_graph *g) {
    if (!g) return EUC_ERR_INVALID;
    cudaSetDevice(g->ctx->device);
    cudaDeviceSynchronize();
    graph_free(g);
    return EUC_OK;
}

int euc_texture_ingest(euc_ctx *ctx, const void *src, uint32_t width, uint32_t height, uint64_t src_pitch,
                       uint32_t src_format, void *dst, uint64_t dst_pitch, void *stream) {
    if (!ctx || !src || !dst || width < 1 || height < 1 || src_format > EUC_SRC_R32F) return EUC_ERR_INVALID;
    const uint32_t sbpp = src_bpp(src_format);
    const uint64_t srow = (uint64_t)width * sbpp, drow = (uint64_t)width * 4;
    if (!src_pitch) src_pitch = srow;
    if (!dst_pitch) dst_pitch = drow;
    if (src_pitch < srow || dst_pitch < drow || (dst_pitch & 3) || ((uintptr_t)dst & 3)) return EUC_ERR_INVALID;
    if (src_format == EUC_SRC_R32F && ((src_pitch & 3) || ((uintptr_t)src & 3))) return EUC_ERR_INVALID;
    std::lock_guard<std::mutex> g(ctx->mu);
    CUDA_TRY(cudaSetDevice(ctx->device));
    const cudaStream_t st = (cudaStream_t)stream;
    cudaPointerAttributes attr{};
    const bool on_device = cudaPointerGetAttributes(&attr, src) == cudaSuccess &&
                           (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged);
    (void)cudaGetLastError();
    const uint8_t *from = (const uint8_t *)src;
    uint64_t pitch = src_pitch;
    if (!on_device) {  // stage the rows, packed, through the context
        int rc;
        if ((rc = grow(ctx->h_tex[0], srow * height))) return rc;
        CUDA_TRY(cudaMemcpy2DAsync(ctx->h_tex[0].p, srow, src, src_pitch, srow, height, cudaMemcpyHostToDevice, st));
        from = (const uint8_t *)ctx->h_tex[0].p;
        pitch = srow;
    }
    const dim3 grid((unsigned)((width + 31) / 32), (unsigned)std::min<uint32_t>(height, 65535u));
    k_ingest<<<grid, dim3(32, 8), 0, st>>>(from, pitch, src_format, (uint8_t *)dst, dst_pitch, width, height);
    ctx->launches += 1;
    CUDA_TRY(cudaGetLastError());
    if (!on_device) CUDA_TRY(cudaStreamSynchronize(st));  // the staging is reused by the next call
    return EUC_OK;
}

int euc_sample_nearest(const void *texels, uint32_t ndim, const uint32_t *size, uint32_t texel_bytes, uint32_t wrap,
                       const float *queries, uint64_t count, void *out, void *stream) {
    if (!size || ndim < 1 || ndim > 4 || texel_bytes < 1 || texel_bytes > 16 || wrap > EUC_WRAP_MIRROR)
        return EUC_ERR_INVALID;
    uint32_t sz[4] = {1, 1, 1, 1};
    for (uint32_t a = 0; a < ndim; ++a) {
        if (size[a] < 1) return EUC_ERR_INVALID;  // Denormalize's `scale - 1` underflows on an empty axis
        sz[a] = size[a];
    }
    if (!count) return EUC_OK;
    if (!texels || !queries || !out) return EUC_ERR_INVALID;
    const cudaStream_t st = (cudaStream_t)stream;
    int nsm = 0, dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const uint64_t blocks = std::min<uint64_t>((count + kBlock - 1) / kBlock, (uint64_t)nsm * 16);
    k_sample_nearest<<<(unsigned)blocks, kBlock, 0, st>>>((const uint8_t *)texels, ndim,
                                                          make_uint4(sz[0], sz[1], sz[2], sz[3]), texel_bytes, wrap,
                                                          queries, count, (uint8_t *)out);
    CUDA_TRY(cudaGetLastError());
    return EUC_OK;
}

}  // extern "C"

namespace {

// Host-side copies for the host-buffer renders: the jobs are split into
// 1 MiB pieces that `threads` host threads take in turn (0: the hardware
// concurrency, at most 16); small totals stay on the calling thread.
struct CopyJob {
    void *dst;
    const void *src;
    size_t bytes;
};

void parallel_copy(const std::vector<CopyJob> &jobs, int threads) {
    constexpr size_t kPiece = 1u << 20;
    size_t total = 0;
    for (const CopyJob &j : jobs) total += j.bytes;
    if (threads <= 0) {
        const unsigned hc = std::thread::hardware_concurrency();
        threads = hc ? (int)std::min(hc, 16u) : 1;
    }
    if (threads <= 1 || total < 4 * kPiece) {
        for (const CopyJob &j : jobs)
            if (j.bytes) std::memcpy(j.dst, j.src, j.bytes);
        return;
    }
    std::vector<CopyJob> pieces;
    for (const CopyJob &j : jobs)
        for (size_t o = 0; o < j.bytes; o += kPiece)
            pieces.push_back({(char *)j.dst + o, (const char *)j.src + o, std::min(kPiece, j.bytes - o)});
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (size_t i; (i = next.fetch_add(1)) < pieces.size();) std::memcpy(pieces[i].dst, pieces[i].src, pieces[i].bytes);
    };
    std::vector<std::thread> pool;
    const size_t nt = std::min<size_t>((size_t)threads, pieces.size());
    for (size_t t = 1; t < nt; ++t) {
        try {
            pool.emplace_back(work);
        } catch (...) {
            break;  // fewer helpers; the calling thread still finishes every piece
        }
    }
    work();
    for (std::thread &th : pool) th.join();
}

// Sampler k (0: the texture, 1: Phong's shadow map) in a scene's copy of its
// uniforms.
euc_sampler *sampler_of(const euc_scene &sc, unsigned char *uni, int k) {
    if (k == 0)
        return sc.desc.shader == EUC_SHADER_TEXTURED ? &((euc_textured_uniforms *)uni)->tex
                                                     : &((euc_phong_uniforms *)uni)->tex;
    return &((euc_phong_uniforms *)uni)->shadow;
}

// The first device-side error (an index out of bounds) of the last batch,
// after its stream has been synchronised.
int first_scene_error(euc_ctx *ctx) {
    if (!ctx->last_nscenes) return EUC_OK;
    std::vector<int> e(ctx->last_nscenes);
    CUDA_TRY(cudaMemcpy(e.data(), ctx->err.p, e.size() * sizeof(int), cudaMemcpyDeviceToHost));
    for (int v : e)
        if (v) return v;
    return EUC_OK;
}

// Scenes whose vertex, index, texture (inside the uniforms) and target
// pointers are host memory, rendered as one batch.  On a device that reads
// pageable host memory, the kernels use the vertices, indices and targets
// where they lie, and one k_copy_pieces launch gathers the textures (sampled
// many times each) into a device arena.  Elsewhere, host threads stage every
// input and target into page-locked memory, one copy moves each direction,
// and the targets are copied back.  A scene that fails draws nothing; the
// others are drawn, as in euc_render_batch.
int host_batch(euc_ctx *ctx, const euc_scene *scenes, size_t n, int threads) {
    struct Region {
        const void *src;
        size_t bytes, off;
    };
    struct alignas(16) UniBuf {
        unsigned char b[512];
        unsigned char *data() { return b; }
    };
    std::vector<euc_scene> dev(scenes, scenes + n);
    std::vector<UniBuf> unis(n);
    std::vector<Region> in, out;
    std::vector<size_t> voff(n, SIZE_MAX), ioff(n, SIZE_MAX), poff(n, SIZE_MAX), doff(n, SIZE_MAX);
    std::vector<std::array<size_t, 2>> toff(n, {SIZE_MAX, SIZE_MAX});
    std::map<const void *, size_t> shared_tex;
    size_t off = 0;
    auto place = [&](std::vector<Region> &list, const void *src, size_t bytes) {
        const size_t at = off;
        list.push_back({src, bytes, at});
        off = pad_up(off + bytes, 256);
        return at;
    };
    static_assert(sizeof(euc_phong_uniforms) <= 512, "uniform copies hold any shader's struct");
    const bool direct = ctx->pageable && ctx->tune.host_copy != EUC_HOST_COPY_STAGED;
    for (size_t i = 0; i < n; ++i) {
        const euc_scene &sc = scenes[i];
        Plan p;
        if (int rc = plan_scene(sc, p)) return rc;
        const size_t need = uniforms_size_for(sc.desc.shader);
        std::memcpy(unis[i].data(), sc.uniforms, need);
        dev[i].uniforms = unis[i].data();
        dev[i].uniforms_size = need;
        if (p.skip) continue;
        const size_t vb = (size_t)sc.nverts * sc.layout.stride;
        if (vb && !direct) voff[i] = place(in, sc.vertices, vb);
        if (sc.indices && sc.nindices && !direct) ioff[i] = place(in, sc.indices, (size_t)sc.nindices * 4);
        const int nsamp = sc.desc.shader == EUC_SHADER_PHONG ? 2 : sc.desc.shader == EUC_SHADER_TEXTURED ? 1 : 0;
        for (int k = 0; k < nsamp; ++k) {
            const euc_sampler *smp = sampler_of(sc, unis[i].data(), k);
            if (!smp->data) continue;
            const size_t pitch = smp->pitch ? smp->pitch : (size_t)smp->width * 4;
            const size_t bytes = pitch * smp->height;
            auto it = shared_tex.find(smp->data);
            toff[i][k] = it != shared_tex.end() ? it->second : (shared_tex[smp->data] = place(in, smp->data, bytes));
        }
    }
    const size_t targets_at = off;  // targets last: one copy back covers them all
    for (size_t i = 0; i < n && !direct; ++i) {
        const euc_scene &sc = scenes[i];
        if (sc.pixel.data) {
            const uint32_t bpp = fmt_bpp(sc.pixel.format);
            if (!bpp) return EUC_ERR_INVALID;
            const size_t pitch = sc.pixel.pitch ? sc.pixel.pitch : (size_t)sc.pixel.width * bpp;
            poff[i] = place(out, sc.pixel.data, pitch * sc.pixel.height);
        }
        if (sc.depth.data) {
            const size_t pitch = sc.depth.pitch ? sc.depth.pitch : (size_t)sc.depth.width * 4;
            doff[i] = place(out, sc.depth.data, pitch * sc.depth.height);
        }
    }
    // direct: the texture piece table follows the regions
    constexpr size_t kPiece = 128u << 10;
    std::vector<CopyPiece> pieces;
    size_t tab = 0, total = std::max<size_t>(off, 256);
    if (direct) {
        for (const Region &r : in)
            for (size_t o = 0; o < r.bytes; o += kPiece)
                pieces.push_back({(const uint8_t *)r.src + o, nullptr, std::min(kPiece, r.bytes - o)});
        tab = pad_up(off, 256);
        total = tab + pieces.size() * sizeof(CopyPiece) + 256;
    }
    int rc;
    if ((rc = grow(ctx->h_arena, total))) return rc;
    if (direct) {
        unsigned char *d = (unsigned char *)ctx->h_arena.p;
        size_t k = 0;
        for (const Region &r : in)
            for (size_t o = 0; o < r.bytes; o += kPiece) pieces[k++].dst = d + r.off + o;
        for (size_t i = 0; i < n; ++i)
            for (int t = 0; t < 2; ++t)
                if (toff[i][t] != SIZE_MAX) sampler_of(dev[i], unis[i].data(), t)->data = d + toff[i][t];
        if (!pieces.empty()) {
            CUDA_TRY(cudaMemcpyAsync(d + tab, pieces.data(), pieces.size() * sizeof(CopyPiece), cudaMemcpyHostToDevice,
                                     nullptr));
            k_copy_pieces<<<(unsigned)std::min<size_t>(pieces.size(), (size_t)ctx->nsm * 4), kBlock, 0, nullptr>>>(
                (const CopyPiece *)(d + tab), (uint32_t)pieces.size());
            CUDA_TRY(cudaGetLastError());
            ctx->launches += 1;
        }
        // the kernels use the caller's buffers: none may still run when this returns
        rc = run_batch(ctx, dev.data(), n, nullptr);
        CUDA_TRY(cudaStreamSynchronize(nullptr));
        return rc ? rc : first_scene_error(ctx);
    }
    if (ctx->h_pinned.cap < total) {
        if (ctx->h_pinned.p) CUDA_TRY(cudaFreeHost(ctx->h_pinned.p));
        ctx->h_pinned.p = nullptr;
        ctx->h_pinned.cap = 0;
        CUDA_TRY(cudaMallocHost(&ctx->h_pinned.p, total));
        ctx->h_pinned.cap = total;
    }
    unsigned char *d = (unsigned char *)ctx->h_arena.p, *h = (unsigned char *)ctx->h_pinned.p;
    for (size_t i = 0; i < n; ++i) {
        if (voff[i] != SIZE_MAX) dev[i].vertices = d + voff[i];
        if (ioff[i] != SIZE_MAX) dev[i].indices = (const uint32_t *)(d + ioff[i]);
        if (poff[i] != SIZE_MAX) dev[i].pixel.data = d + poff[i];
        if (doff[i] != SIZE_MAX) dev[i].depth.data = d + doff[i];
        for (int t = 0; t < 2; ++t)
            if (toff[i][t] != SIZE_MAX) sampler_of(dev[i], unis[i].data(), t)->data = d + toff[i][t];
    }
    std::vector<CopyJob> jobs;
    for (const Region &r : in) jobs.push_back({h + r.off, r.src, r.bytes});
    for (const Region &r : out) jobs.push_back({h + r.off, r.src, r.bytes});
    parallel_copy(jobs, threads);
    CUDA_TRY(cudaMemcpyAsync(d, h, off, cudaMemcpyHostToDevice, nullptr));
    if ((rc = run_batch(ctx, dev.data(), n, nullptr))) {
        CUDA_TRY(cudaStreamSynchronize(nullptr));  // the next call refills the staging
        return rc;
    }
    if (off > targets_at)
        CUDA_TRY(cudaMemcpyAsync(h + targets_at, d + targets_at, off - targets_at, cudaMemcpyDeviceToHost, nullptr));
    CUDA_TRY(cudaStreamSynchronize(nullptr));
    // a scene that failed on the device drew nothing: its targets come back
    // as they went up
    jobs.clear();
    for (const Region &r : out) jobs.push_back({const_cast<void *>(r.src), h + r.off, r.bytes});
    parallel_copy(jobs, threads);
    return first_scene_error(ctx);
}

}  // namespace

extern "C" {

int euc_render_host(euc_ctx *ctx, const euc_pipeline_desc *desc, const void *uniforms, size_t uniforms_size,
                    const euc_vertex_layout *layout, const void *vertices, size_t nverts, const uint32_t *indices,
                    size_t nindices, const euc_target *pixel, const euc_target *depth) {
    if (!ctx || !desc || !layout || !uniforms) return EUC_ERR_INVALID;
    euc_scene sc;
    std::memset(&sc, 0, sizeof(sc));
    sc.desc = *desc;
    sc.layout = *layout;
    sc.vertices = vertices;
    sc.nverts = nverts;
    sc.indices = indices;
    sc.nindices = indices ? nindices : 0;
    if (pixel) sc.pixel = *pixel;
    if (depth) sc.depth = *depth;
    sc.uniforms = uniforms;
    sc.uniforms_size = uniforms_size;
    return euc_render_host_batch(ctx, &sc, 1, 0);
}

int euc_render_host_batch(euc_ctx *ctx, const euc_scene *scenes, size_t n, int threads) {
    if (!ctx || (n && !scenes)) return EUC_ERR_INVALID;
    if (!n) return EUC_OK;
    std::lock_guard<std::mutex> g(ctx->mu);
    CUDA_TRY(cudaSetDevice(ctx->device));
    return host_batch(ctx, scenes, n, threads);
}
}  // extern "C"

// ===========================================================================
// euc_render_noalloc: one render that allocates nothing.
//
// Some callers cannot let a library allocate device memory.  An engine or a
// plugin host may reserve its whole device-memory budget at start-up and give
// libraries only the buffers they must touch.  A latency-critical render
// thread cannot afford cudaMalloc or cudaFree, because both synchronise the
// whole device.  An euc_ctx grows its scratch buffers on demand, so such a
// caller cannot use euc_render.  This entry point takes the same inputs and
// outputs but keeps all of its scratch in one fixed array of this file,
// g_noalloc_scratch (kNaBytes, about 21.0 MiB).  Every GPU that loads this
// library holds that array until the process exits.
//
// Limits: at most kNaMaxVerts vertices, kNaMaxGroups primitive slots (one
// per triangle, one per line, three per triangle of a LineTriangleList) and
// kNaMaxPixels target pixels; larger scenes are rejected with
// EUC_ERR_CAPACITY before anything is enqueued.  The scene table and the
// uniforms reach the device as a kernel parameter, so nothing of the
// caller's host memory is read once the call has returned.
//
// Every call uses the same array and leaves its contents behind for the next
// call.  Each call clears on its stream the parts that must start at zero
// (error flag, counters).  Two calls whose work overlaps on the GPU (calls on
// different streams, or from different host threads without ordering) race on
// the array and corrupt each other's results: issue them on one stream.
//
// Set-up: the first call on a device looks up the array's device address for
// that device (cudaGetSymbolAddress, with that device current) and caches it
// with the CUDA context it was found in; a call in another context (after
// cudaDeviceReset) looks it up again.  The first call on a device, and the
// first after a reset, should come before any stream capture begins.
// ===========================================================================
namespace {

constexpr uint64_t kNaMaxVerts = 65536;
constexpr uint64_t kNaMaxGroups = 65536;
constexpr uint64_t kNaMaxPixels = 1ull << 20;
constexpr int kNaMaxNV = vd_stride(11);  // PhongFn::NV, the largest VertexData, padded
constexpr size_t kNaStage = 4096;  // scene table, bases, uniforms
constexpr size_t kNaOffErr = kNaStage;
constexpr size_t kNaOffStats = kNaOffErr + 256;
constexpr size_t kNaOffTotals = kNaOffStats + 256;
constexpr size_t kNaOffCov = kNaOffTotals + 64;   // inside the 256-byte totals region
constexpr size_t kNaOffPlan = kNaOffTotals + 128;  // plan_chunks's 2 x 2 chunk bases, same region
constexpr size_t kNaOffClip = kNaOffTotals + 256;
constexpr size_t kNaOffVdata = kNaOffClip + kNaMaxVerts * sizeof(float4);
constexpr size_t kNaOffRecs = kNaOffVdata + kNaMaxVerts * kNaMaxNV * sizeof(float);
constexpr size_t kNaOffRows = kNaOffRecs + kNaMaxGroups * sizeof(TriRec);
constexpr size_t kNaOffChunks = kNaOffRows + kNaMaxGroups * sizeof(uint32_t);
constexpr size_t kNaOffLiveTri = kNaOffChunks + (kNaMaxGroups / kBlock) * sizeof(uint2);
constexpr size_t kNaOffLiveOff = kNaOffLiveTri + kNaMaxGroups * sizeof(uint32_t);
constexpr size_t kNaOffVbuf = kNaOffLiveOff + kNaMaxGroups * sizeof(uint64_t);
constexpr size_t kNaBytes = kNaOffVbuf + kNaMaxPixels * sizeof(unsigned long long);
static_assert(kNaOffClip % 256 == 0 && kNaOffVdata % 256 == 0 && kNaOffRecs % 256 == 0 && kNaOffRows % 256 == 0 &&
                  kNaOffChunks % 256 == 0 && kNaOffLiveTri % 256 == 0 && kNaOffLiveOff % 256 == 0 &&
                  kNaOffVbuf % 256 == 0,
              "scratch regions must stay 256-byte aligned");
static_assert(kNaMaxVerts % kBlock == 0 && kNaMaxGroups % kBlock == 0 && kNaMaxPixels % kBlock == 0,
              "limits must be whole blocks");

constexpr int kNaMaxDevices = 64;
std::mutex g_na_mu;
unsigned char *g_na_ptr[kNaMaxDevices];
CUcontext g_na_ctx[kNaMaxDevices];  // the context each address was looked up in
int g_na_nsm[kNaMaxDevices];

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

namespace {

// The driver's cuCtxGetCurrent, found through the runtime (no link to the
// driver library); nullptr when the driver does not offer it.
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
CtxGetCurrentFn ctx_get_current() {
    static CtxGetCurrentFn fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            (void)cudaGetLastError();
            f = nullptr;
        }
        return (CtxGetCurrentFn)f;
    }();
    return fn;
}

// Device address of g_noalloc_scratch on the current device: looked up once
// per device and context, so that after a cudaDeviceReset (a new primary
// context, the module loaded again) it is looked up again.
int na_scratch(int dev, unsigned char **ptr, int *nsm) {
    CUcontext cur = nullptr;
    if (CtxGetCurrentFn f = ctx_get_current())
        if (f(&cur) != CUDA_SUCCESS) cur = nullptr;
    std::lock_guard<std::mutex> g(g_na_mu);
    if (!g_na_ptr[dev] || g_na_ctx[dev] != cur) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            (void)cudaGetLastError();
            return EUC_ERR_CUDA;
        }
        int n = 0;
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess || n <= 0) {
            (void)cudaGetLastError();
            return EUC_ERR_CUDA;
        }
        g_na_ptr[dev] = (unsigned char *)p;
        g_na_ctx[dev] = cur;
        g_na_nsm[dev] = n;
    }
    *ptr = g_na_ptr[dev];
    *nsm = g_na_nsm[dev];
    return EUC_OK;
}

thread_local int t_na_nsm = 1;  // SM count of the device of the current call

// A call's scene table, zero bases and uniforms, handed to the device as a
// kernel parameter (no host memory is read after the call returns).
struct NaStage {
    SceneDev d;
    uint64_t zero[6];             // the vertex / primitive / pixel bases of one scene
    alignas(16) unsigned char uni[512];
};
static_assert(sizeof(euc_phong_uniforms) <= sizeof(NaStage::uni), "uniform copies hold any shader's struct");

// Writes the stage into the scratch array: the scene at 0, the zero bases at
// `off_b`, the uniforms at `off_u` (`usize` bytes).
__global__ void k_na_stage(const NaStage st, unsigned char *__restrict__ a, uint32_t off_b, uint32_t off_u,
                           uint32_t usize) {
    const unsigned char *d = reinterpret_cast<const unsigned char *>(&st.d);
    for (uint32_t i = threadIdx.x; i < sizeof(SceneDev); i += blockDim.x) a[i] = d[i];
    const unsigned char *z = reinterpret_cast<const unsigned char *>(st.zero);
    for (uint32_t i = threadIdx.x; i < sizeof(st.zero); i += blockDim.x) a[off_b + i] = z[i];
    for (uint32_t i = threadIdx.x; i < usize; i += blockDim.x) a[off_u + i] = st.uni[i];
}

template <class F>
void na_vertex_resolve(bool vertex, const SceneDev *sc, const uint64_t *base, uint64_t nblk, unsigned char *a,
                       cudaStream_t st) {
    if (!nblk) return;
    if (vertex)
        k_vertex<F><<<(unsigned)nblk, kBlock, 0, st>>>(sc, base, 0, 1, 0, (float4 *)(a + kNaOffClip),
                                                       (float *)(a + kNaOffVdata), PrepArgs{});
    else
        k_resolve<F><<<chunk_grid(nblk, t_na_nsm), kBlock, 0, st>>>(
            sc, base, 0, 1, chunk_group(nblk, t_na_nsm), (const TriRec *)(a + kNaOffRecs),
            (const float *)(a + kNaOffVdata), (const unsigned long long *)(a + kNaOffVbuf), (const uint4 *)(a + kNaOffCov));
}

void na_dispatch(bool vertex, uint32_t shader, const SceneDev *sc, const uint64_t *base, uint64_t nblk,
                 unsigned char *a, cudaStream_t st) {
    switch (shader) {
    case EUC_SHADER_FLAT: na_vertex_resolve<FlatFn>(vertex, sc, base, nblk, a, st); break;
    case EUC_SHADER_VCOLOR: na_vertex_resolve<VColorFn>(vertex, sc, base, nblk, a, st); break;
    case EUC_SHADER_GOURAUD: na_vertex_resolve<GouraudFn>(vertex, sc, base, nblk, a, st); break;
    case EUC_SHADER_TEXTURED: na_vertex_resolve<TexturedFn>(vertex, sc, base, nblk, a, st); break;
    case EUC_SHADER_PHONG: na_vertex_resolve<PhongFn>(vertex, sc, base, nblk, a, st); break;
    case EUC_SHADER_SHADOW: na_vertex_resolve<ShadowFn>(vertex, sc, base, nblk, a, st); break;
    }
}

}  // namespace

extern "C" int euc_render_noalloc(const euc_pipeline_desc *desc, const void *uniforms, size_t uniforms_size,
                                  const euc_vertex_layout *layout, const void *vertices, size_t nverts,
                                  const uint32_t *indices, size_t nindices, const euc_target *pixel,
                                  const euc_target *depth, void *stream, int *device_status) {
    if (!desc || !layout) return EUC_ERR_INVALID;
    euc_scene sc;
    std::memset(&sc, 0, sizeof(sc));
    sc.desc = *desc;
    sc.layout = *layout;
    sc.vertices = vertices;
    sc.nverts = nverts;
    sc.indices = indices;
    sc.nindices = nindices;
    if (pixel) sc.pixel = *pixel;
    if (depth) sc.depth = *depth;
    sc.uniforms = uniforms;
    sc.uniforms_size = uniforms_size;
    Plan p;
    if (int rc = plan_scene(sc, p)) return rc;
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNaMaxDevices) return EUC_ERR_INVALID;
    unsigned char *a = nullptr;
    int nsm = 0;
    if (int rc = na_scratch(dev, &a, &nsm)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (p.skip) {
        if (device_status) CUDA_TRY(cudaMemsetAsync(device_status, 0, sizeof(int), st));
        return EUC_OK;
    }
    // order-dependent blends keep every fragment in lists whose size is only
    // known on the device; they need euc_render's growable buffers
    // ordered scenes size their fragment lists on the device; a geometry
    // stage's output vertices need room beyond the fixed vertex array
    if (p.d.keytype == KEY_ORDERED || p.d.geom != EUC_GEOM_NONE) return EUC_ERR_CAPACITY;
    if (p.d.nverts > kNaMaxVerts || p.d.ngroups > kNaMaxGroups || (uint64_t)p.d.W * p.d.H > kNaMaxPixels ||
        p.nv > (uint32_t)kNaMaxNV)
        return EUC_ERR_CAPACITY;
    const uint64_t vtx = pad_up(p.d.nverts, kBlock);
    const uint64_t tri = pad_up(std::max<uint64_t>(p.d.ngroups, 1), kBlock);
    const uint64_t pix = pad_up((uint64_t)p.d.W * p.d.H, kBlock);
    // scene table | vtx base | tri base | pix base | uniforms, written by a
    // kernel from its parameter
    const size_t off_b = pad_up(sizeof(SceneDev), 16);
    const size_t off_u = off_b + 3 * 16;
    static_assert((sizeof(SceneDev) + 15) / 16 * 16 + 3 * 16 + sizeof(euc_phong_uniforms) <= kNaStage,
                  "staging area too small");
    NaStage stage;
    std::memset(&stage, 0, sizeof(stage));
    SceneDev &d = stage.d;
    d = p.d;
    d.vtx_base = d.vd_base = d.tri_base = d.pix_base = 0;
    d.uniforms = a + off_u;
    std::memcpy(stage.uni, p.uniforms, p.usize);
    k_na_stage<<<1, 128, 0, st>>>(stage, a, (uint32_t)off_b, (uint32_t)off_u, (uint32_t)p.usize);
    const SceneDev *dsc = (const SceneDev *)a;
    const uint64_t *zero_base = (const uint64_t *)(a + off_b);  // every base is 0 for a single scene
    PrepArgs prep = {};
    prep.err = (int *)(a + kNaOffErr);
    prep.stats = (SceneStats *)(a + kNaOffStats);
    prep.cov = (uint4 *)(a + kNaOffCov);
    prep.chunk_sums = (uint2 *)(a + kNaOffChunks);
    prep.totals = (unsigned long long *)(a + kNaOffTotals);
    prep.nchunks = tri / kBlock;
    prep.n = std::max<uint64_t>(prep.nchunks, 2);
    prep.nsc = 1;
    k_prep<<<(unsigned)((prep.n + kBlock - 1) / kBlock), kBlock, 0, st>>>(prep);
    t_na_nsm = nsm;
    na_dispatch(true, d.shader, dsc, zero_base, vtx / kBlock, a, st);
    k_setup<<<(unsigned)(tri / kBlock), kBlock, 0, st>>>(dsc, nullptr, (const float4 *)(a + kNaOffClip),
                                                          (TriRec *)(a + kNaOffRecs), (uint32_t *)(a + kNaOffRows),
                                                          (uint2 *)(a + kNaOffChunks), (int *)(a + kNaOffErr),
                                                          (SceneStats *)(a + kNaOffStats), (uint4 *)(a + kNaOffCov),
                                                          nullptr, nullptr);
    uint64_t *const ibase = (uint64_t *)(a + kNaOffPlan), *const rbase = ibase + 2;
    const uint32_t nscan = (uint32_t)((tri + kScanBlock - 1) / kScanBlock);
    k_scan_plan<<<nscan + 1, kBlock, 0, st>>>((const uint32_t *)(a + kNaOffRows), (const uint2 *)(a + kNaOffChunks),
                                              tri, (uint32_t *)(a + kNaOffLiveTri), (uint64_t *)(a + kNaOffLiveOff),
                                              (unsigned long long *)(a + kNaOffTotals), nscan, dsc, 1,
                                              (const uint4 *)(a + kNaOffCov), ibase, rbase, nullptr, 0, nullptr, nullptr,
                                              nullptr);
    const uint64_t ichunks = (pix + kInitChunk - 1) / kInitChunk + 1;
    k_init<<<chunk_grid(ichunks, nsm), kBlock, 0, st>>>(dsc, ibase, 1, (const uint4 *)(a + kNaOffCov),
                                                         (unsigned long long *)(a + kNaOffVbuf),
                                                         chunk_group(ichunks, nsm));
    k_raster<<<(unsigned)(nsm * raster_blocks_per_sm()), kBlock, 0, st>>>(
        dsc, (const TriRec *)(a + kNaOffRecs), (const uint32_t *)(a + kNaOffLiveTri), (const uint64_t *)(a + kNaOffLiveOff),
        (unsigned long long *)(a + kNaOffTotals), (const int *)(a + kNaOffErr),
        (unsigned long long *)(a + kNaOffVbuf), (SceneStats *)(a + kNaOffStats), 0, nullptr, kWarpItems, false);
    na_dispatch(false, d.shader, dsc, rbase, resolve_blocks(d), a, st);
    if (device_status)
        CUDA_TRY(cudaMemcpyAsync(device_status, a + kNaOffErr, sizeof(int), cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(cudaGetLastError());
    return EUC_OK;
}
