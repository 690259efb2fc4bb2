// euc_oracle.cpp — CPU restatement of euc 0.6.0's triangle pipeline (and its
// line rasteriser).
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU pipeline:
// only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may
// load it.  The product (euc_gb300/) never links or calls it.
//
// PARITY UNPINNED: euc has no tests, golden vectors or fixtures, and no Rust
// toolchain exists here to run it.  This restatement follows euc's source op
// for op (citations below are file:line in euc 0.6.0) and is cross-checked
// against a second, independent pure-Python restatement (euc_pyref.py) and
// against hand-derived known answers, but not against euc's own output.
//
// Rust semantics that are reproduced explicitly:
//   * no FMA contraction (compile with -ffp-contract=off);
//   * f32::min/max ignore a NaN operand (IEEE minNum/maxNum = fmin/fmax);
//   * `as usize` / `as u8` saturate and map NaN to 0;
//   * f32::fract = x - trunc(x); f32::rem_euclid via fmod;
//   * usize arithmetic wraps (euc's Cargo profiles disable overflow checks).
//
// Example-shader arithmetic (vek Mat4*Vec4, normalize, reflect, derive_more
// Add/Mul) comes from third-party crates (vek 0.17, derive_more 0.99) that are
// not in the reference tree; the op order used here is the one documented in
// include/euc_gb300.h and is shared by the GPU functors.

#include "../include/euc_gb300.h"

#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <utility>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Rust scalar semantics
// ---------------------------------------------------------------------------
inline float rmin(float a, float b) { return std::fmin(a, b); }
inline float rmax(float a, float b) { return std::fmax(a, b); }

// `f as usize` (saturating, NaN -> 0), usize = u64.
inline uint64_t as_usize(float v) {
    if (std::isnan(v) || v < 1.0f) return 0;
    if (v >= 18446744073709551616.0f) return UINT64_MAX;
    return (uint64_t)v;
}

// `f as u8` (saturating, NaN -> 0).
inline uint8_t as_u8(float v) {
    if (std::isnan(v) || v < 1.0f) return 0;
    if (v >= 255.0f) return 255;
    return (uint8_t)(int)v;
}

inline float fract(float v) { return v - std::trunc(v); }

inline float rem_euclid(float x, float m) {
    float r = std::fmod(x, m);
    return r < 0.0f ? r + std::fabs(m) : r;
}

inline uint64_t clamp_u64(uint64_t v, uint64_t lo, uint64_t hi) {
    return v < lo ? lo : (v > hi ? hi : v);
}

// `f as isize` (saturating, NaN -> 0), isize = i64.
inline int64_t as_isize(float v) {
    if (std::isnan(v)) return 0;
    if (v >= 9.2233720368547758e18f) return INT64_MAX;
    if (v <= -9.2233720368547758e18f) return INT64_MIN;
    return (int64_t)v;
}
// f32::clamp with ordered, non-NaN bounds: a NaN input stays NaN.
inline float fclamp(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }
// isize subtraction and abs wrap (overflow checks are off in euc's profiles).
inline int64_t wsub(int64_t a, int64_t b) { return (int64_t)((uint64_t)a - (uint64_t)b); }
inline int64_t wabs(int64_t a) { return a < 0 ? (int64_t)(0 - (uint64_t)a) : a; }

// clipline 0.2 (a dependency of euc, not in the reference tree; its exact
// pixel sequence is not pinned here).  Restated as: the pixels of the
// Bresenham line from (x1, y1) to (x2, y2), both ends included, that lie in
// the inclusive window [wx1, wx2] x [wy1, wy2] (clipline's window clipping
// keeps exactly the unclipped line's pixels inside it).  The major axis is x
// when |dx| >= |dy|; after i major steps the minor offset is
//     m(i) = floor((2 |dminor| i + |dmajor| - 1) / (2 |dmajor|)),
// which is the classic error-term loop (error 2|dminor| - |dmajor|, minor
// step while the error is > 0).  Lines with |dx| or |dy| >= 2^30 draw
// nothing.
template <class Plot>
void bresenham_clipped(int64_t x1, int64_t y1, int64_t x2, int64_t y2, int64_t wx1, int64_t wy1, int64_t wx2,
                       int64_t wy2, Plot plot) {
    if (wx2 < wx1 || wy2 < wy1) return;
    const int64_t lim = (int64_t)1 << 30;
    if (x1 <= -lim || x1 >= lim || x2 <= -lim || x2 >= lim || y1 <= -lim || y1 >= lim || y2 <= -lim || y2 >= lim)
        return;
    const int64_t dx = x2 - x1, dy = y2 - y1;
    const bool xmaj = (dx < 0 ? -dx : dx) >= (dy < 0 ? -dy : dy);
    const int64_t a1 = xmaj ? x1 : y1, a2 = xmaj ? x2 : y2, b1 = xmaj ? y1 : x1;
    const int64_t dmaj = a2 - a1, dmin = xmaj ? dy : dx;
    const int64_t amaj = dmaj < 0 ? -dmaj : dmaj, amin = dmin < 0 ? -dmin : dmin;
    const int64_t smaj = dmaj < 0 ? -1 : 1, smin = dmin < 0 ? -1 : 1;
    const int64_t wa1 = xmaj ? wx1 : wy1, wa2 = xmaj ? wx2 : wy2, wb1 = xmaj ? wy1 : wx1, wb2 = xmaj ? wy2 : wx2;
    // major steps whose major coordinate lies in the window
    int64_t i_lo, i_hi;
    if (smaj > 0) { i_lo = wa1 - a1; i_hi = wa2 - a1; }
    else { i_lo = a1 - wa2; i_hi = a1 - wa1; }
    if (i_lo < 0) i_lo = 0;
    if (i_hi > amaj) i_hi = amaj;
    for (int64_t i = i_lo; i <= i_hi; ++i) {
        // |dmajor|, |dminor| < 2^31: the numerator stays below 2^64
        const int64_t m = amaj ? (int64_t)((2 * (uint64_t)amin * (uint64_t)i + (uint64_t)amaj - 1) /
                                           (2 * (uint64_t)amaj))
                               : 0;
        const int64_t a = a1 + smaj * i, b = b1 + smin * m;
        if (b < wb1 || b > wb2) continue;
        plot(xmaj ? a : b, xmaj ? b : a);
    }
}

// ---------------------------------------------------------------------------
// Vector helpers of the rasteriser (rasterizer/triangles.rs:309-367)
// ---------------------------------------------------------------------------
struct V3 { float v[3]; };

inline V3 cross3(V3 a, V3 b) {
    return {{a.v[1] * b.v[2] - a.v[2] * b.v[1], a.v[2] * b.v[0] - a.v[0] * b.v[2],
             a.v[0] * b.v[1] - a.v[1] * b.v[0]}};
}
inline V3 sub3(V3 a, V3 b) { return {{a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2]}}; }
inline V3 add3(V3 a, V3 b) { return {{a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2]}}; }
inline V3 scale3(V3 a, float s) { return {{a.v[0] * s, a.v[1] * s, a.v[2] * s}}; }
inline float dot3(V3 a, V3 b) { return a.v[0] * b.v[0] + a.v[1] * b.v[1] + a.v[2] * b.v[2]; }
inline float mag2(V3 a) { return a.v[0] * a.v[0] + a.v[1] * a.v[1] + a.v[2] * a.v[2]; }
inline float lerp(float a, float b, float t) { return a + t * (b - a); }

struct M3 { float m[3][3]; };

inline M3 matmul3(const M3 &a, const M3 &b) {
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j];
    return r;
}
inline V3 mat3_vec3(const M3 &m, V3 v) {
    V3 r;
    for (int i = 0; i < 3; ++i) r.v[i] = m.m[i][0] * v.v[0] + m.m[i][1] * v.v[1] + m.m[i][2] * v.v[2];
    return r;
}

// ---------------------------------------------------------------------------
// Shader maths shared by the example pipelines (documented op order)
// ---------------------------------------------------------------------------
inline void mat4_vec4(const float *m, const float v[4], float out[4]) {
    for (int r = 0; r < 4; ++r)
        out[r] = ((m[r * 4 + 0] * v[0] + m[r * 4 + 1] * v[1]) + m[r * 4 + 2] * v[2]) + m[r * 4 + 3] * v[3];
}
inline float sdot3(const float *a, const float *b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
inline void snormalize3(const float *a, float *out) {
    float len = std::sqrt(sdot3(a, a));
    out[0] = a[0] / len; out[1] = a[1] / len; out[2] = a[2] / len;
}

inline float ldf(const uint8_t *v, int32_t off, int i) {
    float f;
    std::memcpy(&f, v + off + 4 * i, 4);
    return f;
}

// ---------------------------------------------------------------------------
// Samplers (sampler/mod.rs:100-179, linear.rs:30-66, nearest.rs:27-33)
// ---------------------------------------------------------------------------
struct Texel { float c[4]; };

inline Texel read_texel(const euc_sampler &s, uint64_t x, uint64_t y) {
    uint32_t pitch = s.pitch;
    const uint8_t *base = (const uint8_t *)s.data;
    Texel t;
    if (s.format == EUC_FMT_R32F) {
        if (!pitch) pitch = s.width * 4;
        float f;
        std::memcpy(&f, base + y * pitch + x * 4, 4);
        t.c[0] = t.c[1] = t.c[2] = t.c[3] = f;
    } else {
        if (!pitch) pitch = s.width * 4;
        const uint8_t *p = base + y * pitch + x * 4;
        for (int i = 0; i < 4; ++i) t.c[i] = (float)p[i] / s.texel_div;  // texture.rs:84-94 map
    }
    return t;
}

inline float wrap_coord(uint32_t wrap, float e) {
    switch (wrap) {
    case EUC_WRAP_CLAMP: return rmin(rmax(e, 0.0f), 1.0f);          // mod.rs:113
    case EUC_WRAP_TILE: return rem_euclid(e, 1.0f);                 // mod.rs:137
    case EUC_WRAP_MIRROR:                                           // mod.rs:160-166
        return rem_euclid(e, 2.0f) >= 1.0f ? 1.0f - rem_euclid(e, 1.0f) : rem_euclid(e, 1.0f);
    default: return e;
    }
}

Texel sample2d(const euc_sampler &s, float u, float v) {
    u = wrap_coord(s.wrap, u);
    v = wrap_coord(s.wrap, v);
    const uint64_t w = s.width, h = s.height;
    if (s.filter == EUC_FILTER_NEAREST) {
        // Denormalize (math.rs:51-53): ((x * scale as f32).max(0.0) as usize).min(scale - 1)
        uint64_t ix = as_usize(rmax(u * (float)w, 0.0f));
        uint64_t iy = as_usize(rmax(v * (float)h, 0.0f));
        if (ix > w - 1) ix = w - 1;
        if (iy > h - 1) iy = h - 1;
        return read_texel(s, ix, iy);
    }
    // Linear (linear.rs:30-66)
    float itx = fract(u) * (float)w;
    float ity = fract(v) * (float)h;
    uint64_t px = as_usize(std::trunc(itx));
    uint64_t py = as_usize(std::trunc(ity));
    float fx = fract(itx);
    float fy = fract(ity);
    uint64_t p0x = px < w - 1 ? px : w - 1;
    uint64_t p0y = py < h - 1 ? py : h - 1;
    uint64_t p1x = (px + 1) < w - 1 ? px + 1 : w - 1;
    uint64_t p1y = (py + 1) < h - 1 ? py + 1 : h - 1;
    Texel t00 = read_texel(s, p0x, p0y);
    Texel t10 = read_texel(s, p1x, p0y);
    Texel t01 = read_texel(s, p0x, p1y);
    Texel t11 = read_texel(s, p1x, p1y);
    Texel out;
    for (int i = 0; i < 4; ++i) {
        float t0 = t00.c[i] * (1.0f - fy) + t01.c[i] * fy;
        float t1 = t10.c[i] * (1.0f - fy) + t11.c[i] * fy;
        out.c[i] = t0 * (1.0f - fx) + t1 * fx;
    }
    return out;
}

// ---------------------------------------------------------------------------
// Shader functors.  NV = VertexData floats, NF = Fragment floats.
// ---------------------------------------------------------------------------
struct FlatShader {
    static constexpr int NV = 1, NF = 4;
    const euc_flat_uniforms *u;
    const euc_vertex_layout *lay;
    void vertex(const uint8_t *v, float clip[4], float *vd) const {
        float p[4] = {ldf(v, lay->position, 0), ldf(v, lay->position, 1), ldf(v, lay->position, 2), 1.0f};
        mat4_vec4(u->mvp, p, clip);
        vd[0] = 0.0f;
    }
    void fragment(const float *, float *f) const {
        for (int i = 0; i < 4; ++i) f[i] = u->color[i];
    }
    float pack(float c) const { return c * 255.0f; }
};

struct VColorShader {  // examples/triangle.rs:14-25
    static constexpr int NV = 4, NF = 4;
    const euc_vcolor_uniforms *u;
    const euc_vertex_layout *lay;
    void vertex(const uint8_t *v, float clip[4], float *vd) const {
        float p[4] = {ldf(v, lay->position, 0), ldf(v, lay->position, 1), ldf(v, lay->position, 2),
                      ldf(v, lay->position, 3)};
        mat4_vec4(u->mvp, p, clip);
        const uint8_t *c = v + lay->color;
        for (int i = 0; i < 4; ++i) vd[i] = (float)c[i] / 255.0f;
    }
    void fragment(const float *vd, float *f) const {
        for (int i = 0; i < 4; ++i) f[i] = vd[i];
    }
    float pack(float c) const { return c * 255.0f; }  // (e * 255.0) as u8
};

struct GouraudShader {  // per-vertex Lambert, spinning_cube.rs-style blend
    static constexpr int NV = 3, NF = 4;
    const euc_gouraud_uniforms *u;
    const euc_vertex_layout *lay;
    void vertex(const uint8_t *v, float clip[4], float *vd) const {
        float p[4] = {ldf(v, lay->position, 0), ldf(v, lay->position, 1), ldf(v, lay->position, 2), 1.0f};
        mat4_vec4(u->mvp, p, clip);
        float n4[4] = {ldf(v, lay->normal, 0), ldf(v, lay->normal, 1), ldf(v, lay->normal, 2), 0.0f};
        float wn[4];
        mat4_vec4(u->model, n4, wn);
        float n[3];
        snormalize3(wn, n);
        float lambert = rmax(sdot3(n, u->to_light), 0.0f);
        float k = u->ambient + lambert * u->diffuse;
        for (int i = 0; i < 3; ++i) vd[i] = u->color[i] * k;
    }
    void fragment(const float *vd, float *f) const {
        f[0] = vd[0]; f[1] = vd[1]; f[2] = vd[2]; f[3] = 1.0f;
    }
    float pack(float c) const { return c * 255.0f; }
};

struct TexturedShader {  // examples/texture_mapping.rs:20-34
    static constexpr int NV = 2, NF = 4;
    const euc_textured_uniforms *u;
    const euc_vertex_layout *lay;
    void vertex(const uint8_t *v, float clip[4], float *vd) const {
        float p[4] = {ldf(v, lay->position, 0), ldf(v, lay->position, 1), ldf(v, lay->position, 2), 1.0f};
        mat4_vec4(u->mvp, p, clip);
        vd[0] = ldf(v, lay->uv, 0);
        vd[1] = ldf(v, lay->uv, 1);
    }
    void fragment(const float *vd, float *f) const {
        Texel t = sample2d(u->tex, vd[0], vd[1]);
        for (int i = 0; i < 4; ++i) f[i] = t.c[i];
    }
    float pack(float c) const { return c; }  // `e as u8`
};

struct PhongShader {  // examples/teapot.rs:69-141, plus a surface texture
    static constexpr int NV = 11, NF = 4;
    const euc_phong_uniforms *u;
    const euc_vertex_layout *lay;
    void vertex(const uint8_t *v, float clip[4], float *vd) const {
        float p[4] = {ldf(v, lay->position, 0), ldf(v, lay->position, 1), ldf(v, lay->position, 2), 1.0f};
        float wpos[4];
        mat4_vec4(u->model, p, wpos);
        float n4[4] = {ldf(v, lay->normal, 0) * u->normal_sign, ldf(v, lay->normal, 1) * u->normal_sign,
                       ldf(v, lay->normal, 2) * u->normal_sign, 0.0f};
        float wnorm[4];
        mat4_vec4(u->model, n4, wnorm);
        float wp1[4] = {wpos[0], wpos[1], wpos[2], 1.0f};
        float lvp4[4];
        mat4_vec4(u->light_vp, wp1, lvp4);
        float vpos[4];
        mat4_vec4(u->view, wpos, vpos);
        mat4_vec4(u->proj, vpos, clip);
        vd[0] = wpos[0]; vd[1] = wpos[1]; vd[2] = wpos[2];
        vd[3] = wnorm[0]; vd[4] = wnorm[1]; vd[5] = wnorm[2];
        vd[6] = lvp4[0] / lvp4[3]; vd[7] = lvp4[1] / lvp4[3]; vd[8] = lvp4[2] / lvp4[3];
        if (lay->uv >= 0) {
            vd[9] = ldf(v, lay->uv, 0);
            vd[10] = ldf(v, lay->uv, 1);
        } else {
            vd[9] = 0.0f;
            vd[10] = 0.0f;
        }
    }
    void fragment(const float *vd, float *f) const {
        float n[3], cam_dir[3], light_dir[3], t[3];
        snormalize3(vd + 3, n);
        for (int i = 0; i < 3; ++i) t[i] = u->cam_pos[i] - vd[i];
        snormalize3(t, cam_dir);
        for (int i = 0; i < 3; ++i) t[i] = vd[i] - u->light_pos[i];
        snormalize3(t, light_dir);
        float surf[4];
        if (u->tex.data) {
            Texel tx = sample2d(u->tex, vd[9], vd[10]);
            for (int i = 0; i < 4; ++i) surf[i] = tx.c[i];
        } else {
            for (int i = 0; i < 4; ++i) surf[i] = u->surf_color[i];
        }
        float nl[3] = {-light_dir[0], -light_dir[1], -light_dir[2]};
        float diffuse = rmax(sdot3(n, nl), 0.0f) * 0.5f;
        // reflect(v, n) = v - n * (d + d), d = dot(v, n)
        float d = sdot3(nl, n);
        float dd = d + d;
        float r[3] = {nl[0] - n[0] * dd, nl[1] - n[1] * dd, nl[2] - n[2] * dd};
        float nc[3] = {-cam_dir[0], -cam_dir[1], -cam_dir[2]};
        float specular = std::pow(rmax(sdot3(r, nc), 0.0f), 30.0f) * 3.0f;
        bool in_light = true;
        if (u->shadow.data) {
            float su = (vd[6] * 1.0f) * 0.5f + 0.5f;
            float sv = (vd[7] * -1.0f) * 0.5f + 0.5f;
            float light_depth = sample2d(u->shadow, su, sv).c[0] + 0.0001f;
            in_light = vd[8] < light_depth;
        }
        float light = u->ambient + (in_light ? diffuse + specular : 0.0f);
        for (int i = 0; i < 4; ++i) f[i] = surf[i] * light;
    }
    float pack(float c) const { return rmin(rmax(c, 0.0f), 1.0f) * 255.0f; }
};

struct ShadowShader {  // examples/teapot.rs:13-50
    static constexpr int NV = 1, NF = 1;
    const euc_shadow_uniforms *u;
    const euc_vertex_layout *lay;
    void vertex(const uint8_t *v, float clip[4], float *vd) const {
        float p[4] = {ldf(v, lay->position, 0), ldf(v, lay->position, 1), ldf(v, lay->position, 2), 1.0f};
        mat4_vec4(u->mvp, p, clip);
        vd[0] = 0.0f;
    }
    void fragment(const float *, float *f) const { f[0] = 0.0f; }
    float pack(float c) const { return c; }
};

// ---------------------------------------------------------------------------
// Targets (buffer.rs:147-219)
// ---------------------------------------------------------------------------
inline uint32_t fmt_bpp(uint32_t f) {
    switch (f) {
    case EUC_FMT_RGBA8: case EUC_FMT_BGRA8: case EUC_FMT_R32F: return 4;
    case EUC_FMT_RGB8: return 3;
    case EUC_FMT_RGBA32F: return 16;
    default: return 0;
    }
}

struct Target {
    uint8_t *data = nullptr;
    uint64_t w = 0, h = 0, pitch = 0;
    uint32_t fmt = EUC_FMT_NONE;
    explicit Target(const euc_target *t) {
        if (t && t->data) {
            data = (uint8_t *)t->data;
            w = t->width;
            h = t->height;
            fmt = t->format;
            pitch = t->pitch ? t->pitch : t->width * fmt_bpp(fmt);
        }
    }
    uint8_t *at(uint64_t x, uint64_t y) const { return data + y * pitch + x * fmt_bpp(fmt); }
    float read_depth(uint64_t x, uint64_t y) const {
        float f;
        std::memcpy(&f, at(x, y), 4);
        return f;
    }
    void write_depth(uint64_t x, uint64_t y, float z) const { std::memcpy(at(x, y), &z, 4); }
};

// Blend: REPLACE packs the fragment (every example blend); ALPHA is src-over.
template <class S>
void blend_pixel(const S &sh, uint32_t blend, uint8_t *px, uint32_t fmt, const float *f) {
    float c[4] = {f[0], S::NF > 1 ? f[1] : 0.0f, S::NF > 2 ? f[2] : 0.0f, S::NF > 3 ? f[3] : 0.0f};
    if (fmt == EUC_FMT_RGBA32F) {  // a float pixel keeps the fragment: no pack, src-over on the floats
        if (blend == EUC_BLEND_ALPHA) {
            float old[4];
            std::memcpy(old, px, sizeof(old));
            const float a = c[3];
            for (int i = 0; i < 4; ++i) c[i] = c[i] * a + old[i] * (1.0f - a);
        }
        std::memcpy(px, c, sizeof(c));
        return;
    }
    int ri = 0, gi = 1, bi = 2, ai = 3;
    if (fmt == EUC_FMT_BGRA8) { ri = 2; bi = 0; }
    if (blend == EUC_BLEND_ALPHA) {
        float old[4] = {0, 0, 0, 0};
        old[0] = (float)px[ri] / 255.0f;
        old[1] = (float)px[gi] / 255.0f;
        old[2] = (float)px[bi] / 255.0f;
        old[3] = fmt == EUC_FMT_RGB8 ? 1.0f : (float)px[ai] / 255.0f;
        float a = c[3];
        for (int i = 0; i < 4; ++i) c[i] = c[i] * a + old[i] * (1.0f - a);
    }
    px[ri] = as_u8(sh.pack(c[0]));
    px[gi] = as_u8(sh.pack(c[1]));
    px[bi] = as_u8(sh.pack(c[2]));
    if (fmt != EUC_FMT_RGB8) px[ai] = as_u8(sh.pack(c[3]));
}

struct Counters {
    std::atomic<uint64_t> triangles{0}, culled{0}, candidates{0}, passed{0};
};

// ---------------------------------------------------------------------------
// BlitterImpl (pipeline.rs:452-579) + Triangles::rasterize (triangles.rs:15-306)
// ---------------------------------------------------------------------------
template <class S>
struct Band {
    const S &sh;
    const euc_pipeline_desc &d;
    const Target &pixel;
    const Target &depth;
    uint64_t tgt_size[2];
    uint64_t tgt_min[2];
    uint64_t tgt_max[2];
    uint32_t msaa_level;
    // MSAA coarse-fragment cache (pipeline.rs:466, :600-610)
    uint64_t msaa_w = 0;
    std::vector<uint64_t> msaa_key;
    std::vector<float> msaa_frag;
    float msaa_div;
    uint64_t primitive_count = 0;
    uint64_t candidates = 0, passed = 0, triangles = 0, culled = 0;

    Band(const S &s, const euc_pipeline_desc &desc, const Target &px, const Target &dp, const uint64_t size[2],
         uint64_t row_start, uint64_t row_end, uint32_t level)
        : sh(s), d(desc), pixel(px), depth(dp), msaa_level(level) {
        tgt_size[0] = size[0]; tgt_size[1] = size[1];
        tgt_min[0] = 0; tgt_min[1] = row_start;
        tgt_max[0] = size[0]; tgt_max[1] = row_end;
        if (level > 0) {
            msaa_w = ((tgt_max[0] - tgt_min[0]) >> level) + 3;
            uint64_t mh = ((tgt_max[1] - tgt_min[1]) >> level) + 3;
            msaa_key.assign(msaa_w * mh, UINT64_MAX);
            msaa_frag.assign(msaa_w * mh * S::NF, 0.0f);
        }
        msaa_div = 1.0f / (float)(1u << level);
    }

    bool test_fragment(uint64_t x, uint64_t y, float z) const {  // pipeline.rs:519-526
        if (d.depth_test == EUC_TEST_NONE) return true;
        float old = depth.read_depth(x, y);
        switch (d.depth_test) {
        case EUC_TEST_LESS: return z < old;
        case EUC_TEST_EQUAL: return z == old;
        default: return z > old;
        }
    }

    // get_v_data (triangles.rs:274-294)
    struct VData {
        const float *o, *dx, *dy;
        const float *vo[3];
        void operator()(float xf, float yf, float *out) const {
            float w[3];
            for (int c = 0; c < 3; ++c) w[c] = (o[c] + dy[c] * yf) + dx[c] * xf;
            float wu[3] = {w[0], w[1], w[2] - w[0] - w[1]};
            float r = 1.0f / w[2];
            float wp[3] = {wu[0] * r, wu[1] * r, wu[2] * r};
            for (int i = 0; i < S::NV; ++i) out[i] = vo[0][i] * wp[0] + vo[1][i] * wp[1] + vo[2][i] * wp[2];
        }
    };

    template <class G>
    void msaa_fragment(uint64_t cx, uint64_t cy, const G &gv, float *out) {  // pipeline.rs:477-494
        uint64_t slot = (cx + 1) + msaa_w * (cy + 1);
        float *f = &msaa_frag[slot * S::NF];
        if (msaa_key[slot] != primitive_count) {
            msaa_key[slot] = primitive_count;
            float vd[S::NV];
            gv((float)(tgt_min[0] + (cx << msaa_level)), (float)(tgt_min[1] + (cy << msaa_level)), vd);
            sh.fragment(vd, f);
        }
        for (int i = 0; i < S::NF; ++i) out[i] = f[i];
    }

    template <class G>
    void emit_fragment(uint64_t x, uint64_t y, const G &gv, float z) {  // pipeline.rs:529-578
        if (d.depth_write) depth.write_depth(x, y, z);
        if (d.pixel_write) {
            float frag[S::NF];
            if (msaa_level == 0) {
                float vd[S::NV];
                gv((float)x, (float)y, vd);
                sh.fragment(vd, frag);
            } else {
                float fractx = fract((float)(x - tgt_min[0]) * msaa_div);
                float fracty = fract((float)(y - tgt_min[1]) * msaa_div);
                uint64_t posix = (x - tgt_min[0]) >> msaa_level;
                uint64_t posiy = (y - tgt_min[1]) >> msaa_level;
                float t00[S::NF], t10[S::NF], t01[S::NF], t11[S::NF];
                msaa_fragment(posix + 0, posiy + 0, gv, t00);
                msaa_fragment(posix + 1, posiy + 0, gv, t10);
                msaa_fragment(posix + 0, posiy + 1, gv, t01);
                msaa_fragment(posix + 1, posiy + 1, gv, t11);
                for (int i = 0; i < S::NF; ++i) {
                    float t0 = t00[i] * (1.0f - fracty) + t01[i] * fracty;
                    float t1 = t10[i] * (1.0f - fracty) + t11[i] * fracty;
                    frag[i] = t0 * (1.0f - fractx) + t1 * fractx;
                }
            }
            blend_pixel(sh, d.blend, pixel.at(x, y), pixel.fmt, frag);
        }
    }

    bool passes_z_clip(float z) const {  // pipeline.rs:151-156
        return !d.z_clip || (d.z_clip_min <= z && z <= d.z_clip_max);
    }

    // One primitive: triangles.rs:54-305.
    void primitive(const float *hom_in[3], const float *out_in[3]) {
        ++primitive_count;  // begin_primitive
        ++triangles;
        const float flip1 = d.y_axis == EUC_Y_UP ? -1.0f : 1.0f;
        float hom[3][4], euc[3][3];
        for (int i = 0; i < 3; ++i) {
            hom[i][0] = hom_in[i][0] * 1.0f;
            hom[i][1] = hom_in[i][1] * flip1;
            hom[i][2] = hom_in[i][2];
            hom[i][3] = hom_in[i][3];
            euc[i][0] = hom[i][0] / hom[i][3];
            euc[i][1] = hom[i][1] / hom[i][3];
            euc[i][2] = hom[i][2] / hom[i][3];
        }
        V3 e0 = {{euc[0][0], euc[0][1], euc[0][2]}};
        V3 e1 = {{euc[1][0], euc[1][1], euc[1][2]}};
        V3 e2 = {{euc[2][0], euc[2][1], euc[2][2]}};
        float winding = cross3(sub3(e1, e0), sub3(e2, e0)).v[2];
        const float *vo[3] = {out_in[0], out_in[1], out_in[2]};
        if (d.cull != EUC_CULL_NONE) {
            float cull_dir = d.cull == EUC_CULL_BACK ? 1.0f : -1.0f;
            if (winding * cull_dir < 0.0f) { ++culled; return; }
        }
        if (winding >= 0.0f) {  // reverse vertex order
            for (int k = 0; k < 4; ++k) std::swap(hom[0][k], hom[2][k]);
            for (int k = 0; k < 3; ++k) std::swap(euc[0][k], euc[2][k]);
            std::swap(vo[0], vo[2]);
        }
        const float size_x = (float)tgt_size[0], size_y = (float)tgt_size[1];
        M3 to_ndc = {{{2.0f / size_x, 0.0f, -1.0f}, {0.0f, -2.0f / size_y, 1.0f}, {0.0f, 0.0f, 1.0f}}};
        // coords_to_weights (triangles.rs:86-102)
        V3 a = {{hom[0][0], hom[0][1], hom[0][3]}};
        V3 b = {{hom[1][0], hom[1][1], hom[1][3]}};
        V3 c = {{hom[2][0], hom[2][1], hom[2][3]}};
        V3 ca = sub3(a, c), cb = sub3(b, c);
        V3 n = cross3(ca, cb);
        float rec_det = mag2(n) > 0.0f ? 1.0f / rmin(dot3(n, c), -__FLT_EPSILON__) : 1.0f;
        V3 r0 = scale3(cross3(cb, c), rec_det), r1 = scale3(cross3(c, ca), rec_det), r2 = scale3(n, rec_det);
        M3 rows = {{{r0.v[0], r0.v[1], r0.v[2]}, {r1.v[0], r1.v[1], r1.v[2]}, {r2.v[0], r2.v[1], r2.v[2]}}};
        M3 ctw = matmul3(rows, to_ndc);
        // screen coordinates (triangles.rs:110-111)
        float scr[3][2];
        for (int i = 0; i < 3; ++i) {
            scr[i][0] = size_x * (euc[i][0] * 0.5f + 0.5f);
            scr[i][1] = size_y * (euc[i][1] * -0.5f + 0.5f);
        }
        // bounding box clamped to this band (triangles.rs:114-139)
        uint64_t bmin[2], bmax[2];
        for (int k = 0; k < 2; ++k) {
            float mn = rmin(rmin(scr[0][k], scr[1][k]), scr[2][k]);
            float mx = rmax(rmax(scr[0][k], scr[1][k]), scr[2][k]);
            bmin[k] = clamp_u64(as_usize(mn + 0.0f), tgt_min[k], tgt_max[k]);
            bmax[k] = clamp_u64(as_usize(mx + 1.0f), tgt_min[k], tgt_max[k]);
        }
        // weights and their per-pixel deltas (triangles.rs:142-145)
        V3 o = mat3_vec3(ctw, V3{{0.0f, 0.0f, 1.0f}});
        V3 dxv = scale3(sub3(mat3_vec3(ctw, V3{{1000.0f, 0.0f, 1.0f}}), o), 1.0f / 1000.0f);
        V3 dyv = scale3(sub3(mat3_vec3(ctw, V3{{0.0f, 1000.0f, 1.0f}}), o), 1.0f / 1000.0f);
        // vertices ordered by height (triangles.rs:148-171)
        float min_y = rmin(rmin(scr[0][1], scr[1][1]), scr[2][1]);
        const float *by[3];
        if (scr[0][1] == min_y) {
            if (scr[1][1] < scr[2][1]) { by[0] = scr[0]; by[1] = scr[1]; by[2] = scr[2]; }
            else { by[0] = scr[0]; by[1] = scr[2]; by[2] = scr[1]; }
        } else if (scr[1][1] == min_y) {
            if (scr[0][1] < scr[2][1]) { by[0] = scr[1]; by[1] = scr[0]; by[2] = scr[2]; }
            else { by[0] = scr[1]; by[1] = scr[2]; by[2] = scr[0]; }
        } else {
            if (scr[0][1] < scr[1][1]) { by[0] = scr[2]; by[1] = scr[0]; by[2] = scr[1]; }
            else { by[0] = scr[2]; by[1] = scr[1]; by[2] = scr[0]; }
        }
        const bool no_clip = passes_z_clip(euc[0][2]) && passes_z_clip(euc[1][2]) && passes_z_clip(euc[2][2]);
        const float zc[3] = {hom[0][2], hom[1][2], hom[2][2]};

        VData gv{o.v, dxv.v, dyv.v, {vo[0], vo[1], vo[2]}};
        // rasterize::<NO_VERTS_CLIPPED> (triangles.rs:203-304)
        for (uint64_t y = bmin[1]; y < bmax[1]; ++y) {
            uint64_t ext = (bmax[0] - bmin[0]) * (bmax[1] - bmin[1]);
            uint64_t xs, xe;
            const float yf = (float)y;
            if (ext < 128) {
                xs = bmin[0];
                xe = bmax[0];
            } else {
                const float *A = by[0], *B = by[1], *C = by[2];
                float ac = lerp(A[0], C[0], (yf - A[1]) / (C[1] - A[1]));
                float lo, hi;
                if (yf < B[1]) {
                    float ab = lerp(A[0], B[0], (yf - A[1]) / (B[1] - A[1]));
                    lo = rmin(ab, ac); hi = rmax(ab, ac);
                } else {
                    float bc = lerp(B[0], C[0], (yf - B[1]) / (C[1] - B[1]));
                    lo = rmin(bc, ac); hi = rmax(bc, ac);
                }
                const float fx0 = (float)bmin[0], fx1 = (float)bmax[0];
                float fl = std::floor(lo), ce = std::ceil(hi);
                xs = (fl >= fx0 && fl < fx1) ? as_usize(fl) : bmin[0];
                xe = (ce >= fx0 && ce < fx1) ? as_usize(ce) : bmax[0];
            }
            float w[3];
            const float xsf = (float)xs;
            for (int k = 0; k < 3; ++k) w[k] = (o.v[k] + dyv.v[k] * yf) + dxv.v[k] * xsf;
            for (uint64_t x = xs; x < xe; ++x) {
                float wu[3] = {w[0], w[1], w[2] - w[0] - w[1]};
                if (wu[0] >= 0.0f && wu[1] >= 0.0f && wu[2] >= 0.0f) {
                    float z = zc[0] * wu[0] + zc[1] * wu[1] + zc[2] * wu[2];
                    if (no_clip || passes_z_clip(z)) {
                        ++candidates;
                        if (test_fragment(x, y, z)) {
                            ++passed;
                            emit_fragment(x, y, gv, z);
                        }
                    }
                }
                w[0] = w[0] + dxv.v[0];
                w[1] = w[1] + dxv.v[1];
                w[2] = w[2] + dxv.v[2];
            }
        }
    }

    // weighted_sum2 of a line's two vertex outputs (lines.rs:98-110)
    struct LineVData {
        bool use_x;
        float sx0, sy0, norm;
        const float *vo[2];
        void operator()(float xf, float yf, float *out) const {
            const float frac = (use_x ? xf - sx0 : yf - sy0) * norm;
            for (int i = 0; i < S::NV; ++i) out[i] = vo[0][i] * (1.0f - frac) + vo[1][i] * frac;
        }
    };

    // One line: Lines::rasterize (lines.rs:30-119) on this band.
    void line(const float *hom_in[2], const float *out_in[2]) {
        ++primitive_count;  // begin_primitive
        ++triangles;        // primitives assembled
        const float flip1 = d.y_axis == EUC_Y_UP ? -1.0f : 1.0f;
        float euc[2][3], scr[2][2];
        const float size_x = (float)tgt_size[0], size_y = (float)tgt_size[1];
        for (int i = 0; i < 2; ++i) {
            const float a0 = hom_in[i][0] * 1.0f, a1 = hom_in[i][1] * flip1, a2 = hom_in[i][2];
            const float w = rmax(hom_in[i][3], 0.0001f);
            euc[i][0] = a0 / w;
            euc[i][1] = a1 / w;
            euc[i][2] = a2 / w;
            scr[i][0] = size_x * (euc[i][0] * 0.5f + 0.5f);
            scr[i][1] = size_y * (euc[i][1] * -0.5f + 0.5f);
        }
        const float smin[2] = {(float)tgt_min[0], (float)tgt_min[1]};
        const float smax[2] = {(float)tgt_max[0], (float)tgt_max[1]};
        const int64_t x1 = as_isize(scr[0][0]), y1 = as_isize(scr[0][1]);
        const int64_t x2 = as_isize(scr[1][0]), y2 = as_isize(scr[1][1]);
        const int64_t wx1 = as_isize(fclamp(rmin(scr[0][0], scr[1][0]) + 0.0f, smin[0], smax[0]));
        const int64_t wy1 = as_isize(fclamp(rmin(scr[0][1], scr[1][1]) + 0.0f, smin[1], smax[1]));
        const int64_t wx2 = as_isize(fclamp(rmax(scr[0][0], scr[1][0]) + 1.0f, smin[0], smax[0]));
        const int64_t wy2 = as_isize(fclamp(rmax(scr[0][1], scr[1][1]) + 1.0f, smin[1], smax[1]));
        const bool use_x = wabs(wsub(x1, x2)) > wabs(wsub(y1, y2));
        const float norm = 1.0f / (use_x ? scr[1][0] - scr[0][0] : scr[1][1] - scr[0][1]);
        const LineVData gv{use_x, scr[0][0], scr[0][1], norm, {out_in[0], out_in[1]}};
        bresenham_clipped(x1, y1, x2, y2, wx1, wy1, wx2 - 1, wy2 - 1, [&](int64_t xi, int64_t yi) {
            const uint64_t x = (uint64_t)xi, y = (uint64_t)yi;
            const float frac = (use_x ? (float)x - scr[0][0] : (float)y - scr[0][1]) * norm;
            const float z = euc[0][2] + frac * (euc[1][2] - euc[0][2]);
            if (!passes_z_clip(z)) return;
            ++candidates;
            if (test_fragment(x, y, z)) {
                ++passed;
                emit_fragment(x, y, gv, z);
            }
        });
    }
};

inline uint64_t read_index(const uint32_t *idx, uint64_t i) { return idx ? idx[i] : i; }

// Built-in geometry stages (Pipeline::geometry, pipeline.rs:221-229, emitted
// in order by pipeline.rs:277-289); the output triangles of each input
// triangle, as documented with enum euc_geometry.  `c`: 3 clip positions,
// `v`: 3 vertex outputs of nv floats.  Returns how many triangles it wrote
// to oc / ov (up to 4).
inline uint32_t geometry_ratio(uint32_t g) {
    return g == EUC_GEOM_SUBDIVIDE ? 4u : g == EUC_GEOM_DUPLICATE ? 2u : 1u;
}

int geometry_stage(uint32_t g, float param, int nv, const float *c[3], const float *v[3], float *oc, float *ov) {
    auto put = [&](int k, int j, const float *cc, const float *vv) {
        for (int i = 0; i < 4; ++i) oc[(k * 3 + j) * 4 + i] = cc[i];
        for (int i = 0; i < nv; ++i) ov[(k * 3 + j) * nv + i] = vv[i];
    };
    if (g == EUC_GEOM_SUBDIVIDE) {
        std::vector<float> mc(3 * 4), mv(3 * (size_t)nv);
        const int e[3][2] = {{0, 1}, {1, 2}, {2, 0}};  // ab, bc, ca
        for (int m = 0; m < 3; ++m) {
            for (int i = 0; i < 4; ++i) mc[m * 4 + i] = c[e[m][0]][i] * 0.5f + c[e[m][1]][i] * 0.5f;
            for (int i = 0; i < nv; ++i) mv[m * nv + i] = v[e[m][0]][i] * 0.5f + v[e[m][1]][i] * 0.5f;
        }
        const float *ab = &mc[0], *bc = &mc[4], *ca = &mc[8];
        const float *vab = &mv[0], *vbc = &mv[nv], *vca = &mv[2 * nv];
        put(0, 0, c[0], v[0]); put(0, 1, ab, vab); put(0, 2, ca, vca);
        put(1, 0, ab, vab); put(1, 1, c[1], v[1]); put(1, 2, bc, vbc);
        put(2, 0, ca, vca); put(2, 1, bc, vbc); put(2, 2, c[2], v[2]);
        put(3, 0, ab, vab); put(3, 1, bc, vbc); put(3, 2, ca, vca);
        return 4;
    }
    if (g == EUC_GEOM_SHRINK) {
        float m[4], s[4];
        for (int i = 0; i < 4; ++i) m[i] = ((c[0][i] + c[1][i]) + c[2][i]) / 3.0f;
        for (int j = 0; j < 3; ++j) {
            for (int i = 0; i < 4; ++i) s[i] = m[i] + (c[j][i] - m[i]) * param;
            put(0, j, s, v[j]);
        }
        return 1;
    }
    if (g == EUC_GEOM_DISCARD) {
        bool beyond = true;
        for (int j = 0; j < 3; ++j) beyond = beyond && (c[j][2] / c[j][3] > param);
        if (beyond) return 0;
    }
    for (int j = 0; j < 3; ++j) put(0, j, c[j], v[j]);
    if (g == EUC_GEOM_DUPLICATE) {
        float s[4];
        for (int j = 0; j < 3; ++j) {
            for (int i = 0; i < 4; ++i) s[i] = c[j][i];
            s[0] = c[j][0] + param * c[j][3];
            put(1, j, s, v[j]);
        }
        return 2;
    }
    return 1;
}

template <class S>
int render_impl(const S &sh, const euc_pipeline_desc &d, const void *verts, uint64_t nverts,
                const euc_vertex_layout &lay, const uint32_t *idx, uint64_t nidx, const Target &pixel,
                const Target &depth, int threads, Counters &cnt) {
    const bool uses_depth = d.depth_test != EUC_TEST_NONE || d.depth_write;
    uint64_t size[2];
    if (!d.pixel_write && !uses_depth) return EUC_OK;  // pipeline.rs:257
    if (d.pixel_write && !uses_depth) { size[0] = pixel.w; size[1] = pixel.h; }
    else if (!d.pixel_write) { size[0] = depth.w; size[1] = depth.h; }
    else {
        if (pixel.w != depth.w || pixel.h != depth.h) return EUC_ERR_SIZE_MISMATCH;
        size[0] = pixel.w; size[1] = pixel.h;
    }
    // Vertex stage: once per stream element, in order (pipeline.rs:273-276, :322).
    const uint64_t n = idx ? nidx : nverts;
    for (uint64_t i = 0; i < n; ++i)
        if (read_index(idx, i) >= nverts) return EUC_ERR_INDEX_OOB;  // index.rs:53 panics before drawing
    // complete primitives of the stream; a trailing partial one is dropped
    // (collect_primitive returns None, pipeline.rs:283)
    const uint32_t per = d.primitives == EUC_PRIM_LINE_LIST ? 2 : 3;
    const uint64_t ngroup = n / per;
    const uint64_t nshade = ngroup * per;
    std::vector<float> clip(nshade * 4), vout(nshade * (uint64_t)S::NV);
    const uint8_t *vb = (const uint8_t *)verts;
    for (uint64_t i = 0; i < nshade; ++i)
        sh.vertex(vb + read_index(idx, i) * lay.stride, &clip[i * 4], &vout[i * S::NV]);
    uint64_t nprim = ngroup;  // triangles (or line groups) handed to the rasteriser
    if (d.geometry != EUC_GEOM_NONE) {  // triangles only (checked by the caller)
        const uint32_t R = geometry_ratio(d.geometry);
        std::vector<float> gclip(ngroup * R * 3 * 4), gvout(ngroup * R * 3 * (uint64_t)S::NV);
        uint64_t out = 0;
        for (uint64_t t = 0; t < ngroup; ++t) {
            const float *c[3] = {&clip[(t * 3 + 0) * 4], &clip[(t * 3 + 1) * 4], &clip[(t * 3 + 2) * 4]};
            const float *v[3] = {&vout[(t * 3 + 0) * S::NV], &vout[(t * 3 + 1) * S::NV], &vout[(t * 3 + 2) * S::NV]};
            out += geometry_stage(d.geometry, d.geometry_param, S::NV, c, v, &gclip[out * 3 * 4],
                                  &gvout[out * 3 * S::NV]);
        }
        gclip.resize(out * 3 * 4);
        gvout.resize(out * 3 * S::NV);
        clip.swap(gclip);
        vout.swap(gvout);
        nprim = out;
    }

    const uint32_t level = d.aa_level > 6 ? 6 : d.aa_level;  // pipeline.rs:291-294
    // Row bands (pipeline.rs:328-345).
    uint64_t gr;
    if (d.band_rows == EUC_BANDS_PAR) {
        gr = 20000ull * (1ull << level) / (size[0] > 1 ? size[0] : 1);
        if (gr == 0) return EUC_ERR_BAND;
        if (size[1] / gr == 0) {
            if (d.flags & EUC_FLAG_PAR_EMPTY) return EUC_OK;  // needed_threads == 0
            gr = size[1] > 0 ? size[1] : 1;
        }
    } else {
        gr = d.band_rows;
        if (gr > size[1]) gr = size[1] > 0 ? size[1] : 1;
    }
    const uint64_t nbands = (size[1] + gr - 1) / gr;
    std::atomic<uint64_t> next{0};
    auto worker = [&]() {
        for (;;) {
            uint64_t b = next.fetch_add(1);
            if (b >= nbands) break;
            uint64_t r0 = b * gr, r1 = r0 + gr < size[1] ? r0 + gr : size[1];
            Band<S> band(sh, d, pixel, depth, size, r0, r1, level);
            if (d.primitives == EUC_PRIM_TRIANGLE_LIST) {
                for (uint64_t t = 0; t < nprim; ++t) {
                    const float *h[3] = {&clip[(t * 3 + 0) * 4], &clip[(t * 3 + 1) * 4], &clip[(t * 3 + 2) * 4]};
                    const float *o[3] = {&vout[(t * 3 + 0) * S::NV], &vout[(t * 3 + 1) * S::NV],
                                         &vout[(t * 3 + 2) * S::NV]};
                    band.primitive(h, o);
                }
            } else {
                // LineList: (0 1) (2 3) ...; LineTriangleList: (a b) (b c) (c a)
                // per triangle (primitives.rs:46-104)
                const uint64_t nlines = d.primitives == EUC_PRIM_LINE_LIST ? ngroup : 3 * ngroup;
                for (uint64_t l = 0; l < nlines; ++l) {
                    uint64_t e0, e1;
                    if (d.primitives == EUC_PRIM_LINE_LIST) {
                        e0 = 2 * l;
                        e1 = 2 * l + 1;
                    } else {
                        const uint64_t t = l / 3, k = l % 3;
                        e0 = 3 * t + k;
                        e1 = 3 * t + (k + 1) % 3;
                    }
                    const float *h[2] = {&clip[e0 * 4], &clip[e1 * 4]};
                    const float *o[2] = {&vout[e0 * S::NV], &vout[e1 * S::NV]};
                    band.line(h, o);
                }
            }
            cnt.candidates += band.candidates;
            cnt.passed += band.passed;
            if (b == 0) { cnt.triangles += band.triangles; cnt.culled += band.culled; }
        }
    };
    const int nt = threads < 1 ? 1 : threads;
    if (nt == 1 || nbands == 1) {
        worker();
    } else {
        std::vector<std::thread> pool;
        int k = (uint64_t)nt < nbands ? nt : (int)nbands;
        for (int i = 0; i < k; ++i) pool.emplace_back(worker);
        for (auto &t : pool) t.join();
    }
    return EUC_OK;
}

}  // namespace

extern "C" {

typedef struct oracle_stats {
    uint64_t triangles, culled, candidates, passed;
} oracle_stats;

// Renders on host buffers; `threads` row-band workers (1 = serial).  Output
// does not depend on `threads`, as in euc's render_par.
int oracle_render(const euc_pipeline_desc *d, const void *uniforms, size_t usize, const euc_vertex_layout *lay,
                  const void *verts, size_t nverts, const uint32_t *idx, size_t nidx, const euc_target *pixel,
                  const euc_target *depth, int threads, oracle_stats *st) {
    if (!d || !lay || !uniforms) return EUC_ERR_INVALID;
    // the C ABI's enum ranges (euc's Rust enums cannot hold other values)
    if (d->depth_test > EUC_TEST_GREATER || d->cull > EUC_CULL_FRONT || d->y_axis > EUC_Y_UP ||
        d->blend > EUC_BLEND_ALPHA)
        return EUC_ERR_INVALID;
    if (d->primitives > EUC_PRIM_LINE_LIST || d->geometry > EUC_GEOM_DISCARD) return EUC_ERR_INVALID;
    if (d->geometry != EUC_GEOM_NONE && d->primitives != EUC_PRIM_TRIANGLE_LIST) return EUC_ERR_INVALID;
    if (nverts && !verts) return EUC_ERR_INVALID;
    Target px(pixel), dp(depth);
    if (d->pixel_write && px.data && fmt_bpp(px.fmt) == 0) return EUC_ERR_INVALID;
    if (d->pixel_write && px.data && px.fmt == EUC_FMT_R32F) return EUC_ERR_INVALID;
    if (dp.data && dp.fmt != EUC_FMT_R32F) return EUC_ERR_INVALID;
    Counters cnt;
    int rc = EUC_ERR_INVALID;
    switch (d->shader) {
#define EUC_CASE(KIND, SH, UT)                                                                          \
    case KIND: {                                                                                        \
        if (usize < sizeof(UT)) return EUC_ERR_INVALID;                                                 \
        SH sh{(const UT *)uniforms, lay};                                                               \
        rc = render_impl(sh, *d, verts, nverts, *lay, idx, nidx, px, dp, threads, cnt);                 \
        break;                                                                                          \
    }
        EUC_CASE(EUC_SHADER_FLAT, FlatShader, euc_flat_uniforms)
        EUC_CASE(EUC_SHADER_VCOLOR, VColorShader, euc_vcolor_uniforms)
        EUC_CASE(EUC_SHADER_GOURAUD, GouraudShader, euc_gouraud_uniforms)
        EUC_CASE(EUC_SHADER_TEXTURED, TexturedShader, euc_textured_uniforms)
        EUC_CASE(EUC_SHADER_PHONG, PhongShader, euc_phong_uniforms)
        EUC_CASE(EUC_SHADER_SHADOW, ShadowShader, euc_shadow_uniforms)
#undef EUC_CASE
    default: return EUC_ERR_INVALID;
    }
    if (st) {
        st->triangles = cnt.triangles;
        st->culled = cnt.culled;
        st->candidates = cnt.candidates;
        st->passed = cnt.passed;
    }
    return rc;
}

// N-D nearest sampling (sampler/nearest.rs:27-33, math.rs:40-60,
// buffer.rs:85-100) after the wrap of sampler/mod.rs:100-179.
int oracle_sample_nearest(const void *texels, uint32_t ndim, const uint32_t *size, uint32_t tb, uint32_t wrap,
                          const float *queries, uint64_t count, void *out) {
    if (!size || ndim < 1 || ndim > 4 || tb < 1 || tb > 16 || wrap > EUC_WRAP_MIRROR) return EUC_ERR_INVALID;
    for (uint32_t a = 0; a < ndim; ++a)
        if (size[a] < 1) return EUC_ERR_INVALID;
    for (uint64_t i = 0; i < count; ++i) {
        uint64_t lin = 0, factor = 1;
        for (uint32_t a = 0; a < ndim; ++a) {
            const float e = wrap_coord(wrap, queries[i * ndim + a]);
            uint64_t idx = as_usize(rmax(e * (float)size[a], 0.0f));  // Denormalize::denormalize_to
            if (idx > size[a] - 1u) idx = size[a] - 1u;
            lin += idx * factor;  // Buffer::linear_index
            factor *= size[a];
        }
        std::memcpy((uint8_t *)out + i * tb, (const uint8_t *)texels + lin * tb, tb);
    }
    return EUC_OK;
}

// Texture ingest: image's to_rgba8 expansion of the 8-bit layouts into RGBA8
// texels, f32 copied as is (texture.rs:321-344 read through Buffer::from_texture).
int oracle_texture_ingest(const void *src, uint32_t w, uint32_t h, uint64_t spitch, uint32_t fmt, void *dst,
                          uint64_t dpitch) {
    static const uint32_t bpp[6] = {4, 4, 3, 1, 2, 4};
    if (fmt > EUC_SRC_R32F) return EUC_ERR_INVALID;
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) {
            const uint8_t *p = (const uint8_t *)src + y * spitch + (uint64_t)x * bpp[fmt];
            uint8_t *q = (uint8_t *)dst + y * dpitch + 4ull * x;
            uint8_t px[4];
            switch (fmt) {
            case EUC_SRC_RGBA8: px[0] = p[0]; px[1] = p[1]; px[2] = p[2]; px[3] = p[3]; break;
            case EUC_SRC_BGRA8: px[0] = p[2]; px[1] = p[1]; px[2] = p[0]; px[3] = p[3]; break;
            case EUC_SRC_RGB8: px[0] = p[0]; px[1] = p[1]; px[2] = p[2]; px[3] = 255; break;
            case EUC_SRC_LUMA8: px[0] = px[1] = px[2] = p[0]; px[3] = 255; break;
            case EUC_SRC_LUMA_ALPHA8: px[0] = px[1] = px[2] = p[0]; px[3] = p[1]; break;
            default: std::memcpy(px, p, 4); break;
            }
            std::memcpy(q, px, 4);
        }
    return EUC_OK;
}

// Scalar helpers exposed for known-answer tests of Rust semantics.
uint64_t oracle_as_usize(float v) { return as_usize(v); }
uint8_t oracle_as_u8(float v) { return as_u8(v); }
float oracle_rem_euclid(float x, float m) { return rem_euclid(x, m); }
float oracle_fract(float x) { return fract(x); }
void oracle_sample(const euc_sampler *s, float u, float v, float out[4]) {
    Texel t = sample2d(*s, u, v);
    for (int i = 0; i < 4; ++i) out[i] = t.c[i];
}
int oracle_hw_threads(void) {
    unsigned n = std::thread::hardware_concurrency();
    return n ? (int)n : 1;
}

}  // extern "C"
