// euc_device.cuh — device-side arithmetic of the euc triangle pipeline.
//
// Everything here reproduces euc 0.6.0's f32 operation order.  The file is
// compiled with -fmad=false -prec-div=true -prec-sqrt=true -ftz=false, so no
// multiply-add is contracted (Rust never contracts), division and sqrt are
// IEEE round-to-nearest and denormals are kept, as on the CPU.
#pragma once

#include <cstdint>

#include "../../include/euc_gb300.h"

#define EUC_DEV __device__ __forceinline__

namespace eucg {

// ---------------------------------------------------------------------------
// Rust scalar semantics
// ---------------------------------------------------------------------------
// f32::min / f32::max ignore a NaN operand, like fminf / fmaxf.
EUC_DEV float rmin(float a, float b) { return fminf(a, b); }
EUC_DEV float rmax(float a, float b) { return fmaxf(a, b); }

// `v as usize` (saturating, NaN -> 0), further capped at 2^32 - 1.  Every use
// clamps the result to a target extent below 2^32, so the cap changes nothing.
EUC_DEV uint32_t sat_u32(float v) {
    if (!(v >= 1.0f)) return 0u;
    if (v >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)v;
}

// `v as u8` (saturating, NaN -> 0).
EUC_DEV uint32_t sat_u8(float v) {
    if (!(v >= 1.0f)) return 0u;
    if (v >= 255.0f) return 255u;
    return (uint32_t)v;
}

EUC_DEV float rfract(float v) { return v - truncf(v); }  // f32::fract

// fmodf(x, m) for m = 1 or 2 (the wraps' moduli): x - m * trunc(x / m) is
// exact there (the quotient by a power of two, its truncation and the product
// are exact, and the difference, a multiple of x's ulp below 2 in magnitude,
// is representable), and fmodf's result has the sign of x.
__host__ __device__ inline float fmod_1_or_2(float x, float m) {
    return copysignf(x - m * truncf(x * (m == 1.0f ? 1.0f : 0.5f)), x);
}

EUC_DEV float rem_euclid(float x, float m) {  // f32::rem_euclid, m = 1 or 2
    float r = fmod_1_or_2(x, m);
    return r < 0.0f ? r + fabsf(m) : r;
}

EUC_DEV float ld_f32(const uint8_t *p) { return *reinterpret_cast<const float *>(p); }

// ---------------------------------------------------------------------------
// Example-shader maths (op order documented in include/euc_gb300.h)
// ---------------------------------------------------------------------------
EUC_DEV void mat4_vec4(const float *m, const float v[4], float out[4]) {
#pragma unroll
    for (int r = 0; r < 4; ++r)
        out[r] = ((m[r * 4 + 0] * v[0] + m[r * 4 + 1] * v[1]) + m[r * 4 + 2] * v[2]) + m[r * 4 + 3] * v[3];
}
EUC_DEV float dot3(const float *a, const float *b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
EUC_DEV void normalize3(const float *a, float *out) {
    float len = sqrtf(dot3(a, a));
    out[0] = a[0] / len;
    out[1] = a[1] / len;
    out[2] = a[2] / len;
}

// normalize3 with the hardware reciprocal square root: for lighting terms
// only, whose result is a colour quantised to 8 bits.  Its relative error
// (about 2^-22) moves a colour channel by far less than one step, so the
// quantised colour stays within the +-1 per channel that colour parity
// allows; coordinates that pick texels or shadow-map depths stay exact.
EUC_DEV void normalize3_light(const float *a, float *out) {
    const float r = rsqrtf(dot3(a, a));
    out[0] = a[0] * r;
    out[1] = a[1] * r;
    out[2] = a[2] * r;
}

// ---------------------------------------------------------------------------
// Samplers: sampler/mod.rs:100-179 (wraps), linear.rs:30-66, nearest.rs:27-33
// ---------------------------------------------------------------------------
struct Texel {
    float c[4];
};

// (float)b / 255.0f for every byte b, evaluated by the compiler (correctly
// rounded, as the division on the device is): an RGBA8 texel's channels are
// looked up here instead of divided, four divisions per texel saved.
struct ByteOver255 {
    float v[256];
    constexpr ByteOver255() : v() {
        for (int i = 0; i < 256; ++i) v[i] = (float)i / 255.0f;
    }
};
__device__ const ByteOver255 g_byte_over_255 = ByteOver255();

EUC_DEV Texel read_texel(const euc_sampler &s, uint32_t x, uint32_t y) {
    const uint32_t pitch = s.pitch ? s.pitch : s.width * 4u;
    const uint8_t *p = reinterpret_cast<const uint8_t *>(s.data) + (uint64_t)y * pitch + (uint64_t)x * 4u;
    Texel t;
    if (s.format == EUC_FMT_R32F) {
        float f = __ldg(reinterpret_cast<const float *>(p));
        t.c[0] = t.c[1] = t.c[2] = t.c[3] = f;
    } else {
        // (u8 as f32) / texel_div (texture.rs:84-94); texel_div is 1 or 255
        uint32_t w = __ldg(reinterpret_cast<const unsigned int *>(p));
        if (s.texel_div == 255.0f) {
#pragma unroll
            for (int i = 0; i < 4; ++i) t.c[i] = __ldg(g_byte_over_255.v + ((w >> (8 * i)) & 0xFFu));
        } else if (s.texel_div == 1.0f) {
#pragma unroll
            for (int i = 0; i < 4; ++i) t.c[i] = (float)((w >> (8 * i)) & 0xFFu);
        } else {
#pragma unroll
            for (int i = 0; i < 4; ++i) t.c[i] = (float)((w >> (8 * i)) & 0xFFu) / s.texel_div;
        }
    }
    return t;
}

EUC_DEV float wrap_coord(uint32_t wrap, float e) {
    switch (wrap) {
    case EUC_WRAP_CLAMP: return rmin(rmax(e, 0.0f), 1.0f);
    case EUC_WRAP_TILE: return rem_euclid(e, 1.0f);
    case EUC_WRAP_MIRROR: return rem_euclid(e, 2.0f) >= 1.0f ? 1.0f - rem_euclid(e, 1.0f) : rem_euclid(e, 1.0f);
    default: return e;
    }
}

EUC_DEV Texel sample2d(const euc_sampler &s, float u, float v) {
    u = wrap_coord(s.wrap, u);
    v = wrap_coord(s.wrap, v);
    const uint32_t w = s.width, h = s.height;
    if (s.filter == EUC_FILTER_NEAREST) {
        uint32_t ix = sat_u32(rmax(u * (float)w, 0.0f));
        uint32_t iy = sat_u32(rmax(v * (float)h, 0.0f));
        ix = ix < w - 1u ? ix : w - 1u;
        iy = iy < h - 1u ? iy : h - 1u;
        return read_texel(s, ix, iy);
    }
    const float itx = rfract(u) * (float)w;
    const float ity = rfract(v) * (float)h;
    const uint32_t px = sat_u32(truncf(itx));
    const uint32_t py = sat_u32(truncf(ity));
    const float fx = rfract(itx);
    const float fy = rfract(ity);
    const uint32_t p0x = px < w - 1u ? px : w - 1u;
    const uint32_t p0y = py < h - 1u ? py : h - 1u;
    const uint32_t p1x = px + 1u < w - 1u ? px + 1u : w - 1u;
    const uint32_t p1y = py + 1u < h - 1u ? py + 1u : h - 1u;
    const Texel t00 = read_texel(s, p0x, p0y);
    const Texel t10 = read_texel(s, p1x, p0y);
    const Texel t01 = read_texel(s, p0x, p1y);
    const Texel t11 = read_texel(s, p1x, p1y);
    Texel out;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float t0 = t00.c[i] * (1.0f - fy) + t01.c[i] * fy;
        const float t1 = t10.c[i] * (1.0f - fy) + t11.c[i] * fy;
        out.c[i] = t0 * (1.0f - fx) + t1 * fx;
    }
    return out;
}

// ---------------------------------------------------------------------------
// Shader functors.  NV = VertexData floats, NF = Fragment floats.
// vertex(): one vertex -> clip position + VertexData
// fragment(): interpolated VertexData -> Fragment (RGBA f32)
// pack(): per-channel scale applied before the saturating `as u8`
// ---------------------------------------------------------------------------
struct FlatFn {
    static constexpr int NV = 1, NF = 4;
    static constexpr bool kDirect = true;  // shaded in place, without the job list of k_resolve
    static constexpr int kResolveBlocks = 4;  // k_resolve blocks per SM
    using U = euc_flat_uniforms;
    static EUC_DEV void vertex(const U &u, const euc_vertex_layout &l, const uint8_t *v, float clip[4], float *vd) {
        const float p[4] = {ld_f32(v + l.position), ld_f32(v + l.position + 4), ld_f32(v + l.position + 8), 1.0f};
        mat4_vec4(u.mvp, p, clip);
        vd[0] = 0.0f;
    }
    static EUC_DEV void fragment(const U &u, const float *, float *f) {
#pragma unroll
        for (int i = 0; i < 4; ++i) f[i] = u.color[i];
    }
    static EUC_DEV float pack(float c) { return c * 255.0f; }
};

struct VColorFn {  // examples/triangle.rs:14-25
    static constexpr int NV = 4, NF = 4;
    static constexpr bool kDirect = true;  // shaded in place, without the job list of k_resolve
    static constexpr int kResolveBlocks = 4;  // k_resolve blocks per SM
    using U = euc_vcolor_uniforms;
    static EUC_DEV void vertex(const U &u, const euc_vertex_layout &l, const uint8_t *v, float clip[4], float *vd) {
        const float p[4] = {ld_f32(v + l.position), ld_f32(v + l.position + 4), ld_f32(v + l.position + 8),
                            ld_f32(v + l.position + 12)};
        mat4_vec4(u.mvp, p, clip);
        const uint32_t c = *reinterpret_cast<const uint32_t *>(v + l.color);
#pragma unroll
        for (int i = 0; i < 4; ++i) vd[i] = (float)((c >> (8 * i)) & 0xFFu) / 255.0f;
    }
    static EUC_DEV void fragment(const U &, const float *vd, float *f) {
#pragma unroll
        for (int i = 0; i < 4; ++i) f[i] = vd[i];
    }
    static EUC_DEV float pack(float c) { return c * 255.0f; }
};

struct GouraudFn {
    static constexpr int NV = 3, NF = 4;
    static constexpr bool kDirect = true;  // shaded in place, without the job list of k_resolve
    static constexpr int kResolveBlocks = 5;  // k_resolve blocks per SM: 5 (no spills) was 4 % faster than 4 on the sphere
    using U = euc_gouraud_uniforms;
    static EUC_DEV void vertex(const U &u, const euc_vertex_layout &l, const uint8_t *v, float clip[4], float *vd) {
        const float p[4] = {ld_f32(v + l.position), ld_f32(v + l.position + 4), ld_f32(v + l.position + 8), 1.0f};
        mat4_vec4(u.mvp, p, clip);
        const float n4[4] = {ld_f32(v + l.normal), ld_f32(v + l.normal + 4), ld_f32(v + l.normal + 8), 0.0f};
        float wn[4], n[3];
        mat4_vec4(u.model, n4, wn);
        normalize3(wn, n);
        const float lambert = rmax(dot3(n, u.to_light), 0.0f);
        const float k = u.ambient + lambert * u.diffuse;
#pragma unroll
        for (int i = 0; i < 3; ++i) vd[i] = u.color[i] * k;
    }
    static EUC_DEV void fragment(const U &, const float *vd, float *f) {
        f[0] = vd[0];
        f[1] = vd[1];
        f[2] = vd[2];
        f[3] = 1.0f;
    }
    static EUC_DEV float pack(float c) { return c * 255.0f; }
};

struct TexturedFn {  // examples/texture_mapping.rs:20-34
    static constexpr int NV = 2, NF = 4;
    static constexpr bool kDirect = true;  // shaded in place, without the job list of k_resolve
    static constexpr int kResolveBlocks = 4;  // k_resolve blocks per SM
    using U = euc_textured_uniforms;
    static EUC_DEV void vertex(const U &u, const euc_vertex_layout &l, const uint8_t *v, float clip[4], float *vd) {
        const float p[4] = {ld_f32(v + l.position), ld_f32(v + l.position + 4), ld_f32(v + l.position + 8), 1.0f};
        mat4_vec4(u.mvp, p, clip);
        vd[0] = ld_f32(v + l.uv);
        vd[1] = ld_f32(v + l.uv + 4);
    }
    static EUC_DEV void fragment(const U &u, const float *vd, float *f) {
        const Texel t = sample2d(u.tex, vd[0], vd[1]);
#pragma unroll
        for (int i = 0; i < 4; ++i) f[i] = t.c[i];
    }
    static EUC_DEV float pack(float c) { return c; }
};

struct PhongFn {  // examples/teapot.rs:69-141 with a surface texture
    static constexpr int NV = 11, NF = 4;
    static constexpr bool kDirect = false;  // costly: shaded through the job list of k_resolve
    static constexpr int kResolveBlocks = 4;  // k_resolve blocks per SM: at 5 its registers spill (12 % slower)
    using U = euc_phong_uniforms;
    static EUC_DEV void vertex(const U &u, const euc_vertex_layout &l, const uint8_t *v, float clip[4], float *vd) {
        const float p[4] = {ld_f32(v + l.position), ld_f32(v + l.position + 4), ld_f32(v + l.position + 8), 1.0f};
        float wpos[4];
        mat4_vec4(u.model, p, wpos);
        const float n4[4] = {ld_f32(v + l.normal) * u.normal_sign, ld_f32(v + l.normal + 4) * u.normal_sign,
                             ld_f32(v + l.normal + 8) * u.normal_sign, 0.0f};
        float wnorm[4];
        mat4_vec4(u.model, n4, wnorm);
        const float wp1[4] = {wpos[0], wpos[1], wpos[2], 1.0f};
        float lvp[4], vpos[4];
        mat4_vec4(u.light_vp, wp1, lvp);
        mat4_vec4(u.view, wpos, vpos);
        mat4_vec4(u.proj, vpos, clip);
        vd[0] = wpos[0];
        vd[1] = wpos[1];
        vd[2] = wpos[2];
        vd[3] = wnorm[0];
        vd[4] = wnorm[1];
        vd[5] = wnorm[2];
        vd[6] = lvp[0] / lvp[3];
        vd[7] = lvp[1] / lvp[3];
        vd[8] = lvp[2] / lvp[3];
        if (l.uv >= 0) {
            vd[9] = ld_f32(v + l.uv);
            vd[10] = ld_f32(v + l.uv + 4);
        } else {
            vd[9] = 0.0f;
            vd[10] = 0.0f;
        }
    }
    static EUC_DEV void fragment(const U &u, const float *vd, float *f) {
        float n[3], cam_dir[3], light_dir[3], t[3];
        // lighting terms: hardware reciprocal square root and power (see normalize3_light)
        normalize3_light(vd + 3, n);
#pragma unroll
        for (int i = 0; i < 3; ++i) t[i] = u.cam_pos[i] - vd[i];
        normalize3_light(t, cam_dir);
#pragma unroll
        for (int i = 0; i < 3; ++i) t[i] = vd[i] - u.light_pos[i];
        normalize3_light(t, light_dir);
        float surf[4];
        if (u.tex.data) {
            const Texel tx = sample2d(u.tex, vd[9], vd[10]);
#pragma unroll
            for (int i = 0; i < 4; ++i) surf[i] = tx.c[i];
        } else {
#pragma unroll
            for (int i = 0; i < 4; ++i) surf[i] = u.surf_color[i];
        }
        const float nl[3] = {-light_dir[0], -light_dir[1], -light_dir[2]};
        const float diffuse = rmax(dot3(n, nl), 0.0f) * 0.5f;
        const float d = dot3(nl, n);
        const float dd = d + d;
        const float r[3] = {nl[0] - n[0] * dd, nl[1] - n[1] * dd, nl[2] - n[2] * dd};
        const float nc[3] = {-cam_dir[0], -cam_dir[1], -cam_dir[2]};
        const float specular = __powf(rmax(dot3(r, nc), 0.0f), 30.0f) * 3.0f;
        bool in_light = true;
        if (u.shadow.data) {
            const float su = (vd[6] * 1.0f) * 0.5f + 0.5f;
            const float sv = (vd[7] * -1.0f) * 0.5f + 0.5f;
            const float light_depth = sample2d(u.shadow, su, sv).c[0] + 0.0001f;
            in_light = vd[8] < light_depth;
        }
        const float light = u.ambient + (in_light ? diffuse + specular : 0.0f);
#pragma unroll
        for (int i = 0; i < 4; ++i) f[i] = surf[i] * light;
    }
    static EUC_DEV float pack(float c) { return rmin(rmax(c, 0.0f), 1.0f) * 255.0f; }
};

struct ShadowFn {  // examples/teapot.rs:13-50
    static constexpr int NV = 1, NF = 1;
    static constexpr bool kDirect = true;  // shaded in place, without the job list of k_resolve
    static constexpr int kResolveBlocks = 4;  // k_resolve blocks per SM
    using U = euc_shadow_uniforms;
    static EUC_DEV void vertex(const U &u, const euc_vertex_layout &l, const uint8_t *v, float clip[4], float *vd) {
        const float p[4] = {ld_f32(v + l.position), ld_f32(v + l.position + 4), ld_f32(v + l.position + 8), 1.0f};
        mat4_vec4(u.mvp, p, clip);
        vd[0] = 0.0f;
    }
    static EUC_DEV void fragment(const U &, const float *, float *f) { f[0] = 0.0f; }
    static EUC_DEV float pack(float c) { return c; }
};

}  // namespace eucg
