/*
 * euc_gb300.h — C ABI of the GB300 (sm_103a) triangle pipeline that stands in
 * for euc's `Pipeline::render` (euc 0.6.0, src/pipeline.rs:248-300).
 *
 * Every entry point is plain C: pointers, sizes and the POD structs below.
 * A Rust façade implements `euc::Pipeline::render` by forwarding to
 * `euc_render_host` (host buffers, blocking like the Rust call) or
 * `euc_render` (device buffers, ordered on a CUDA stream).
 *
 * Semantics follow euc exactly: the same per-triangle setup, the same
 * incremental f32 weight walk per row, the same row bands of `render_par`,
 * the same depth-test/blend order, the same coarse-grid "MSAA".  Coverage,
 * depth bits and fragment counts are bit-identical to euc's CPU render.
 */
#ifndef EUC_GB300_H
#define EUC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EUC_ABI_VERSION 1

/* ------------------------------------------------------------------------ */
/* Status codes.  euc reports failures by panicking; each panic site maps to
 * one code, and nothing is drawn when a render fails.                       */
/* ------------------------------------------------------------------------ */
enum euc_status {
    EUC_OK = 0,
    EUC_ERR_INVALID = 1,       /* null pointer, unknown enum, unsupported format       */
    EUC_ERR_SIZE_MISMATCH = 2, /* pixel/depth sizes differ: assert at pipeline.rs:262-266 */
    EUC_ERR_INDEX_OOB = 3,     /* index >= vertex count: slice panic at index.rs:53      */
    EUC_ERR_OOM = 4,           /* device allocation failed                               */
    EUC_ERR_CUDA = 5,          /* a CUDA call failed                                     */
    EUC_ERR_BAND = 6,          /* band height 0 (width > 20000<<level): division by zero
                                  at pipeline.rs:330                                    */
    EUC_ERR_TIMEOUT = 7,       /* a bounded device wait ran out                          */
    EUC_ERR_BUDGET = 8,        /* serving: request larger than the framebuffer budget    */
    EUC_ERR_CAPACITY = 9       /* a fixed-capacity variant was given more than it holds  */
};

/* DepthMode.test (pipeline.rs:14-19): Option<Ordering>, compared with
 * `z.partial_cmp(&old_z) == Some(test)` (pipeline.rs:519-526).             */
enum euc_depth_test {
    EUC_TEST_NONE = 0,
    EUC_TEST_LESS = 1,
    EUC_TEST_EQUAL = 2,
    EUC_TEST_GREATER = 3
};

/* CullMode (rasterizer/mod.rs:9-18); euc's default is Back.                 */
enum euc_cull { EUC_CULL_NONE = 0, EUC_CULL_BACK = 1, EUC_CULL_FRONT = 2 };

/* CoordinateMode (pipeline.rs:94-163).                                       */
enum euc_y_axis { EUC_Y_DOWN = 0, EUC_Y_UP = 1 };
enum euc_handedness { EUC_LEFT = 0, EUC_RIGHT = 1 };

/* Texel / pixel formats.  EUC_FMT_NONE with a NULL pointer and a 0x0 size is
 * euc's `Empty` target (texture.rs:285-319).                                */
enum euc_format {
    EUC_FMT_NONE = 0,
    EUC_FMT_RGBA8 = 1, /* bytes r,g,b,a                                       */
    EUC_FMT_BGRA8 = 2, /* bytes b,g,r,a (u32::from_le_bytes of Rgba(b,g,r,a)) */
    EUC_FMT_RGB8 = 3,  /* bytes r,g,b                                         */
    EUC_FMT_R32F = 4   /* f32                                                  */
};

/* Shader kinds: device functors that mirror the Pipeline impls of euc's
 * examples (vertex -> fragment -> blend).                                   */
enum euc_shader {
    EUC_SHADER_FLAT = 0,     /* uniform colour                                        */
    EUC_SHADER_VCOLOR = 1,   /* per-vertex RGBA8 colour (examples/triangle.rs:14-25)  */
    EUC_SHADER_GOURAUD = 2,  /* per-vertex Lambert colour (spinning_cube.rs shape)    */
    EUC_SHADER_TEXTURED = 3, /* sampled texture (examples/texture_mapping.rs:20-34)   */
    EUC_SHADER_PHONG = 4,    /* Phong + shadow map + texture (examples/teapot.rs:69-141) */
    EUC_SHADER_SHADOW = 5,   /* depth-only pass (examples/teapot.rs:13-50)            */
    EUC_SHADER_COUNT = 6
};

/* Blend: REPLACE packs the fragment and ignores the old pixel (every blend in
 * euc's examples); ALPHA is src-over on the unpacked old pixel.            */
enum euc_blend { EUC_BLEND_REPLACE = 0, EUC_BLEND_ALPHA = 1 };

/* Sampler (sampler/mod.rs, linear.rs, nearest.rs).                          */
enum euc_filter { EUC_FILTER_NEAREST = 0, EUC_FILTER_LINEAR = 1 };
enum euc_wrap {
    EUC_WRAP_NONE = 0,   /* raw Linear/Nearest                       */
    EUC_WRAP_CLAMP = 1,  /* Clamped: max(0).min(1)      mod.rs:100-118 */
    EUC_WRAP_TILE = 2,   /* Tiled: rem_euclid(1)        mod.rs:124-142 */
    EUC_WRAP_MIRROR = 3  /* Mirrored                     mod.rs:149-179 */
};

/* band_rows: the row bands that euc's render_par hands to threads
 * (pipeline.rs:328-345).  The band origin feeds the bbox clamp, the
 * `extent < 128` span switch and the MSAA grid, so it changes the output.   */
#define EUC_BANDS_PAR 0u          /* 20000 * 2^level / width rows (euc default)       */
#define EUC_BANDS_SEQ 0xFFFFFFFFu /* one band = render_seq (euc without `par`)        */
/* With EUC_BANDS_PAR euc draws nothing when height < band rows
 * (pipeline.rs:330).  By default such targets use one band (render_seq);
 * this flag reproduces the blank output instead.                             */
#define EUC_FLAG_PAR_EMPTY 1u
/* Resolve every candidate fragment in submission order from per-pixel lists
 * (the path that EUC_BLEND_ALPHA always takes); with a replace blend the
 * result is the same as the default visibility-key path.  Costs one stream
 * synchronisation per render (to size the lists).                          */
#define EUC_FLAG_ORDERED 2u

/* Mirrors the mode methods of `Pipeline` (pipeline.rs:178-209).            */
typedef struct euc_pipeline_desc {
    uint32_t shader;      /* enum euc_shader                                  */
    uint32_t pixel_write; /* PixelMode.write                                  */
    uint32_t depth_test;  /* enum euc_depth_test                              */
    uint32_t depth_write; /* DepthMode.write                                  */
    uint32_t handedness;  /* CoordinateMode.handedness (unused by triangles)  */
    uint32_t y_axis;      /* CoordinateMode.y_axis_direction                  */
    uint32_t z_clip;      /* 1: z_clip_range = Some(z_clip_min..z_clip_max)   */
    float z_clip_min;
    float z_clip_max;
    uint32_t aa_level;    /* AaMode: 0 = None, n = Msaa{level:n} (clamped to 6) */
    uint32_t cull;        /* enum euc_cull                                    */
    uint32_t blend;       /* enum euc_blend                                   */
    uint32_t band_rows;   /* EUC_BANDS_PAR, EUC_BANDS_SEQ or an explicit height */
    uint32_t flags;       /* EUC_FLAG_*                                       */
} euc_pipeline_desc;

/* A 2-D target (Buffer2d, buffer.rs:183-219): row-major, y*pitch + x*bpp. */
typedef struct euc_target {
    void *data;      /* NULL for Empty                                         */
    uint32_t width;
    uint32_t height;
    uint32_t pitch;  /* bytes per row; 0 = width * bytes per pixel             */
    uint32_t format; /* enum euc_format                                        */
} euc_target;

/* A texture plus its sampler chain, e.g. `tex.map(u8 -> f32).linear().tiled()`.
 * RGBA8 texels are mapped channel-wise to `(u8 as f32) / texel_div`
 * (texture.rs:84-94 `map`).  R32F texels are read as they are.             */
typedef struct euc_sampler {
    const void *data; /* NULL = no texture (shader-specific fallback)         */
    uint32_t width;
    uint32_t height;
    uint32_t pitch;   /* bytes per row; 0 = packed                            */
    uint32_t format;  /* EUC_FMT_RGBA8 or EUC_FMT_R32F                        */
    uint32_t filter;  /* enum euc_filter                                      */
    uint32_t wrap;    /* enum euc_wrap                                        */
    float texel_div;  /* RGBA8 only: 1.0 or 255.0                             */
    uint32_t reserved;
} euc_sampler;

/* Where a shader's attributes sit in one vertex (byte offsets; -1 = absent). */
typedef struct euc_vertex_layout {
    uint32_t stride;  /* bytes between vertices                               */
    int32_t position; /* f32 x3 (x4 for VCOLOR: a clip-space position)        */
    int32_t normal;   /* f32 x3                                               */
    int32_t uv;       /* f32 x2                                               */
    int32_t color;    /* RGBA8                                                */
} euc_vertex_layout;

/* Uniforms, one struct per shader kind.  Matrices are row-major:
 * out[r] = ((m[r][0]*v0 + m[r][1]*v1) + m[r][2]*v2) + m[r][3]*v3.          */
typedef struct euc_flat_uniforms {
    float mvp[16];
    float color[4]; /* fragment colour, packed as sat_u8(c * 255)            */
} euc_flat_uniforms;

typedef struct euc_vcolor_uniforms {
    float mvp[16];  /* applied to the f32x4 position                         */
} euc_vcolor_uniforms;

typedef struct euc_gouraud_uniforms {
    float mvp[16];
    float model[16];   /* normal transform: model * (n, 0)                    */
    float to_light[3]; /* unit vector towards the directional light           */
    float ambient;
    float color[3];
    float diffuse;
} euc_gouraud_uniforms;

typedef struct euc_textured_uniforms {
    float mvp[16];
    euc_sampler tex;   /* fragment = sample(uv); blend = sat_u8(c) per channel */
} euc_textured_uniforms;

typedef struct euc_phong_uniforms {
    float model[16];
    float view[16];
    float proj[16];
    float light_vp[16];
    float light_pos[3];
    float normal_sign; /* -1 reproduces teapot.rs's `-normal`                 */
    float cam_pos[3];
    float ambient;     /* teapot.rs: 0.1                                      */
    float surf_color[4];
    euc_sampler tex;    /* data NULL: surface = surf_color                     */
    euc_sampler shadow; /* R32F depth map; data NULL: always lit               */
} euc_phong_uniforms;

typedef struct euc_shadow_uniforms {
    float mvp[16];
} euc_shadow_uniforms;

/* Per-render statistics (device-side exact counters).                       */
typedef struct euc_stats {
    uint64_t triangles;  /* primitives assembled                              */
    uint64_t culled;     /* primitives culled by winding                      */
    uint64_t candidates; /* (pixel, primitive) pairs that pass the inside test
                            and the z-clip test, summed over bands           */
} euc_stats;

/* One scene of a batch (device pointers).                                    */
typedef struct euc_scene {
    euc_pipeline_desc desc;
    euc_vertex_layout layout;
    const void *vertices;
    uint64_t nverts;
    const uint32_t *indices; /* NULL: vertices are drawn in order             */
    uint64_t nindices;
    euc_target pixel;
    euc_target depth;
    const void *uniforms; /* host pointer to the shader's uniform struct      */
    uint64_t uniforms_size;
} euc_scene;

typedef struct euc_ctx euc_ctx;

/* ---- context --------------------------------------------------------- */

/* Creates a context on `device`.  Replaces nothing in euc (euc has no
 * device state); owns scratch buffers, streams and launch tuning.          */
int euc_ctx_create(int device, euc_ctx **out);
int euc_ctx_destroy(euc_ctx *ctx);
/* Pre-sizes the scratch buffers so that later renders allocate nothing.    */
int euc_ctx_reserve(euc_ctx *ctx, uint64_t max_verts, uint64_t max_tris, uint64_t max_pixels,
                    uint64_t max_scenes);
/* Waits for `stream` and returns the first device-side error of renders
 * issued on it (EUC_ERR_INDEX_OOB), then clears it.                         */
int euc_ctx_sync(euc_ctx *ctx, void *stream);
/* Statistics of the most recent render / batch (synchronises the stream).   */
int euc_ctx_stats(euc_ctx *ctx, void *stream, euc_stats *out);
const char *euc_status_string(int status);
int euc_abi_version(void);

/* Pipeline stages, for per-stage timing.                                    */
enum euc_stage {
    EUC_STAGE_VERTEX = 0,  /* vertex functor                                   */
    EUC_STAGE_SETUP = 1,   /* primitive setup                                  */
    EUC_STAGE_SCAN = 2,    /* row-count scan + compaction                      */
    EUC_STAGE_INIT = 3,    /* visibility keys of the stored depth              */
    EUC_STAGE_RASTER = 4,  /* row walk + depth test                            */
    EUC_STAGE_RESOLVE = 5, /* shading of the winners + colour / depth writes   */
    EUC_STAGE_COUNT = 6
};

/* Profiling aid (no counterpart in euc): while enabled, each render records
 * CUDA events around its stages on its own stream.  euc_ctx_profile waits for
 * them, returns the summed milliseconds per stage and the number of kernel
 * launches issued since the last call, and resets both.                     */
int euc_ctx_set_profiling(euc_ctx *ctx, int enable);
int euc_ctx_profile(euc_ctx *ctx, double ms[EUC_STAGE_COUNT], uint64_t *launches);

/* ---- rendering --------------------------------------------------------- */

/* `Pipeline::render(vertices, pixel, depth)` (pipeline.rs:248-300) on device
 * buffers, ordered on `stream` (a cudaStream_t, NULL = legacy default).
 * `indices` NULL draws `vertices` in order (a plain vertex slice);
 * otherwise it is `IndexedVertices::new(indices, vertices)` (index.rs:4-55).
 * Returns host-detectable errors at once; device-side errors are reported by
 * euc_ctx_sync.                                                              */
int euc_render(euc_ctx *ctx, const euc_pipeline_desc *desc, const void *uniforms,
               size_t uniforms_size, const euc_vertex_layout *layout, const void *vertices,
               size_t nverts, const uint32_t *indices, size_t nindices, const euc_target *pixel,
               const euc_target *depth, void *stream);

/* The same render on HOST buffers, blocking, like the Rust call: copies the
 * vertices, indices, textures and targets to the device, renders, copies the
 * targets back and returns the final status.  Texture pointers inside the
 * uniforms are host pointers here.                                          */
int euc_render_host(euc_ctx *ctx, const euc_pipeline_desc *desc, const void *uniforms,
                    size_t uniforms_size, const euc_vertex_layout *layout, const void *vertices,
                    size_t nverts, const uint32_t *indices, size_t nindices,
                    const euc_target *pixel, const euc_target *depth);

/* Batched form: renders `n` independent scenes with one set of launches
 * (grouped by shader kind).  Each output is byte-identical to the scene
 * rendered alone with euc_render.  No counterpart in euc.                   */
int euc_render_batch(euc_ctx *ctx, const euc_scene *scenes, size_t n, void *stream);

/* euc_render without a context and without any allocation.  No counterpart in
 * euc: it exists for callers that may not allocate device memory, such as an
 * engine or plugin host that owns a fixed device-memory budget, or a render
 * thread that cannot pay for cudaMalloc/cudaFree (both synchronise the whole
 * device).  Scratch lives in one fixed array inside the library (about 20.8
 * MiB per device that loads it, held until exit).  Limits: 65,536 vertices,
 * 65,536 primitives (index triples), 1,048,576 target pixels; larger scenes
 * return EUC_ERR_CAPACITY, and so do order-dependent blends (EUC_BLEND_ALPHA,
 * EUC_FLAG_ORDERED), whose fragment lists are sized on the device.  Runs on
 * the current device, ordered on `stream`.
 * `device_status` (nullable, device memory) receives EUC_OK or
 * EUC_ERR_INDEX_OOB once the render has run.  All calls share the scratch
 * array: calls whose work overlaps on the GPU race, so issue them on one
 * stream.  The first call on a device looks up the array's device address;
 * make it before any stream capture starts.                                 */
int euc_render_noalloc(const euc_pipeline_desc *desc, const void *uniforms, size_t uniforms_size,
                       const euc_vertex_layout *layout, const void *vertices, size_t nverts,
                       const uint32_t *indices, size_t nindices, const euc_target *pixel,
                       const euc_target *depth, void *stream, int *device_status);

#ifdef __cplusplus
}
#endif

#endif /* EUC_GB300_H */
