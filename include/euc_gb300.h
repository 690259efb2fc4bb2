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

#define EUC_ABI_VERSION 2

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
    EUC_ERR_CAPACITY = 9,      /* a fixed-capacity variant was given more than it holds  */
    EUC_ERR_STALE = 10,        /* a recorded graph whose context scratch has since moved */
    EUC_ERR_BUSY = 11          /* serving: the admission queue is full                   */
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
    EUC_FMT_R32F = 4,  /* f32                                                  */
    /* f32 r,g,b,a: a colour target that keeps the fragment as it is, as a
     * Buffer2d<[f32; 4]> (or Rgba<f32>) pixel type does: REPLACE stores the
     * fragment's four values (no pack, no saturation), ALPHA is src-over on
     * the stored floats.  Colour targets only (not a texture format).       */
    EUC_FMT_RGBA32F = 5
};

/* Source layouts for texture ingest: the image crate's 8-bit pixel types
 * and f32.                                                                  */
enum euc_src_format {
    EUC_SRC_RGBA8 = 0,       /* r,g,b,a                                        */
    EUC_SRC_BGRA8 = 1,       /* b,g,r,a                                        */
    EUC_SRC_RGB8 = 2,        /* r,g,b                                          */
    EUC_SRC_LUMA8 = 3,       /* l                                              */
    EUC_SRC_LUMA_ALPHA8 = 4, /* l,a                                            */
    EUC_SRC_R32F = 5         /* f32                                            */
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

/* `Pipeline::Primitives` (primitives.rs): how the vertex stream is grouped
 * and which rasteriser draws it.                                           */
enum euc_primitives {
    EUC_PRIM_TRIANGLE_LIST = 0,      /* TriangleList: 0 1 2 | 3 4 5 (primitives.rs:18-44)   */
    EUC_PRIM_LINE_TRIANGLE_LIST = 1, /* LineTriangleList: lines 0-1, 1-2, 2-0 (:46-77)      */
    EUC_PRIM_LINE_LIST = 2           /* LineList: lines 0-1, 2-3 (:79-104)                  */
};

/* Built-in geometry stages: `Pipeline::geometry` (pipeline.rs:221-229)
 * turns each assembled triangle into 0..4 triangles, emitted in order
 * (pipeline.rs:277-289).  New vertices are made the way a Rust geometry
 * stage would with VertexData's Add/Mul: componentwise on the clip position
 * and the vertex outputs.  TriangleList only.                              */
enum euc_geometry {
    EUC_GEOM_NONE = 0,      /* emit the triangle as it is (the default)                 */
    EUC_GEOM_SUBDIVIDE = 1, /* 4 triangles on the edge midpoints p*0.5 + q*0.5:
                               (a, ab, ca), (ab, b, bc), (ca, bc, c), (ab, bc, ca)        */
    EUC_GEOM_SHRINK = 2,    /* each clip position pulled to the centroid
                               m = ((a + b) + c) / 3: m + (v - m) * param                */
    EUC_GEOM_DUPLICATE = 3, /* the triangle, then a copy with x += param * w           */
    EUC_GEOM_DISCARD = 4    /* nothing when z / w > param at all three vertices         */
};

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
    uint32_t primitives;  /* enum euc_primitives (Pipeline::Primitives)       */
    uint32_t geometry;    /* enum euc_geometry (Pipeline::geometry)           */
    float geometry_param; /* parameter of the geometry stage                  */
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

/* Launch shape of the pipeline (no counterpart in euc).  None of these
 * changes a result, only how work is spread over the GPU; 0 keeps the
 * default.  Set by an autotuner that times a batch under several shapes.   */
typedef struct euc_tuning {
    uint32_t raster_blocks_per_sm; /* persistent k_raster blocks per SM (default: occupancy limit) */
    uint32_t raster_warp_rows;     /* (primitive, row) items a warp claims at once, 32..256, x32 (256) */
    uint32_t chunk_group;          /* 256-pixel chunks per scene lookup in init/resolve (adaptive)   */
    uint32_t chunk_blocks_per_sm;  /* init/resolve grid cap per SM (16)                              */
    uint32_t raster_probe;         /* 1: read a key before its atomicMin, 2: atomics only (default)  */
    uint32_t host_copy;            /* host-buffer renders: EUC_HOST_COPY_* (AUTO)                    */
    uint32_t strip_path;           /* shared-memory strips: 0 for overdrawn scenes, 1 off, 2 always  */
} euc_tuning;

/* How euc_render_host / euc_render_host_batch reach host buffers.  DIRECT
 * has the kernels use the vertices, indices and targets in host memory and
 * gathers only the textures; it needs a device that accesses pageable host
 * memory coherently (cudaDevAttrPageableMemoryAccess, e.g. over
 * NVLink-C2C), and euc_ctx_set_tuning refuses it elsewhere.  STAGED copies
 * everything through page-locked memory with host threads.  AUTO takes
 * DIRECT where it can.                                                      */
enum euc_host_copy { EUC_HOST_COPY_AUTO = 0, EUC_HOST_COPY_STAGED = 1, EUC_HOST_COPY_DIRECT = 2 };
int euc_ctx_set_tuning(euc_ctx *ctx, const euc_tuning *tuning);
int euc_ctx_get_tuning(euc_ctx *ctx, euc_tuning *tuning);

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

/* The same render on HOST buffers, blocking, like the Rust call; it returns
 * the final status.  Texture pointers inside the uniforms are host pointers
 * here.  The buffers reach the device as euc_tuning.host_copy says: in
 * place where the device reads pageable host memory (textures gathered),
 * else copied through page-locked memory and the targets copied back.      */
int euc_render_host(euc_ctx *ctx, const euc_pipeline_desc *desc, const void *uniforms,
                    size_t uniforms_size, const euc_vertex_layout *layout, const void *vertices,
                    size_t nverts, const uint32_t *indices, size_t nindices,
                    const euc_target *pixel, const euc_target *depth);

/* Batched form on host buffers (blocking): every scene's vertex, index,
 * texture (in its uniforms) and target pointers are host memory, as for
 * euc_render_host, and the batch renders as euc_render_batch.  Under
 * EUC_HOST_COPY_DIRECT the kernels read the vertices and indices and update
 * the targets where they lie in host memory; only the textures are gathered
 * into device memory, by one kernel.  Under EUC_HOST_COPY_STAGED `threads`
 * host threads (0: the hardware concurrency, at most 16) stage every input
 * and target into page-locked memory, one copy moves each direction, and
 * the targets are copied back.  A scene that fails draws nothing and the
 * others are drawn; the first failure's status is returned.  Textures that
 * several scenes share (the same host pointer) are copied once.  No
 * counterpart in euc.                                                       */
int euc_render_host_batch(euc_ctx *ctx, const euc_scene *scenes, size_t n, int threads);

/* Batched form: renders `n` independent scenes with one set of launches
 * (grouped by shader kind).  Each output is byte-identical to the scene
 * rendered alone with euc_render.  No counterpart in euc.                   */
int euc_render_batch(euc_ctx *ctx, const euc_scene *scenes, size_t n, void *stream);

/* A batch recorded once as a CUDA graph and replayed with one launch.  The
 * graph holds the scene table, the uniforms and every device pointer of
 * `scenes` as they were at creation: between launches the caller may change
 * the contents of vertex, index, texture and target buffers, not the
 * pointers or sizes.  It renders with `ctx`'s scratch buffers, so its
 * launches must be ordered with every other render on that context.  A later
 * render on the context that needs more scratch than the context held at
 * creation moves that scratch; the graph then refuses to launch
 * (EUC_ERR_STALE) and must be recreated (euc_ctx_reserve before creation
 * avoids that).  Destroy graphs before their context.  Scenes on the ordered
 * path (EUC_BLEND_ALPHA, EUC_FLAG_ORDERED) cannot be recorded
 * (EUC_ERR_INVALID).  No counterpart in euc.                                */
typedef struct euc_graph euc_graph;
int euc_graph_create(euc_ctx *ctx, const euc_scene *scenes, size_t n, euc_graph **out);
int euc_graph_launch(euc_graph *graph, void *stream);
int euc_graph_destroy(euc_graph *graph);

/* Texture ingest: `Buffer::from_texture` of an `image::ImageBuffer`
 * (buffer.rs:32-58, texture.rs:321-344), done on the device.  Converts
 * width x height texels of `src_format` (rows `src_pitch` bytes apart, in
 * host or device memory) into `dst` (device memory, rows `dst_pitch` bytes
 * apart) in a sampler layout: RGBA8 for the 8-bit sources, as image's
 * to_rgba8 expands them (grey -> l,l,l,255; grey+alpha -> l,l,l,a;
 * RGB -> alpha 255; BGRA reordered), and R32F for R32F.  A host source is
 * staged through the context and the call waits for `stream`; a device
 * source is converted in order on `stream`.  No counterpart in euc beyond
 * the two calls it stands for.                                              */
int euc_texture_ingest(euc_ctx *ctx, const void *src, uint32_t width, uint32_t height, uint64_t src_pitch,
                       uint32_t src_format, void *dst, uint64_t dst_pitch, void *stream);

/* Nearest sampling of an N-dimensional texture (N = 1..4): what
 * `Nearest::sample` (sampler/nearest.rs:27-33) returns after the wrap of
 * sampler/mod.rs:100-179 (`wrap`: euc_wrap), `Denormalize` per axis
 * (math.rs:40-60) and the linear index of `Buffer<T, N>` (buffer.rs:85-100,
 * axis 0 fastest).  `texels`: packed texels of `texel_bytes` (1..16) each,
 * `size[ndim]` of them per axis; `queries`: `count` points of `ndim` f32;
 * the texel of each point is copied to `out` (count * texel_bytes bytes).
 * All three are device memory; ordered on `stream` of the current device.  */
int euc_sample_nearest(const void *texels, uint32_t ndim, const uint32_t *size, uint32_t texel_bytes, uint32_t wrap,
                       const float *queries, uint64_t count, void *out, void *stream);

/* euc_render without a context and without any allocation.  No counterpart in
 * euc: it exists for callers that may not allocate device memory, such as an
 * engine or plugin host that owns a fixed device-memory budget, or a render
 * thread that cannot pay for cudaMalloc/cudaFree (both synchronise the whole
 * device).  Scratch lives in one fixed array inside the library (about 21.0
 * MiB per device that loads it, held until exit).  Limits: 65,536 vertices,
 * 65,536 primitive slots (one per triangle, one per line, three per triangle
 * of a LineTriangleList), 1,048,576 target pixels; larger scenes return
 * EUC_ERR_CAPACITY, and so do order-dependent blends (EUC_BLEND_ALPHA,
 * EUC_FLAG_ORDERED), whose fragment lists are sized on the device, and
 * geometry stages, whose output vertices need room beyond the fixed array.  Runs on
 * the current device, ordered on `stream`.
 * `device_status` (nullable, device memory) receives EUC_OK or
 * EUC_ERR_INDEX_OOB once the render has run.  All calls share the scratch
 * array: calls whose work overlaps on the GPU race, so issue them on one
 * stream.  The first call on a device (and the first after cudaDeviceReset)
 * looks up the array's device address; make it before any stream capture
 * starts.  The scene table and uniforms travel as a kernel parameter: no
 * host memory is read after the call returns.                               */
int euc_render_noalloc(const euc_pipeline_desc *desc, const void *uniforms, size_t uniforms_size,
                       const euc_vertex_layout *layout, const void *vertices, size_t nverts,
                       const uint32_t *indices, size_t nindices, const euc_target *pixel,
                       const euc_target *depth, void *stream, int *device_status);

/* ---- serving (no counterpart in euc) ------------------------------------
 *
 * A request loop on one device.  Meshes and textures are uploaded once and
 * stay resident; each request names them by id, brings its uniforms and
 * lists its targets (framebuffers), which the server carves out of a fixed
 * device-memory budget when it admits the request.  A serving thread admits
 * requests in submission order as soon as their arrival time has passed and
 * the budget has room, gathers whatever is admissible into a batch when one
 * of its `slots` (a stream with its own euc_ctx) is free, and runs the batch
 * as euc_render_batch calls (pass k of every request in the k-th call; the
 * passes of one request stay in order), so batches of several slots overlap
 * on the device while new requests keep arriving.  Each request's targets are
 * cleared to their clear value first; after the last pass, targets marked
 * `readback` are copied to the request's `out` buffer and the request
 * completes.  Every image is byte-identical to the same passes rendered with
 * euc_render on targets cleared the same way.                               */
typedef struct euc_server euc_server;

typedef struct euc_server_config {
    int32_t device;
    uint32_t max_batch;          /* requests per batch (0: 256)                         */
    uint64_t framebuffer_budget; /* device bytes for the targets of admitted requests   */
    uint32_t slots;              /* batches in flight, one stream + context each (0: 3) */
    uint32_t max_pending;        /* submitted, not yet admitted requests (0: 1 << 20)   */
} euc_server_config;

typedef struct euc_server_target {
    uint32_t width, height;
    uint32_t format;   /* euc_format, not EUC_FMT_RGBA32F (rejected: EUC_ERR_INVALID)    */
    uint32_t clear;    /* colour: little-endian packed texel; R32F: the f32 bit pattern */
    uint32_t readback; /* non-zero: copied to the request's `out` on completion         */
    uint32_t reserved;
} euc_server_target;

/* Points the euc_sampler at byte `offset` of a pass's uniforms at a resident
 * texture (`texture` >= 0) or at one of the request's own targets written by
 * an earlier pass (`target` >= 0).  The sampler keeps its filter, wrap and
 * texel_div; its data, width, height, pitch and format are set here.        */
typedef struct euc_server_binding {
    uint32_t offset;
    int32_t texture;
    int32_t target;
    uint32_t reserved;
} euc_server_binding;

typedef struct euc_server_pass {
    euc_pipeline_desc desc;
    uint32_t mesh;         /* resident mesh id                                      */
    int32_t pixel_target;  /* index into the request's targets, -1: Empty           */
    int32_t depth_target;  /* index into the request's targets, -1: Empty           */
    uint32_t nbindings;
    const euc_server_binding *bindings;
    const void *uniforms;  /* the shader's uniform struct (copied at submission)    */
    uint64_t uniforms_size;
} euc_server_pass;

#define EUC_SERVER_MAX_TARGETS 4
#define EUC_SERVER_MAX_PASSES 4

typedef struct euc_server_request {
    uint64_t tag;        /* returned with the completion                              */
    uint64_t arrival_ns; /* euc_server_now_ns() time from which it may be admitted; 0: now */
    void *out;           /* host memory for the readback targets, in target order,
                            rows of width * bytes-per-texel; page-locked memory keeps
                            the copy asynchronous                                     */
    uint64_t out_size;
    uint32_t ntargets, npasses;
    const euc_server_target *targets;
    const euc_server_pass *passes;
} euc_server_request;

typedef struct euc_server_completion {
    uint64_t id, tag;
    int32_t status;
    uint32_t batch_size;  /* requests in the batch it ran in                            */
    uint64_t arrival_ns;  /* the request's arrival (its submission time if it gave 0)   */
    uint64_t admit_ns;    /* admitted into a batch                                      */
    uint64_t done_ns;     /* its batch finished on the device, readback included        */
} euc_server_completion;

typedef struct euc_server_stats {
    uint64_t submitted, completed, failed, refused;
    uint64_t pending, in_flight;
    uint64_t batches, batched_requests;
    uint64_t budget_bytes, budget_used, budget_peak;
    uint64_t launches;  /* kernels launched so far (target clears + renders)      */
} euc_server_stats;

int euc_server_create(const euc_server_config *config, euc_server **out);
/* Waits for the batches in flight, drops requests not yet admitted.         */
int euc_server_destroy(euc_server *srv);
/* Uploads a mesh (host vertices of nverts * layout->stride bytes, u32 indices
 * or NULL) and returns its id; indices are checked against nverts here.     */
int euc_server_add_mesh(euc_server *srv, const euc_vertex_layout *layout, const void *vertices, size_t nverts,
                        const uint32_t *indices, size_t nindices, uint32_t *id);
/* Uploads a texture (RGBA8 or R32F, the sampler formats; rows `pitch` bytes
 * apart on the host, packed on the device) and returns its id.             */
int euc_server_add_texture(euc_server *srv, const void *texels, uint32_t width, uint32_t height, uint64_t pitch,
                           uint32_t format, uint32_t *id);
/* Nanoseconds of a steady clock since the server was created.               */
uint64_t euc_server_now_ns(euc_server *srv);
/* Queues `n` requests with consecutive ids from *first_id.  Every request is
 * checked first (ids, target indices, sizes, uniforms, `out` size); if one
 * fails, none is queued (EUC_ERR_INVALID, or EUC_ERR_BUDGET for a request
 * whose targets alone exceed the budget).  When the admission queue holds
 * max_pending requests the rest are refused: *accepted says how many were
 * queued and the call returns EUC_ERR_BUSY.                                 */
int euc_server_submit(euc_server *srv, const euc_server_request *reqs, size_t n, uint64_t *first_id,
                      size_t *accepted);
/* Moves up to `max` completions into `out`, waiting up to `wait_ms` for the
 * first one (0: no wait).                                                   */
int euc_server_poll(euc_server *srv, euc_server_completion *out, size_t max, size_t *n, int wait_ms);
/* Waits until nothing is pending or in flight (EUC_ERR_TIMEOUT after
 * `timeout_ms`, < 0: no limit).                                             */
int euc_server_drain(euc_server *srv, int timeout_ms);
int euc_server_stats_get(euc_server *srv, euc_server_stats *out);

#ifdef __cplusplus
}
#endif

#endif /* EUC_GB300_H */
