"""ctypes mirror of include/euc_gb300.h (structs, enums, constants).

Field order and types match the C header exactly; `tests/test_abi.py` checks
the struct sizes against the C compiler's.
"""
import ctypes as C

ABI_VERSION = 2

# status codes
OK = 0
ERR_INVALID = 1
ERR_SIZE_MISMATCH = 2
ERR_INDEX_OOB = 3
ERR_OOM = 4
ERR_CUDA = 5
ERR_BAND = 6
ERR_TIMEOUT = 7
ERR_BUDGET = 8
ERR_CAPACITY = 9
ERR_STALE = 10
ERR_BUSY = 11

STATUS_NAMES = {
    OK: "EUC_OK", ERR_INVALID: "EUC_ERR_INVALID", ERR_SIZE_MISMATCH: "EUC_ERR_SIZE_MISMATCH",
    ERR_INDEX_OOB: "EUC_ERR_INDEX_OOB", ERR_OOM: "EUC_ERR_OOM", ERR_CUDA: "EUC_ERR_CUDA",
    ERR_BAND: "EUC_ERR_BAND", ERR_TIMEOUT: "EUC_ERR_TIMEOUT", ERR_BUDGET: "EUC_ERR_BUDGET",
    ERR_CAPACITY: "EUC_ERR_CAPACITY",
    ERR_STALE: "EUC_ERR_STALE",
    ERR_BUSY: "EUC_ERR_BUSY",
}

TEST_NONE, TEST_LESS, TEST_EQUAL, TEST_GREATER = 0, 1, 2, 3
PRIM_TRIANGLE_LIST, PRIM_LINE_TRIANGLE_LIST, PRIM_LINE_LIST = 0, 1, 2
SRC_RGBA8, SRC_BGRA8, SRC_RGB8, SRC_LUMA8, SRC_LUMA_ALPHA8, SRC_R32F = 0, 1, 2, 3, 4, 5
GEOM_NONE, GEOM_SUBDIVIDE, GEOM_SHRINK, GEOM_DUPLICATE, GEOM_DISCARD = 0, 1, 2, 3, 4
HOST_COPY_AUTO, HOST_COPY_STAGED, HOST_COPY_DIRECT = 0, 1, 2
CULL_NONE, CULL_BACK, CULL_FRONT = 0, 1, 2
Y_DOWN, Y_UP = 0, 1
LEFT, RIGHT = 0, 1
FMT_NONE, FMT_RGBA8, FMT_BGRA8, FMT_RGB8, FMT_R32F, FMT_RGBA32F = 0, 1, 2, 3, 4, 5
SHADER_FLAT, SHADER_VCOLOR, SHADER_GOURAUD, SHADER_TEXTURED, SHADER_PHONG, SHADER_SHADOW = range(6)
BLEND_REPLACE, BLEND_ALPHA = 0, 1
FILTER_NEAREST, FILTER_LINEAR = 0, 1
WRAP_NONE, WRAP_CLAMP, WRAP_TILE, WRAP_MIRROR = 0, 1, 2, 3
BANDS_PAR = 0
BANDS_SEQ = 0xFFFFFFFF
FLAG_PAR_EMPTY = 1
FLAG_ORDERED = 2

STAGE_NAMES = ("vertex", "setup", "scan", "init", "raster", "resolve")
STAGE_COUNT = len(STAGE_NAMES)

FMT_BPP = {FMT_NONE: 0, FMT_RGBA8: 4, FMT_BGRA8: 4, FMT_RGB8: 3, FMT_R32F: 4, FMT_RGBA32F: 16}


class PipelineDesc(C.Structure):
    _fields_ = [
        ("shader", C.c_uint32), ("pixel_write", C.c_uint32), ("depth_test", C.c_uint32),
        ("depth_write", C.c_uint32), ("handedness", C.c_uint32), ("y_axis", C.c_uint32),
        ("z_clip", C.c_uint32), ("z_clip_min", C.c_float), ("z_clip_max", C.c_float),
        ("aa_level", C.c_uint32), ("cull", C.c_uint32), ("blend", C.c_uint32),
        ("band_rows", C.c_uint32), ("flags", C.c_uint32), ("primitives", C.c_uint32),
        ("geometry", C.c_uint32), ("geometry_param", C.c_float),
    ]


class Target(C.Structure):
    _fields_ = [("data", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32),
                ("pitch", C.c_uint32), ("format", C.c_uint32)]


class Sampler(C.Structure):
    _fields_ = [("data", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32),
                ("pitch", C.c_uint32), ("format", C.c_uint32), ("filter", C.c_uint32),
                ("wrap", C.c_uint32), ("texel_div", C.c_float), ("reserved", C.c_uint32)]


class VertexLayout(C.Structure):
    _fields_ = [("stride", C.c_uint32), ("position", C.c_int32), ("normal", C.c_int32),
                ("uv", C.c_int32), ("color", C.c_int32)]


Mat4 = C.c_float * 16


class FlatUniforms(C.Structure):
    _fields_ = [("mvp", Mat4), ("color", C.c_float * 4)]


class VColorUniforms(C.Structure):
    _fields_ = [("mvp", Mat4)]


class GouraudUniforms(C.Structure):
    _fields_ = [("mvp", Mat4), ("model", Mat4), ("to_light", C.c_float * 3), ("ambient", C.c_float),
                ("color", C.c_float * 3), ("diffuse", C.c_float)]


class TexturedUniforms(C.Structure):
    _fields_ = [("mvp", Mat4), ("tex", Sampler)]


class PhongUniforms(C.Structure):
    _fields_ = [("model", Mat4), ("view", Mat4), ("proj", Mat4), ("light_vp", Mat4),
                ("light_pos", C.c_float * 3), ("normal_sign", C.c_float), ("cam_pos", C.c_float * 3),
                ("ambient", C.c_float), ("surf_color", C.c_float * 4), ("tex", Sampler),
                ("shadow", Sampler)]


class ShadowUniforms(C.Structure):
    _fields_ = [("mvp", Mat4)]


UNIFORMS_FOR_SHADER = {
    SHADER_FLAT: FlatUniforms, SHADER_VCOLOR: VColorUniforms, SHADER_GOURAUD: GouraudUniforms,
    SHADER_TEXTURED: TexturedUniforms, SHADER_PHONG: PhongUniforms, SHADER_SHADOW: ShadowUniforms,
}


class Stats(C.Structure):
    _fields_ = [("triangles", C.c_uint64), ("culled", C.c_uint64), ("candidates", C.c_uint64)]


class Tuning(C.Structure):
    _fields_ = [("raster_blocks_per_sm", C.c_uint32), ("raster_warp_rows", C.c_uint32),
                ("chunk_group", C.c_uint32), ("chunk_blocks_per_sm", C.c_uint32), ("raster_probe", C.c_uint32),
                ("host_copy", C.c_uint32), ("strip_path", C.c_uint32)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class Scene(C.Structure):
    _fields_ = [("desc", PipelineDesc), ("layout", VertexLayout), ("vertices", C.c_void_p),
                ("nverts", C.c_uint64), ("indices", C.c_void_p), ("nindices", C.c_uint64),
                ("pixel", Target), ("depth", Target), ("uniforms", C.c_void_p),
                ("uniforms_size", C.c_uint64)]


def mat4(values):
    """Row-major float[16] from any 4x4 array-like."""
    flat = [float(v) for row in values for v in row] if hasattr(values[0], "__len__") else [float(v) for v in values]
    return Mat4(*flat)


def status_name(code):
    return STATUS_NAMES.get(code, "EUC_STATUS_%d" % code)


# ---- serving --------------------------------------------------------------
SERVER_MAX_TARGETS = 4
SERVER_MAX_PASSES = 4


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_batch", C.c_uint32), ("framebuffer_budget", C.c_uint64),
                ("slots", C.c_uint32), ("max_pending", C.c_uint32)]


class ServerTarget(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("format", C.c_uint32), ("clear", C.c_uint32),
                ("readback", C.c_uint32), ("reserved", C.c_uint32)]


class ServerBinding(C.Structure):
    _fields_ = [("offset", C.c_uint32), ("texture", C.c_int32), ("target", C.c_int32), ("reserved", C.c_uint32)]


class ServerPass(C.Structure):
    _fields_ = [("desc", PipelineDesc), ("mesh", C.c_uint32), ("pixel_target", C.c_int32),
                ("depth_target", C.c_int32), ("nbindings", C.c_uint32), ("bindings", C.POINTER(ServerBinding)),
                ("uniforms", C.c_void_p), ("uniforms_size", C.c_uint64)]


class ServerRequest(C.Structure):
    _fields_ = [("tag", C.c_uint64), ("arrival_ns", C.c_uint64), ("out", C.c_void_p), ("out_size", C.c_uint64),
                ("ntargets", C.c_uint32), ("npasses", C.c_uint32), ("targets", C.POINTER(ServerTarget)),
                ("passes", C.POINTER(ServerPass))]


class ServerCompletion(C.Structure):
    _fields_ = [("id", C.c_uint64), ("tag", C.c_uint64), ("status", C.c_int32), ("batch_size", C.c_uint32),
                ("arrival_ns", C.c_uint64), ("admit_ns", C.c_uint64), ("done_ns", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("submitted", "completed", "failed", "refused", "pending", "in_flight",
                                          "batches", "batched_requests", "budget_bytes", "budget_used",
                                          "budget_peak", "launches")]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}
