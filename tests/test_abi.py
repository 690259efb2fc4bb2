"""The C ABI without a GPU: struct layouts agree between include/euc_gb300.h
(as the C compiler sees it) and the ctypes mirror, and libeuc_gb300.so loads
and exports every function the header declares."""
import ctypes as C
import os
import re
import subprocess

import pytest

from euc_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "euc_gb300.h")

STRUCTS = {
    "euc_pipeline_desc": abi.PipelineDesc, "euc_target": abi.Target, "euc_sampler": abi.Sampler,
    "euc_vertex_layout": abi.VertexLayout, "euc_flat_uniforms": abi.FlatUniforms,
    "euc_vcolor_uniforms": abi.VColorUniforms, "euc_gouraud_uniforms": abi.GouraudUniforms,
    "euc_textured_uniforms": abi.TexturedUniforms, "euc_phong_uniforms": abi.PhongUniforms,
    "euc_shadow_uniforms": abi.ShadowUniforms, "euc_stats": abi.Stats, "euc_scene": abi.Scene,
    "euc_tuning": abi.Tuning, "euc_server_config": abi.ServerConfig, "euc_server_target": abi.ServerTarget,
    "euc_server_binding": abi.ServerBinding, "euc_server_pass": abi.ServerPass,
    "euc_server_request": abi.ServerRequest, "euc_server_completion": abi.ServerCompletion,
    "euc_server_stats": abi.ServerStats,
}


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^[a-z][\w\s\*]*?\b(euc_\w+)\s*\(", text, flags=re.M)))


def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / "sz.c"
    lines = ['#include "%s"' % HEADER, "#include <stdio.h>", "#include <stddef.h>", "int main(void){"]
    for name, cls in STRUCTS.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (name, name))
        for fname, _ in cls._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (name, fname, name, fname))
    lines.append("return 0;}")
    src.write_text("\n".join(lines))
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-std=c11", str(src), "-o", str(exe)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                         check=True).stdout.split("\n") if l)
    for name, cls in STRUCTS.items():
        assert int(out[name]) == C.sizeof(cls), name
        for fname, _ in cls._fields_:
            assert int(out["%s.%s" % (name, fname)]) == getattr(cls, fname).offset, (name, fname)


def test_header_declares_the_abi():
    fns = declared_functions()
    for f in ("euc_ctx_create", "euc_ctx_destroy", "euc_render", "euc_render_host", "euc_render_batch",
              "euc_ctx_sync", "euc_ctx_stats", "euc_ctx_reserve", "euc_status_string", "euc_abi_version"):
        assert f in fns


def test_library_loads_and_exports_every_declared_symbol():
    from euc_gb300 import build, capi
    build.build()
    lib = C.CDLL(build.LIB)
    missing = [f for f in declared_functions() if not hasattr(lib, f)]
    assert not missing, missing
    assert set(declared_functions()) <= set(capi.SIGNATURES)
    assert lib.euc_abi_version() == abi.ABI_VERSION


def test_library_has_no_cpu_fallback():
    """Without a GPU the library refuses to create a context instead of
    rendering on the CPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from euc_gb300 import capi
    h = C.c_void_p()
    rc = capi.lib().euc_ctx_create(0, C.byref(h))
    assert rc != abi.OK
