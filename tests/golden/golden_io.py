"""Serialises scenes.FrameSpec inputs and reference outputs to .npz fixtures.

A fixture stores every input byte (vertex buffers, indices, descriptor,
layout, uniforms, textures, target specs), so it does not depend on the
generators producing the same floats on another machine.
"""
import ctypes as C
import json

import numpy as np

from euc_gb300 import abi, scenes


def save(path, frame, targets, stats):
    arrays = {}
    meta = {"name": frame.name, "targets": [], "passes": [], "stats": stats}
    for t in frame.targets:
        meta["targets"].append([t.name, t.width, t.height, t.fmt,
                                float(t.clear) if t.fmt == abi.FMT_R32F else int(t.clear)])
        arrays["out_" + t.name] = targets[t.name]
    for k, p in enumerate(frame.passes):
        arrays["p%d_desc" % k] = np.frombuffer(bytes(p.desc), dtype=np.uint8)
        arrays["p%d_layout" % k] = np.frombuffer(bytes(p.layout), dtype=np.uint8)
        arrays["p%d_uniforms" % k] = np.frombuffer(C.string_at(C.addressof(p.uniforms), C.sizeof(p.uniforms)),
                                                  dtype=np.uint8)
        arrays["p%d_vertices" % k] = p.vertices
        if p.indices is not None:
            arrays["p%d_indices" % k] = p.indices
        samp = []
        for j, s in enumerate(p.samplers):
            if isinstance(s.source, str):
                src = s.source
            else:
                src = None
                arrays["p%d_tex%d" % (k, j)] = s.source
            samp.append([s.field, src, s.filter, s.wrap, s.texel_div])
        meta["passes"].append({"shader": p.desc.shader, "nverts": p.nverts, "pixel": p.pixel, "depth": p.depth,
                               "samplers": samp})
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(path, **arrays)


def load(path):
    """Returns (FrameSpec, expected targets dict, stats list)."""
    z = np.load(path)
    meta = json.loads(bytes(z["meta"]).decode())
    targets = [scenes.TargetSpec(n, w, h, f, c) for n, w, h, f, c in meta["targets"]]
    passes = []
    for k, pm in enumerate(meta["passes"]):
        raw = z["p%d_desc" % k].tobytes()
        # fixtures written before the desc grew its `primitives` field hold a
        # shorter struct: the missing fields are 0 (TriangleList)
        raw += bytes(max(0, C.sizeof(abi.PipelineDesc) - len(raw)))
        desc = abi.PipelineDesc.from_buffer_copy(raw)
        lay = abi.VertexLayout.from_buffer_copy(z["p%d_layout" % k].tobytes())
        uni = abi.UNIFORMS_FOR_SHADER[pm["shader"]].from_buffer_copy(z["p%d_uniforms" % k].tobytes())
        idx = z["p%d_indices" % k] if ("p%d_indices" % k) in z.files else None
        samp = []
        for j, (field, src, filt, wrap, div) in enumerate(pm["samplers"]):
            source = src if src is not None else z["p%d_tex%d" % (k, j)]
            samp.append(scenes.SamplerSpec(field, source, filt, wrap, div))
        passes.append(scenes.PassSpec(desc, lay, z["p%d_vertices" % k], pm["nverts"], idx, uni, samp,
                                      pm["pixel"], pm["depth"]))
    frame = scenes.FrameSpec(meta["name"], targets, passes)
    expected = {t.name: z["out_" + t.name] for t in targets}
    return frame, expected, meta["stats"]
