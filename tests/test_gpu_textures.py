"""N-D nearest sampling (euc_sample_nearest) and texture ingest
(euc_texture_ingest) on the GPU against the oracle: byte-exact."""
import ctypes as C

import numpy as np
import pytest

from euc_gb300 import abi, capi
from oracle import oracle

pytestmark = pytest.mark.gpu


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("shape,tb", [((17,), 1), ((9, 33), 4), ((5, 7, 11), 3), ((3, 4, 5, 6), 16),
                                      ((1, 1), 2), ((2049,), 8)])
@pytest.mark.parametrize("wrap", [abi.WRAP_NONE, abi.WRAP_CLAMP, abi.WRAP_TILE, abi.WRAP_MIRROR])
def test_sample_nearest_matches_oracle(shape, tb, wrap):
    import torch
    rng = np.random.default_rng(len(shape) * 10 + tb + wrap)
    ndim = len(shape)
    tex = rng.integers(0, 256, tuple(reversed(shape)) + (tb,), dtype=np.uint8)
    q = rng.uniform(-2.5, 2.5, (4099, ndim)).astype(np.float32)
    q[:50] = rng.choice(np.array([0.0, 1.0, -0.0, 0.5, np.nan, np.inf, -np.inf, 1e30], dtype=np.float32), (50, ndim))
    want = oracle.sample_nearest(tex, q, wrap)
    dt = torch.from_numpy(tex).cuda()
    dq = torch.from_numpy(q).cuda()
    out = torch.zeros((len(q), tb), dtype=torch.uint8, device="cuda")
    size = (C.c_uint32 * ndim)(*shape)
    rc = capi.lib().euc_sample_nearest(dt.data_ptr(), ndim, size, tb, wrap, dq.data_ptr(), len(q), out.data_ptr(),
                                       _stream())
    assert rc == abi.OK
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), want)


def test_sample_nearest_refuses_bad_shapes():
    size = (C.c_uint32 * 2)(4, 0)
    assert capi.lib().euc_sample_nearest(None, 2, size, 4, 0, None, 1, None, None) == abi.ERR_INVALID
    size = (C.c_uint32 * 5)(1, 1, 1, 1, 1)
    assert capi.lib().euc_sample_nearest(None, 5, size, 4, 0, None, 1, None, None) == abi.ERR_INVALID


@pytest.mark.parametrize("fmt,ch,dtype", [(abi.SRC_RGBA8, 4, np.uint8), (abi.SRC_BGRA8, 4, np.uint8),
                                          (abi.SRC_RGB8, 3, np.uint8), (abi.SRC_LUMA8, 1, np.uint8),
                                          (abi.SRC_LUMA_ALPHA8, 2, np.uint8), (abi.SRC_R32F, 1, np.float32)])
@pytest.mark.parametrize("where", ["host", "device"])
def test_texture_ingest_matches_oracle(fmt, ch, dtype, where):
    import torch
    rng = np.random.default_rng(fmt * 2 + (where == "device"))
    h, w = 37, 53
    if dtype == np.float32:
        img = rng.standard_normal((h, w)).astype(np.float32)
    else:
        img = rng.integers(0, 256, (h, w, ch), dtype=np.uint8)
        if ch == 1:
            img = img[..., 0]
    want = oracle.texture_ingest(img, fmt)
    ctx = capi.Context(0)
    try:
        dst = torch.zeros((h, w + 3, 4), dtype=torch.uint8, device="cuda")  # padded rows
        src = np.ascontiguousarray(img)
        keep = src
        ptr = src.ctypes.data
        if where == "device":
            keep = torch.from_numpy(src).cuda()
            ptr = keep.data_ptr()
        rc = capi.lib().euc_texture_ingest(ctx.handle, ptr, w, h, src.strides[0], fmt, dst.data_ptr(),
                                           dst.stride(0), _stream())
        assert rc == abi.OK
        torch.cuda.synchronize()
        got = dst.cpu().numpy()[:, :w]
        assert np.array_equal(got, want)
        assert (dst.cpu().numpy()[:, w:] == 0).all()  # the row padding is not written
        del keep
    finally:
        ctx.close()
