"""The C++ oracle against the independent pure-Python restatement
(oracle/euc_pyref.py) on small scenes covering every mode: targets
bit-identical and candidate-fragment counts equal."""
import ctypes as C

import numpy as np
import pytest

from euc_gb300 import abi, scenes
from oracle import euc_pyref, oracle


def _run_both(make):
    fa, fb = make(), make()
    ref, stats, codes = oracle.run_frame(fa)
    py, res = euc_pyref.run_frame(fb)
    assert codes == [r[0] for r in res]
    assert [s.candidates for s in stats] == [r[1] for r in res]
    for k in ref:
        if ref[k].dtype == np.float32:
            assert np.array_equal(ref[k].view(np.uint32), py[k].view(np.uint32)), k
        else:
            assert np.array_equal(ref[k], py[k]), k


def _soup(seed, w=48, h=32, n=60, hi=400.0, alpha=False, **desc):
    def make():
        f = scenes.soup_frame(seed=seed, width=w, height=h, ntris=n, area_lo=2.0, area_hi=hi, alpha=alpha)
        for k, v in desc.items():
            setattr(f.passes[0].desc, k, v)
        return f
    return make


CASES = {
    "sphere": lambda: scenes.sphere_frame(seed=2, width=61, height=45, lon=12, lat=6),
    "sphere_bands3": lambda: scenes.sphere_frame(seed=2, width=61, height=45, lon=12, lat=6, band_rows=3),
    "sphere_yup_front": lambda: _mod(scenes.sphere_frame(seed=4, width=50, height=40, lon=10, lat=5),
                                     y_axis=abi.Y_UP, cull=abi.CULL_FRONT),
    "soup_less": _soup(1),
    "soup_greater": _soup(2, depth_test=abi.TEST_GREATER),
    "soup_equal": _soup(3, depth_test=abi.TEST_EQUAL),
    "soup_none_write": _soup(4, depth_test=abi.TEST_NONE),
    "soup_pass": _soup(5, depth_write=0),
    "soup_depth_only": _soup(6, pixel_write=0),
    "soup_big": _soup(7, w=64, h=48, n=12, hi=6000.0),
    "soup_bands2": _soup(8, band_rows=2),
    "soup_alpha": _soup(9, alpha=True),
    "soup_alpha_pass": _soup(10, alpha=True, depth_write=0),
    "soup_alpha_msaa1": _soup(11, alpha=True, aa_level=1),
    "knot_msaa1": lambda: scenes.knot_frame(seed=1, width=40, height=30, shadow_size=32, tubular=24, radial=6,
                                            tex_size=16, aa_level=1),
    "knot_msaa2_bands": lambda: scenes.knot_frame(seed=2, width=44, height=30, shadow_size=32, tubular=24, radial=6,
                                                  tex_size=16, aa_level=2, band_rows=5),
}


def _mod(f, **desc):
    for k, v in desc.items():
        setattr(f.passes[0].desc, k, v)
    return f


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_python_restatement(name):
    _run_both(CASES[name])


@pytest.mark.parametrize("filt", [abi.FILTER_NEAREST, abi.FILTER_LINEAR])
@pytest.mark.parametrize("wrap", [abi.WRAP_NONE, abi.WRAP_CLAMP, abi.WRAP_TILE, abi.WRAP_MIRROR])
def test_sampler_matches_python_restatement(filt, wrap):
    rng = np.random.default_rng(filt * 10 + wrap)
    tex = rng.integers(0, 256, (7, 9, 4), dtype=np.uint8)
    s = abi.Sampler(tex.ctypes.data, 9, 7, 36, abi.FMT_RGBA8, filt, wrap, 255.0, 0)
    py = euc_pyref.Tex((tex, filt, wrap, 255.0))
    coords = np.concatenate([rng.uniform(-2.5, 2.5, 300), [0.0, -0.0, 1.0, -1.0, 0.5, 2.0, 1e-9, -1e-9, 0.999999]])
    for u in coords.astype(np.float32):
        for v in coords[::7].astype(np.float32):
            a = oracle.sample(s, float(u), float(v))
            b = np.array(py.sample(u, v), dtype=np.float32)
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (u, v, a, b)
