"""Two shortcuts of the samplers (euc_device.cuh) that must give the same bits
as the operations they replace; each test compiles a host program against the
header and compares.  No GPU is needed.

- An RGBA8 channel is read as (u8 as f32) / 255.0 from a table that the
  compiler fills (ByteOver255): all 256 entries against a run-time division.
- The wraps' rem_euclid takes fmodf(x, m) for m = 1 or 2 as
  x - m * trunc(x / m) with x's sign (fmod_1_or_2): every 257th bit pattern of
  the floats (all exponents, both signs), and the special values, against
  fmod.  (Checked once over all 2^32 patterns as well: no difference.)"""
import os
import shutil
import subprocess

import pytest

from euc_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include <cstdio>
#include <cstring>
#include "euc_device.cuh"
int main() {
    constexpr eucg::ByteOver255 table{};
    volatile float div = 255.0f;  // a run-time division, not folded
    int bad = 0;
    for (int i = 0; i < 256; ++i) {
        const float q = (float)i / div;
        unsigned a, b;
        std::memcpy(&a, &q, 4);
        std::memcpy(&b, &table.v[i], 4);
        if (a != b) {
            std::printf("byte %d: table %08x, division %08x\n", i, b, a);
            ++bad;
        }
    }
    std::printf("%d mismatches\n", bad);
    return bad != 0;
}
"""


FMOD_SRC = r"""
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include "euc_device.cuh"
int main() {
    long bad = 0;
    auto check = [&](float x, float m) {
        const float a = std::fmod(x, m), b = eucg::fmod_1_or_2(x, m);
        uint32_t ua, ub;
        std::memcpy(&ua, &a, 4);
        std::memcpy(&ub, &b, 4);
        if (ua != ub && !(std::isnan(a) && std::isnan(b))) {
            if (bad < 10) std::printf("x %a m %g: fmod %a, shortcut %a\n", x, m, a, b);
            ++bad;
        }
    };
    for (uint64_t u = 0; u < (1ull << 32); u += 257) {
        const uint32_t v = (uint32_t)u;
        float x;
        std::memcpy(&x, &v, 4);
        check(x, 1.0f);
        check(x, 2.0f);
    }
    const float special[] = {0.0f, -0.0f, 1.0f, -1.0f, 2.0f, -2.0f, 0.5f, -0.5f, 1e-45f, -1e-45f, 16777216.0f,
                             -16777216.0f, 16777218.0f, 8388607.5f, -8388607.5f, 3.0e38f, -3.0e38f,
                             INFINITY, -INFINITY, NAN};
    for (float x : special) {
        check(x, 1.0f);
        check(x, 2.0f);
    }
    std::printf("%ld mismatches\n", bad);
    return bad != 0;
}
"""


def _run(tmp_path, name, src):
    nvcc = build.nvcc()
    if not (os.path.exists(nvcc) or shutil.which(nvcc)):
        pytest.skip("nvcc not found")
    path = tmp_path / (name + ".cu")
    path.write_text(src)
    exe = tmp_path / name
    cmd = [nvcc] + build.ARCH + ["-O2", "-std=c++17", "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"),
                                 "-I", os.path.join(ROOT, "euc_gb300", "csrc"), str(path), "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True, timeout=300)
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout
    assert "0 mismatches" in run.stdout


def test_byte_table_equals_division(tmp_path):
    _run(tmp_path, "texel_table", SRC)


def test_wrap_fmod_equals_fmod(tmp_path):
    _run(tmp_path, "wrap_fmod", FMOD_SRC)
