"""The samplers read an RGBA8 channel as (u8 as f32) / 255.0 from a table that
the compiler fills (ByteOver255 in euc_device.cuh) instead of dividing.  The
table must hold exactly the correctly rounded quotients that the division
gives: this compiles the header's table as a constant expression in a host
program and compares all 256 entries, bit for bit, with a run-time division.
No GPU is needed."""
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


def test_byte_table_equals_division(tmp_path):
    nvcc = build.nvcc()
    if not (os.path.exists(nvcc) or shutil.which(nvcc)):
        pytest.skip("nvcc not found")
    src = tmp_path / "texel_table.cu"
    src.write_text(SRC)
    exe = tmp_path / "texel_table"
    cmd = [nvcc] + build.ARCH + ["-std=c++17", "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"),
                                 "-I", os.path.join(ROOT, "euc_gb300", "csrc"), str(src), "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True, timeout=300)
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, run.stdout
    assert "0 mismatches" in run.stdout
