"""Committed golden fixtures (tests/golden/*.npz, made by make_golden.py):
the oracle and the pure-Python restatement reproduce them on the CPU, and the
GPU pipeline reproduces them through the C ABI."""
import glob
import os
import sys

import numpy as np
import pytest

from euc_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import golden_io  # noqa: E402
from frameutil import assert_targets_match, run_gpu  # noqa: E402

FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
IDS = [os.path.basename(f)[:-4] for f in FIXTURES]


def _tol(frame):
    return 1 if any(p.desc.shader == abi.SHADER_PHONG for p in frame.passes) else 0


def test_fixtures_exist():
    assert len(FIXTURES) >= 6


@pytest.mark.parametrize("path", FIXTURES, ids=IDS)
def test_oracle_reproduces_fixture(path):
    from oracle import oracle
    frame, expected, stats = golden_io.load(path)
    got, st, codes = oracle.run_frame(frame)
    assert codes == [abi.OK] * len(frame.passes)
    assert [int(s.candidates) for s in st] == [s[0] for s in stats]
    assert_targets_match(frame, expected, got, color_tol=0)


@pytest.mark.parametrize("path", FIXTURES, ids=IDS)
def test_python_restatement_reproduces_fixture(path):
    from oracle import euc_pyref
    frame, expected, stats = golden_io.load(path)
    got, res = euc_pyref.run_frame(frame)
    assert [r[1] for r in res] == [s[0] for s in stats]
    assert_targets_match(frame, expected, got, color_tol=_tol(frame))


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=IDS)
def test_gpu_reproduces_fixture(path, gpu_ctx):
    frame, expected, stats = golden_io.load(path)
    got, st = run_gpu(gpu_ctx, frame)
    assert [s[0] for s in st] == [abi.OK] * len(frame.passes)
    assert [s[1] for s in st] == [s[0] for s in stats]
    assert_targets_match(frame, expected, got, color_tol=_tol(frame))
