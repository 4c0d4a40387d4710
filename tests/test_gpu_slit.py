"""The 256x4x768 slit-array workload (eps 4.0, 80 cells thick, one 64-cell
air slit per period, 16-cell UPML, TF/SF at z = 40, DFT planes z = 30 and
z = 738) on its full grid over its full 8000 steps, against the FP64
oracle's spectra in tests/golden/slit_256x4x768_oracle.npz (written by
tests/golden/make_slit_fixture.py; 24 of the 300 frequencies, every output
block).

FP64 mode: every flux spectrum within 1e-12 norm-wise of the oracle's.
FP32 mode (the default stepping, the persistent kernel on a grid this size;
tensor-core DFT): R = J5/(J5+J6) and T = J6/(J5+J6)
of the final block within 1e-4 of the oracle's, per spectrum; the errors
are printed.
"""
import importlib
import os
import sys
import tempfile

import numpy as np
import pytest

from conftest import golden
from helpers import engine_params_from_oracle, rel_err

pytestmark = pytest.mark.gpu
cfg = importlib.import_module("irisfdtd-academic_gb300.configs")
sys.path.insert(0, os.path.dirname(golden("x")))
import make_slit_fixture as F  # noqa: E402


@pytest.fixture(scope="module")
def fixture():
    return np.load(golden("slit_256x4x768_oracle.npz"))


def run(iris, oracle, precision):
    d = tempfile.mkdtemp(prefix="slit_")
    path, w = F.deck(d)
    op = oracle.setparam(path)
    e = iris.Engine(engine_params_from_oracle(iris, op, precision=precision), op.fw)
    e.set_material(cfg.slit_material(w))
    blocks, its, it = [], [], 1
    for t in range(1, op.texit + 1):
        if t >= op.to_fourier and (t == op.texit or (t - op.to_fourier) % op.no_downloads == 0):
            e.step(it, t - it + 1)
            blocks.append(e.flux(0))
            its.append(t)
            it = t + 1
    e.close()
    return op, np.asarray(blocks), its


def test_slit_fp64_spectra_against_oracle(iris, oracle, fixture):
    op, J, its = run(iris, oracle, 0)
    assert its == list(fixture["its"]) and op.texit == int(fixture["steps"]) == 8000
    assert np.array_equal(np.asarray(op.fw), fixture["fw"])
    Jo = fixture["J"]
    assert rel_err(J, Jo) <= 1e-12
    for f in range(6):
        assert rel_err(J[-1, f], Jo[-1, f]) <= 1e-12, f


def test_slit_fp32_tr_against_oracle(iris, oracle, fixture):
    op, J, its = run(iris, oracle, 1)
    Jo = fixture["J"]
    R, T = iris.tr_normalise(J[-1, 4], J[-1, 5])
    Ro, To = oracle.tr_normalise(Jo[-1, 4], Jo[-1, 5])
    eR, eT = float(np.max(np.abs(R - Ro))), float(np.max(np.abs(T - To)))
    print(f"slit 256x4x768, 8000 steps, FP32 vs FP64 oracle: max |dR| = {eR:.3e}, max |dT| = {eT:.3e}")
    assert eR <= 1e-4 and eT <= 1e-4
