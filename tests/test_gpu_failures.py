"""Failure handling that faults nothing (the reference's only failure path is
err() -> STOP, code/files.f90:352-381; here every call returns a status):

* a non-finite value put into the material on the host spreads through the
  fields and reaches the DFT planes: iris_flux returns IRIS_ENAN (in both
  precisions), and the engine object is still usable (destroyed cleanly, a
  new one steps normally);
* a device allocation that cannot succeed (a grid whose fields exceed the
  GPU's memory, or DFT accumulators that exceed what is left) makes
  iris_create return IRIS_ENOMEM after freeing what it had allocated; the
  next engine is created and steps as if nothing happened.
The bounded device waits are covered in tests/test_gpu_stream.py and
tests/test_gpu_persistent.py.
"""
import importlib

import numpy as np
import pytest

from helpers import engine_params_from_oracle

pytestmark = pytest.mark.gpu
cfg = importlib.import_module("irisfdtd-academic_gb300.configs")


def small(oracle, tmp_path, name="f"):
    w = cfg.Workload(name, 8, 6, 60, 6, 55, 24, 8, 4.0, 0, 10, (1, 8, 1, 6, 8, 52), 6, 200)
    return w, oracle.setparam(cfg.write_input(str(tmp_path / f"{name}.dat"), w, no_downloads=2))


@pytest.mark.parametrize("precision", [0, 1])
def test_nan_in_material_is_reported_by_flux(iris, oracle, tmp_path, precision):
    w, op = small(oracle, tmp_path)
    e = iris.Engine(engine_params_from_oracle(iris, op, precision=precision), op.fw)
    eps = np.asarray(iris.set_emconstants(e.p)).real.copy()
    eps[3, 2, 4] = np.nan  # one structure cell
    e.set_material(eps)
    e.step(1, 120)
    with pytest.raises(iris.IrisError) as x:
        e.flux(0)
    assert x.value.code == -6
    e.close()
    # a clean engine on the same device steps normally afterwards
    ok = iris.Engine(engine_params_from_oracle(iris, op, precision=precision), op.fw)
    ok.step(1, 120)
    assert np.all(np.isfinite(ok.flux(0)))


def test_allocation_failures_return_enomem(iris, oracle, tmp_path):
    w, op = small(oracle, tmp_path)
    # fields of 3000^3 cells: about 650 GB per field in FP32
    big = engine_params_from_oracle(iris, op, precision=1)
    big.nx = big.ny = big.nz = 3000
    big.pmlzf, big.hi, big.hf = 2990, 1000, 1010
    big.box1[:] = big.box2[:] = [1, 3000, 1, 3000, 30, 2970]
    with pytest.raises(iris.IrisError) as x:
        iris.Engine(big, op.fw)
    assert x.value.code == -2
    # fields that fit, DFT accumulators that do not: 1e5 frequencies on every face of a 512x512x64 cell
    acc = engine_params_from_oracle(iris, op, precision=1)
    acc.nx, acc.ny, acc.nz, acc.pmlzf, acc.hi, acc.hf = 512, 512, 64, 58, 20, 27
    acc.box1[:] = acc.box2[:] = [1, 512, 1, 512, 8, 56]
    acc.nof = 100000
    fw = np.linspace(0.01, 0.2, acc.nof)
    with pytest.raises(iris.IrisError) as x:
        iris.Engine(acc, fw)
    assert x.value.code == -2
    assert b"exceed" in iris.lib().iris_last_error()
    # the device is unharmed: a normal engine creates, steps and reads its flux
    ok = iris.Engine(engine_params_from_oracle(iris, op, precision=1), op.fw)
    ok.step(1, 50)
    assert np.all(np.isfinite(ok.flux(0)))
