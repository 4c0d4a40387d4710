"""Material generated on the device (iris_material_spheres, _pattern, _design,
iris_batch_material_pattern) against the host voxelisers of configs.py:
the stored eps_inv (iris_get_material) equal value for value in both
precisions, and the fields stepped from either material equal bit for bit.
Cases cover spheres that cross the periodic x and y boundaries, spheres
wider than half the cell (bounding box cut at nx, ny cells), spheres that
reach past the structure layer in z, and design regions that touch the
cell's edges."""
import importlib

import numpy as np
import pytest

from helpers import engine_params_from_oracle

pytestmark = pytest.mark.gpu
cfg = importlib.import_module("irisfdtd-academic_gb300.configs")


def engine(iris, oracle, tmp_path, w, precision, name="m"):
    op = oracle.setparam(cfg.write_input(str(tmp_path / f"{name}.dat"), w))
    return op, iris.Engine(engine_params_from_oracle(iris, op, precision=precision), op.fw,
                           stencil=iris.STENCIL_SPLIT)


def same_material(iris, a, b):
    return np.array_equal(a.get_material(), b.get_material())


SPHERES = [
    # nx, ny, nz, hi, dh, nspheres, rmin, rmax
    (37, 21, 64, 20, 24, 9, 2.0, 7.0),
    (16, 12, 48, 14, 10, 5, 6.5, 9.5),   # wider than half the cell, taller than the layer
]


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("case", SPHERES)
def test_spheres_on_device_equal_host(iris, oracle, tmp_path, case, precision):
    nx, ny, nz, hi, dh, n, rmin, rmax = case
    w = cfg.Workload("sph", nx, ny, nz, 6, nz - 5, hi, dh, 1.0, 0, 10, (1, nx, 1, ny, 8, nz - 8), 5, 40,
                     structure="spheres", extra=dict(nspheres=n, rmin=rmin, rmax=rmax, emin=1.5, emax=6.0))
    host = cfg.spheres_material(w, seed=4)
    op, a = engine(iris, oracle, tmp_path, w, precision, "a")
    _, b = engine(iris, oracle, tmp_path, w, precision, "b")
    a.set_material(host)
    b.material_spheres(cfg.sphere_params(w, seed=4))
    assert same_material(iris, a, b)
    ref = host[1:-1].astype(np.complex64 if precision else np.complex128).astype(np.complex128)
    assert np.array_equal(b.get_material(), ref)
    for e in (a, b):
        e.step(1, 60)
    for which in (iris.E, iris.H):
        assert np.array_equal(a.get_field(which), b.get_field(which))


@pytest.mark.parametrize("precision", [0, 1])
def test_pattern_and_design_on_device_equal_host(iris, oracle, tmp_path, precision):
    w = cfg.Workload("pat", 33, 9, 48, 6, 43, 18, 8, 1.0, 0, 10, (1, 33, 1, 9, 8, 40), 5, 40,
                     structure="pattern", extra=dict(seed=77, fill=0.45))
    op, a = engine(iris, oracle, tmp_path, w, precision, "pa")
    _, b = engine(iris, oracle, tmp_path, w, precision, "pb")
    a.set_material(cfg.binary_pattern_material(w))
    b.material_pattern(cfg.pattern_seed(w), 0.45, 4.0, 1.0)
    assert same_material(iris, a, b)
    d = cfg.Workload("des", 20, 14, 48, 6, 43, 18, 8, 1.0, 0, 10, (1, 20, 1, 14, 8, 40), 5, 40, structure="design",
                     extra=dict(x0=1, x1=20, y0=3, y1=14, emin=1.0, emax=12.0))
    _, c = engine(iris, oracle, tmp_path, d, precision, "da")
    _, e = engine(iris, oracle, tmp_path, d, precision, "db")
    c.set_material(cfg.design_region_material(d, seed=9).real)
    e.material_design(9, (1, 20, 3, 14), 1.0, 12.0)
    assert same_material(iris, c, e)


def test_batch_pattern_on_device(iris, oracle, tmp_path):
    ws = cfg.batch_cells(3, seed=40, nsteps=30, nof=4)
    ws = [cfg.Workload(w.name, min(w.nx, 40), min(w.ny, 36), 300, 16, 285, 118, 64, 1.0, 0, 40,
                       (1, min(w.nx, 40), 1, min(w.ny, 36), 30, 270), 4, 30, structure="pattern", extra=w.extra)
          for w in ws]
    params = []
    for i, w in enumerate(ws):
        op = oracle.setparam(cfg.write_input(str(tmp_path / f"c{i}.dat"), w))
        params.append(engine_params_from_oracle(iris, op, precision=1))
    fw = oracle.setparam(str(tmp_path / "c0.dat")).fw
    host = iris.Batch(params, fw, dft_faces=iris.DFT_Z)
    dev = iris.Batch(params, fw, dft_faces=iris.DFT_Z)
    for i, w in enumerate(ws):
        host.set_material(i, cfg.binary_pattern_material(w))
        dev.material_pattern(i, cfg.pattern_seed(w), w.extra["fill"], 4.0, 1.0)
    for b in (host, dev):
        b.set_tile(5)
        b.step(1, 25)
    for i in range(len(ws)):
        assert np.array_equal(host.get_field(i, iris.E), dev.get_field(i, iris.E)), i
        assert np.array_equal(host.flux(i), dev.flux(i)), i
