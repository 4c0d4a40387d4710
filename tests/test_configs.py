"""The geometry front-end (configs.py) on the CPU: the voxelisers' layout
(eps_inv over (hi-1:hf+1, 0:ny+1, 0:nx+1), the planes hi-1 and hf+1 holding
1/eps1 and 1/eps3 as in code/mesh.f90:57-109), periodic ghosts, seeded
determinism, the slit against struct_limit (code/files.f90:385-409) as both
the oracle and the engine's parser compute it, and the batched form's cell
sizes."""
import importlib
import math

import numpy as np
import pytest

cfg = importlib.import_module("irisfdtd-academic_gb300.configs")


def small_spheres():
    w = cfg.resized(cfg.workload(3), 40, 24, 160, nof=8)
    w.extra = dict(w.extra, nspheres=12, rmin=2, rmax=6)
    return w


def test_spheres_layout_and_ghosts():
    w = small_spheres()
    a = cfg.spheres_material(w, seed=4)
    hf = w.hi + w.dh - 1
    assert a.shape == (hf - w.hi + 3, w.ny + 2, w.nx + 2) and a.dtype == np.complex128
    assert np.all(a[0] == 1.0 / w.eps1) and np.all(a[-1] == 1.0 / w.eps3)
    inner = a[1:-1]
    assert np.array_equal(inner[:, :, 0], inner[:, :, -2]) and np.array_equal(inner[:, :, -1], inner[:, :, 1])
    assert np.array_equal(inner[:, 0, :], inner[:, -2, :]) and np.array_equal(inner[:, -1, :], inner[:, 1, :])
    ex = w.extra
    v = inner[:, 1:-1, 1:-1].real
    spheres = v != 1.0 / w.eps_bbox
    assert spheres.any() and (~spheres).any()
    assert np.all(v[spheres] >= 1.0 / ex["emax"] - 1e-15) and np.all(v[spheres] <= 1.0 / ex["emin"] + 1e-15)
    assert not np.any(inner.imag)
    assert np.array_equal(a, cfg.spheres_material(w, seed=4))
    assert not np.array_equal(a, cfg.spheres_material(w, seed=5))


def test_binary_pattern_and_design_region():
    c = cfg.batch_cells(3, seed=7, nof=8)[2]
    a = cfg.binary_pattern_material(c)
    v = a[1:-1, 1:-1, 1:-1]
    assert set(np.unique(v.real)) <= {1.0, 0.25}
    fill = np.mean(v.real == 0.25)
    assert abs(fill - c.extra["fill"]) < 0.05
    w = cfg.workload(5)
    d = cfg.design_region_material(w, seed=1)
    ex = w.extra
    region = d[1:-1, ex["y0"]:ex["y1"] + 1, ex["x0"]:ex["x1"] + 1].real
    assert np.all(region >= 1.0 / ex["emax"]) and np.all(region <= 1.0 / ex["emin"])
    outside = d[1:-1].real.copy()
    outside[:, ex["y0"]:ex["y1"] + 1, ex["x0"]:ex["x1"] + 1] = 1.0
    assert np.all(outside == 1.0)


@pytest.mark.parametrize("n,d", [(256, 64), (100, 20), (7, 3), (8, 3), (9, 4), (10, 5), (31, 1)])
def test_slit_matches_struct_limit(iris, oracle, tmp_path, n, d):
    w = cfg.Workload("slit", n, 1, 64, 8, 57, 24, 10, 4.0, d, 12, (1, n, 1, 1, 10, 50), 8, 10, structure="slit")
    a = cfg.slit_material(w)
    cols = np.nonzero(np.all(a[1:-1, 1:-1, :].real == 1.0, axis=(0, 1)))[0]
    ai, af = oracle.struct_limit(n, d)
    assert (cols.min(), cols.max(), cols.size) == (ai, af, af - ai + 1)
    p, _, _ = iris.setparam(cfg.write_input(str(tmp_path / "in.dat"), w))
    assert (p.aix, p.afx) == (ai, af)


def test_batch_cells_sizes_and_seeds():
    cells = cfg.batch_cells(64, seed=3, nof=8)
    for w in cells:
        assert 32 <= w.nx <= 160 and 32 <= w.ny <= 160 and 256 <= w.nz <= 768
        assert w.pmlzi == 16 and w.pmlzf == w.nz - 15 and w.dh == 64 and w.hi == w.nz // 2 - 32
        assert w.box[4] < w.hi and w.box[5] > w.hi + w.dh - 1
    again = cfg.batch_cells(64, seed=3, nof=8)
    assert [(w.nx, w.ny, w.nz) for w in cells] == [(w.nx, w.ny, w.nz) for w in again]
    assert len({(w.nx, w.ny, w.nz) for w in cells}) > 50  # uneven


def test_resized_keeps_distances_to_the_ends():
    w = cfg.workload(3)
    r = cfg.resized(w, 256, 128, 200, nof=16)
    assert (r.nx, r.ny, r.nz, r.nof) == (256, 128, 200, 16)
    assert r.pmlzi == w.pmlzi and r.nz - r.pmlzf == w.nz - w.pmlzf
    assert r.box[4] == w.box[4] and r.nz - r.box[5] == w.nz - w.box[5]
    assert r.tfsf_zi == w.tfsf_zi and r.hi >= r.tfsf_zi + 8
    assert math.isclose(r.akx, 0.3 * math.pi * 256)
