"""The persistent whole-step kernel for small grids (IRIS_STENCIL_PERSISTENT,
the default up to PERSISTENT_MAX_CELLS cells in FP64 and
PERSISTENT_MAX_CELLS_FP32 in FP32): one cooperative launch runs a
span of steps (E pass, H pass, TF/SF, DFT sample) with grid-wide barriers
between the passes, using the split passes' per-cell functions.  Every
stored value (fields with their ghosts, UPML auxiliaries, DFT accumulators
and spectra) equals the split passes' bit for bit, in both precisions, for
both TF/SF variants, the CW source, complex materials and Bloch phases, DFT
sampling that starts late and skips steps, and DFT blocks that fill inside
a span, on grids small enough for 128-thread CTAs and on one that takes
1024.  Against the FP64 oracle it inherits the split passes' 1e-12
(the parity tests' small grids step with it by default).  The grid
barrier's bounded wait gives up cleanly (IRIS_OP_BARRIER_CHECK).
"""
import importlib
import os

import numpy as np
import pytest

from helpers import engine_params_from_oracle, output_steps, rel_err, run_engine_blocks

pytestmark = pytest.mark.gpu
cfg = importlib.import_module("irisfdtd-academic_gb300.configs")
THREADS = max(1, min(16, os.cpu_count() or 1))

# name, workload, ak, material kind, extra write_input keys, dft_faces
CASES = [
    ("slab_4x4x512_all_faces", cfg.Workload("w1", 4, 4, 512, 16, 497, 236, 40, 2.25, 0, 40, (1, 4, 1, 4, 30, 480), 20,
                                            300), (0j, 0j, 0j), None, {}, 0),
    ("slab_4x4x512_z_faces", cfg.Workload("w1z", 4, 4, 512, 16, 497, 236, 40, 2.25, 0, 40, (1, 4, 1, 4, 30, 480), 20,
                                          300), (0j, 0j, 0j), None, {}, 1),
    ("1d_slab_variant2", cfg.Workload("d1", 1, 1, 120, 12, 109, 50, 20, 9.0, 0, 20, (1, 1, 1, 1, 15, 100), 11, 260),
     (0j, 0j, 0j), None, {}, 0),
    ("3d_spheres_complex_bloch", cfg.Workload("sp", 37, 21, 64, 8, 57, 24, 14, 2.25, 0, 12, (1, 37, 1, 21, 9, 54), 9,
                                              150, structure="spheres",
                                              extra=dict(nspheres=6, rmin=2, rmax=5, emin=1.5, emax=6.0)),
     (0.4 + 0.05j, -0.2 + 0j, 0j), "complex", {"i_pol": 1}, 0),
    ("cw_late_sparse_sampling", cfg.Workload("cw", 12, 7, 60, 8, 53, 24, 10, 4.0, 0, 14, (2, 11, 1, 7, 10, 50), 7, 200,
                                             structure="slit"), (0.3 + 0j, 0j, 0j), None,
     {"plane_wave": 0, "to_fourier": 17, "sample_fourier": 3}, 0),
    # 294,912 cells: CTAs of 1024 threads in both precisions (the width grows with the grid)
    ("3d_wide_ctas", cfg.Workload("wide", 96, 64, 48, 8, 41, 18, 10, 2.25, 0, 12, (1, 96, 1, 64, 9, 38), 9, 120,
                                  structure="spheres", extra=dict(nspheres=8, rmin=2, rmax=6, emin=1.5, emax=6.0)),
     (0.3 + 0j, 0.1 + 0j, 0j), None, {}, 0),
]
CALLS = [(1, 1), (2, 37), (39, 64), (103, 5)]


def material(w, op, kind):
    if kind == "complex":
        r = np.random.default_rng(5)
        shp = (op.hf - op.hi + 3, op.ny + 2, op.nx + 2)
        return 1.0 / r.uniform(1, 5, shp) + 1j * r.uniform(-0.05, 0.05, shp)
    if w.structure == "spheres":
        return cfg.spheres_material(w, seed=3)
    return cfg.slit_material(w)


def make(iris, oracle, tmp_path, case, precision):
    name, w, ak, kind, kw, faces = case
    op = oracle.setparam(cfg.write_input(str(tmp_path / f"{name}.dat"), w, no_downloads=2, **kw))
    p = engine_params_from_oracle(iris, op, precision=precision, ak=ak)
    p.dft_faces = faces
    return w, op, p, material(w, op, kind)


def engines(iris, p, op, eps, block):
    out = []
    for st in (iris.STENCIL_SPLIT, iris.STENCIL_PERSISTENT):
        e = iris.Engine(p, op.fw, stencil=st, dft_block=block)
        e.set_material(eps)
        out.append(e)
    return out


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_persistent_equals_split(iris, oracle, tmp_path, case, precision):
    w, op, p, eps = make(iris, oracle, tmp_path, case, precision)
    split, pers = engines(iris, p, op, eps, block=16)
    for it0, n in CALLS:
        split.step(it0, n)
        pers.step(it0, n)
    for which in (iris.E, iris.H):
        assert np.array_equal(split.get_field(which), pers.get_field(which)), which
    for which in (0, 1):
        for slab in (0, 1):
            assert np.array_equal(split.get_pml(which, slab), pers.get_pml(which, slab)), (which, slab)
    assert split.info()["dft_buffered"] == pers.info()["dft_buffered"]
    assert np.array_equal(split.flux(0), pers.flux(0))
    for j in (1, 2, 3):
        assert np.array_equal(split.get_fdata(0, j), pers.get_fdata(0, j)), j


def test_persistent_selection_and_launches(iris, oracle, tmp_path):
    """Small grids step with the persistent kernel by default: one launch per
    span (spans end where the DFT block fills), none of the per-pass kernels."""
    w, op, p, eps = make(iris, oracle, tmp_path, CASES[1], 0)
    e = iris.Engine(p, op.fw, dft_block=32)
    e.set_material(eps)
    e.timing_start()
    e.step(1, 100)
    _, ms, n = e.timing_read()
    assert n["persistent"] == 4 and n["update_e"] == n["update_h"] == n["tfsf"] == n["dft_gather"] == 0
    assert n["dft_block"] == 3 and e.info()["dft_buffered"] == 100 - 96


def test_persistent_workload1_against_oracle(iris, oracle, tmp_path):
    """The 4x4x512 FP64 slab (z-plane DFT at 200 frequencies) through the
    persistent kernel against the oracle at 1e-12 over 1500 steps."""
    w = cfg.workload(1)
    op = oracle.setparam(cfg.write_input(str(tmp_path / "w1.dat"), w, no_downloads=4))
    op.texit = 1500
    o = oracle.Oracle(op, threads=THREADS)
    its = output_steps(op)
    Jo, ito = o.run(1, op.texit, max_out=len(its) + 1)
    p = engine_params_from_oracle(iris, op, precision=0)
    p.dft_faces = iris.DFT_Z
    e = iris.Engine(p, op.fw, stencil=iris.STENCIL_PERSISTENT)
    Jg = run_engine_blocks(e, op, its)
    assert rel_err(Jg[:, 4:], Jo[:, 4:]) <= 1e-12
    assert rel_err(Jg[-1, 4:], Jo[-1, 4:]) <= 1e-12


def test_barrier_gives_up_and_engine_stays_usable(iris, oracle, tmp_path):
    w, op, p, eps = make(iris, oracle, tmp_path, CASES[2], 0)
    twin, e = engines(iris, p, op, eps, block=16)
    e.step(1, 20)
    twin.step(1, 20)
    # the wait gives up after about a millisecond (the persistent limit / 2^10)
    assert e.L.iris_apply(e.h, iris.OP_BARRIER_CHECK, 10) == -7
    assert b"grid barrier" in e.L.iris_last_error()
    e.step(21, 40)
    twin.step(21, 40)
    assert np.array_equal(e.get_field(iris.E), twin.get_field(iris.E))
    assert np.array_equal(e.flux(0), twin.flux(0))
