"""The fused FP32 E+H pass (IRIS_STENCIL_FUSED) against the split FP32 passes
and against the FP64 oracle.

The fused pass computes every cell with the same per-cell arithmetic as the
split passes but reorders the work (one z-marching pass over double buffers,
overlapping tiles whose edge cells are recomputed, Bloch ghosts as index
images; TF/SF and the DFT sample run after it as after the split passes).
Fields, fluxes and the reference-order DFT accumulators of every face pair
equal those of the split FP32 run to the last bit; against the FP64 oracle
the tolerance is 1e-4.
"""
import importlib
import os

import numpy as np
import pytest

from helpers import engine_params_from_oracle, interior, output_steps, rel_err, run_engine_blocks

pytestmark = pytest.mark.gpu
cfg = importlib.import_module("irisfdtd-academic_gb300.configs")
THREADS = max(1, min(16, os.cpu_count() or 1))

# name, (nx, ny, nz, pmlzi, pmlzf, hi, dh, eps_bbox, tfsf_zi, box), i_pol, ak, material, steps
CASES = [
    ("3d_partial_tiles_pol2", (37, 21, 64, 8, 57, 24, 14, 2.25, 12, (1, 37, 1, 21, 9, 54)), 2,
     (0.4 + 0j, -0.2 + 0j, 0j), "spheres", 160),
    ("3d_pol1_complex_eps", (33, 9, 48, 6, 43, 18, 10, 4.0, 10, (2, 30, 1, 9, 7, 40)), 1,
     (0j, 0.3 + 0j, 0j), "complex", 140),
    ("2d_xz_slit", (40, 1, 80, 10, 71, 30, 12, 9.0, 16, (1, 40, 1, 1, 12, 66)), 2, (0j, 0j, 0j), "slit", 200),
    ("1d_slab", (1, 1, 120, 12, 109, 50, 20, 9.0, 20, (1, 1, 1, 1, 15, 100)), 2, (0j, 0j, 0j), "slab", 300),
    # several column tiles and z chunks, long enough for the pulse to work the UPML slabs
    ("3d_tiles_upml_long", (70, 40, 120, 10, 111, 50, 10, 4.0, 16, (1, 70, 1, 40, 13, 104)), 2,
     (0.25 + 0j, 0j, 0j), "spheres", 420),
]


def make_case(oracle, tmp_path, spec, i_pol):
    nx, ny, nz, pmlzi, pmlzf, hi, dh, eps, zi, box = spec
    w = cfg.Workload("fused", nx, ny, nz, pmlzi, pmlzf, hi, dh, eps, 8 if nx >= 16 else 0, zi, box, 11, 50,
                     structure="spheres", extra=dict(nspheres=6, rmin=2, rmax=5, emin=1.5, emax=6.0))
    op = oracle.setparam(cfg.write_input(str(tmp_path / "in.dat"), w, i_pol=i_pol, no_downloads=3))
    return w, op


def material(w, op, kind, rng):
    if kind == "spheres":
        return cfg.spheres_material(w, seed=3)
    if kind == "complex":
        shp = (op.hf - op.hi + 3, op.ny + 2, op.nx + 2)
        return 1.0 / rng.uniform(1, 5, shp) + 1j * rng.uniform(-0.05, 0.05, shp)
    if kind == "slit":
        return cfg.slit_material(w)
    return None


def run(iris, op, stencil, ak, eps, precision=1):
    eng = iris.Engine(engine_params_from_oracle(iris, op, precision=precision, ak=ak), op.fw, stencil=stencil)
    if eps is not None:
        eng.set_material(eps)
    J = run_engine_blocks(eng, op, output_steps(op))
    return eng, J


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_fused_against_split_and_oracle(iris, oracle, tmp_path, case):
    name, spec, i_pol, ak, kind, steps = case
    w, op = make_case(oracle, tmp_path, spec, i_pol)
    op.texit = steps
    eps = material(w, op, kind, np.random.default_rng(5))
    es, Js = run(iris, op, 1, ak, eps)
    ef, Jf = run(iris, op, 2, ak, eps)
    assert ef.info()["dft_points"] == es.info()["dft_points"]
    # the fused pass evaluates every cell with the split passes' expressions on
    # the same operands: the results are the same to the last bit (a norm-wise
    # tolerance would hide errors confined to the small fields in the UPML)
    for which in (iris.E, iris.H):
        fs, ff = interior(es.get_field(which), op), interior(ef.get_field(which), op)
        assert np.array_equal(ff, fs), (which, rel_err(ff, fs))
    assert np.array_equal(Jf, Js)
    for j in (1, 2, 3):
        assert np.array_equal(ef.get_fdata(0, j), es.get_fdata(0, j)), j
    # against the FP64 oracle
    o = oracle.Oracle(op, ak=ak, threads=THREADS)
    if eps is not None:
        o.set_eps_inv(eps)
    Jo, _ = o.run(1, op.texit, max_out=len(output_steps(op)))
    assert rel_err(Jf, Jo) <= 1e-4
    assert rel_err(interior(ef.get_field(iris.E), op), interior(o.get_field(o.E_CUR), op)) <= 1e-4


def test_fused_two_boxes(iris, oracle, tmp_path):
    w, op = make_case(oracle, tmp_path, (20, 12, 56, 7, 50, 22, 12, 2.25, 10, (1, 20, 1, 12, 8, 48)), 2)
    op.box2 = (3, 17, 2, 10, 12, 40)
    op.texit = 120
    es, Js = run(iris, op, 1, (0j, 0j, 0j), None)
    ef, Jf = run(iris, op, 2, (0j, 0j, 0j), None)
    assert np.array_equal(ef.flux(1), es.flux(1))
    for j in (1, 2, 3):
        assert np.array_equal(ef.get_fdata(1, j), es.get_fdata(1, j))


@pytest.mark.parametrize("pmlzf", [8, 9])
def test_fused_without_interior_range(iris, oracle, tmp_path, pmlzf):
    """pmlzf <= pmlzi + 2 leaves no planes for the launch without UPML code:
    every plane goes through the slab launch, still bitwise the split passes."""
    w, op = make_case(oracle, tmp_path, (16, 8, 20, 6, pmlzf, 7, 1, 4.0, 7, (1, 16, 1, 8, 3, 17)), 2)
    op.texit = 60
    es, Js = run(iris, op, 1, (0.2 + 0j, 0j, 0j), None)
    ef, Jf = run(iris, op, 2, (0.2 + 0j, 0j, 0j), None)
    for which in (iris.E, iris.H):
        assert np.array_equal(interior(ef.get_field(which), op), interior(es.get_field(which), op)), which
    assert np.array_equal(Jf, Js)


def test_fused_without_structure_layer(iris, oracle, tmp_path):
    """A deck whose structure layer is empty (hf < hi: no eps table at all)."""
    w, op = make_case(oracle, tmp_path, (24, 10, 48, 6, 43, 20, 0, 4.0, 10, (1, 24, 1, 10, 8, 40)), 2)
    op.texit = 80
    es, Js = run(iris, op, 1, (0.3 + 0j, 0j, 0j), None)
    ef, Jf = run(iris, op, 2, (0.3 + 0j, 0j, 0j), None)
    for which in (iris.E, iris.H):
        assert np.array_equal(interior(ef.get_field(which), op), interior(es.get_field(which), op)), which
    assert np.array_equal(Jf, Js)


def test_fused_rejected_in_fp64(iris, oracle, tmp_path):
    w, op = make_case(oracle, tmp_path, (8, 6, 40, 6, 35, 15, 10, 4.0, 10, (1, 8, 1, 6, 8, 32)), 2)
    with pytest.raises(iris.IrisError) as e:
        iris.Engine(engine_params_from_oracle(iris, op, precision=0), op.fw, stencil=2)
    assert e.value.code == -1


def test_stencil_selection(iris, oracle, tmp_path):
    """The per-kernel timers show which pass ran.  By default the persistent
    kernel up to PERSISTENT_MAX_CELLS cells in FP64 and
    PERSISTENT_MAX_CELLS_FP32 in FP32 (one launch for the five steps);
    above them FP64 steps with the split passes and FP32 with the fused pass
    (one timer a step over its two concurrent launches: the planes outside
    the UPML slabs and the slabs), or with the split passes on a grid whose
    x-y plane would leave most of the fused tiles' threads idle (4 cells in
    y); split, fused or persistent on request."""
    small = make_case(oracle, tmp_path, (16, 8, 40, 6, 35, 15, 10, 4.0, 10, (1, 16, 1, 8, 8, 32)), 2)[1]
    mid = make_case(oracle, tmp_path, (48, 40, 40, 6, 35, 15, 10, 4.0, 10, (1, 48, 1, 40, 8, 32)), 2)[1]
    big64 = make_case(oracle, tmp_path, (128, 96, 88, 6, 83, 30, 10, 4.0, 10, (1, 128, 1, 96, 8, 80)), 2)[1]
    big32 = make_case(oracle, tmp_path, (256, 256, 136, 6, 131, 60, 10, 4.0, 10, (1, 256, 1, 256, 8, 128)), 2)[1]
    thin = make_case(oracle, tmp_path, (2048, 4, 1100, 6, 1095, 500, 10, 4.0, 10, (1, 2048, 1, 4, 8, 1090)), 2)[1]
    assert 48 * 40 * 40 <= iris.PERSISTENT_MAX_CELLS < 128 * 96 * 88
    assert 256 * 256 * 136 > iris.PERSISTENT_MAX_CELLS_FP32 and 2048 * 4 * 1100 > iris.PERSISTENT_MAX_CELLS_FP32
    for op, prec, stencil, kind in ((big32, 1, 0, "fused"), (thin, 1, 0, "split"), (mid, 1, 0, "persistent"),
                                    (small, 1, 0, "persistent"), (mid, 0, 0, "persistent"), (big64, 0, 0, "split"),
                                    (small, 1, 1, "split"), (small, 1, 2, "fused"), (small, 1, 4, "persistent"),
                                    (big64, 0, 4, "persistent")):
        q = engine_params_from_oracle(iris, op, precision=prec)
        q.dft_faces = iris.DFT_Z  # the large grids' x and y faces would hold tens of millions of points
        eng = iris.Engine(q, op.fw, stencil=stencil)
        eng.timing_start()
        eng.step(1, 5)
        _, ms, n = eng.timing_read()
        if kind == "fused":
            assert n["fused_eh"] == 5 and n["update_e"] == 0 and n["update_h"] == 0 and n["persistent"] == 0
        elif kind == "split":
            assert n["fused_eh"] == 0 and n["update_e"] == 5 and n["update_h"] == 5 and n["persistent"] == 0
        else:
            assert n["persistent"] == 1 and n["fused_eh"] == 0 and n["update_e"] == 0 and n["update_h"] == 0
        eng.close()
