"""GPU engine vs the CPU oracle (FP64 parity mode: 1e-12 norm-wise relative).

Per-operator tests put the same random state (fields, ghosts, UPML
auxiliaries, material) into both and apply one operator group; full-run
tests step both from zero through the reference driver's output schedule.
"""
import importlib
import os

import numpy as np
import pytest

from conftest import golden
from helpers import engine_params_from_oracle, interior, output_steps, rel_err, run_engine_blocks

pytestmark = pytest.mark.gpu

TOL = 1e-12
cfg = importlib.import_module("irisfdtd-academic_gb300.configs")
THREADS = max(1, min(16, os.cpu_count() or 1))


def small_case(oracle, tmp_path, nx=5, ny=3, nz=40, i_pol=2, plane_wave=1, cosine=0, tfsf_zi=10, hi=15, dh=10,
               eps=4.0, box=None, nof=7, name="in.dat"):
    w = cfg.Workload("small", nx, ny, nz, 6, nz - 5, hi, dh, eps, 0, tfsf_zi,
                     box or (1, nx, 1, ny, 8, nz - 8), nof, 50)
    path = cfg.write_input(str(tmp_path / name), w, i_pol=i_pol, plane_wave=plane_wave, cosine=cosine)
    return oracle.setparam(path)


def rfield(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def make_pair(iris, oracle, op, ak=(0j, 0j, 0j), eps=None):
    o = oracle.Oracle(op, ak=ak, threads=THREADS)
    eng = iris.Engine(engine_params_from_oracle(iris, op, ak=ak), op.fw)
    if eps is not None:
        o.set_eps_inv(eps)
        eng.set_material(eps)
    return o, eng


def max_ghost_mask(p):
    m = np.zeros((p.nz + 2, p.ny + 2, p.nx + 2), bool)
    m[1:-1, 1:-1, 1:-1] = True
    m[1:-1, 1:-1, -1] = True
    m[1:-1, -1, 1:-1] = True
    m[-1, 1:-1, 1:-1] = True
    return m


def min_ghost_mask(p, with_interior=True):
    m = np.zeros((p.nz + 2, p.ny + 2, p.nx + 2), bool)
    if with_interior:
        m[1:-1, 1:-1, 1:-1] = True
    m[1:-1, 1:-1, 0] = True
    m[1:-1, 0, 1:-1] = True
    m[0, 1:-1, 1:-1] = True
    return m


AKS = [(0j, 0j, 0j), (0.7 + 0j, -0.3 + 0j, 0.2 + 0.05j)]


@pytest.mark.parametrize("ak", AKS)
@pytest.mark.parametrize("complex_eps", [False, True])
def test_op_e(iris, oracle, tmp_path, ak, complex_eps):
    op = small_case(oracle, tmp_path)
    rng = np.random.default_rng(1)
    eps = 1.0 / rng.uniform(1, 6, (op.hf - op.hi + 3, op.ny + 2, op.nx + 2)) + (
        1j * rng.uniform(-0.1, 0.1, (op.hf - op.hi + 3, op.ny + 2, op.nx + 2)) if complex_eps else 0)
    o, eng = make_pair(iris, oracle, op, ak, eps)
    shp = o.field_shape
    E0, H0 = rfield(rng, shp), rfield(rng, shp)
    D = [rfield(rng, o.pml_shape(s)) for s in (0, 1)]
    o.set_field(o.E_PREV, E0)
    o.set_field(o.E_CUR, E0)
    o.set_field(o.H_PREV, H0)
    for s in (0, 1):
        o.set_pml(0, 0, s, D[s])
        eng.set_pml(0, s, D[s])
    eng.set_field(iris.E, E0)
    eng.set_field(iris.H, H0)
    o.op("e_fdtd")
    o.op("upml_e")
    o.op("bloch_max")
    eng.e_fdtd()
    m = max_ghost_mask(op)
    Eo, Eg = o.get_field(o.E_CUR), eng.get_field(iris.E)
    assert rel_err(Eg[m], Eo[m]) <= TOL
    for s in (0, 1):
        assert rel_err(eng.get_pml(0, s), o.get_pml(0, 1, s)) <= TOL


@pytest.mark.parametrize("ak", AKS)
def test_op_h(iris, oracle, tmp_path, ak):
    op = small_case(oracle, tmp_path, nx=6, ny=4, nz=36)
    rng = np.random.default_rng(2)
    o, eng = make_pair(iris, oracle, op, ak)
    shp = o.field_shape
    E1, H0 = rfield(rng, shp), rfield(rng, shp)
    B = [rfield(rng, o.pml_shape(s)) for s in (0, 1)]
    o.set_field(o.E_CUR, E1)
    o.set_field(o.H_PREV, H0)
    o.set_field(o.H_CUR, H0)
    for s in (0, 1):
        o.set_pml(1, 0, s, B[s])
        eng.set_pml(1, s, B[s])
    eng.set_field(iris.E, E1)
    eng.set_field(iris.H, H0)
    o.op("h_fdtd")
    o.op("upml_h")
    o.op("bloch_min")
    eng.h_fdtd()
    m = min_ghost_mask(op)
    assert rel_err(eng.get_field(iris.H)[m], o.get_field(o.H_CUR)[m]) <= TOL
    mg = min_ghost_mask(op, with_interior=False)
    assert rel_err(eng.get_field(iris.E)[mg], o.get_field(o.E_CUR)[mg]) <= TOL
    for s in (0, 1):
        assert rel_err(eng.get_pml(1, s), o.get_pml(1, 1, s)) <= TOL


TFSF_CASES = [
    # (nx, ny, i_pol, plane_wave, cosine, tfsf_zi, hi)   3D / 2D variants, both polarisations,
    (5, 3, 2, 1, 0, 10, 15),    # update_3DArray, E//x
    (5, 3, 1, 1, 0, 10, 15),    # update_3DArray, E//y
    (1, 1, 2, 1, 0, 10, 15),    # update_2DArray
    (7, 1, 2, 1, 1, 10, 15),    # update_2DArray, real-valued source
    (1, 4, 1, 1, 0, 10, 15),    # 2D grid with E//y takes update_3DArray
    (5, 3, 2, 1, 0, 30, 15),    # source inside the substrate side: sign_kz = -1
    (5, 3, 2, 0, 0, 10, 15),    # CW source with ramps
    (4, 1, 1, 0, 1, 12, 15),    # CW, E//y, real-valued
]


@pytest.mark.parametrize("case", TFSF_CASES)
def test_op_tfsf(iris, oracle, tmp_path, case):
    nx, ny, i_pol, pw, cos_, zi, hi = case
    op = small_case(oracle, tmp_path, nx=nx, ny=ny, i_pol=i_pol, plane_wave=pw, cosine=cos_, tfsf_zi=zi, hi=hi)
    rng = np.random.default_rng(3)
    o, eng = make_pair(iris, oracle, op)
    for it in (1, 37, 3000, 9000):
        E0, H0 = rfield(rng, o.field_shape), rfield(rng, o.field_shape)
        o.set_field(o.E_CUR, E0)
        o.set_field(o.H_CUR, H0)
        eng.set_field(iris.E, E0)
        eng.set_field(iris.H, H0)
        o.op("tfsf", it)
        eng.tfsf(it)
        Eo, Ho = o.get_field(o.E_CUR), o.get_field(o.H_CUR)
        Eg, Hg = eng.get_field(iris.E), eng.get_field(iris.H)
        # the correction itself (tiny against the random state) must match too
        assert rel_err(Eg - E0, Eo - E0) <= 1e-11, it
        assert rel_err(Hg - H0, Ho - H0) <= 1e-11, it
        assert rel_err(Eg, Eo) <= TOL and rel_err(Hg, Ho) <= TOL


@pytest.mark.parametrize("dims", [(5, 3), (1, 1), (6, 1), (1, 4)])
def test_op_dft(iris, oracle, tmp_path, dims):
    nx, ny = dims
    op = small_case(oracle, tmp_path, nx=nx, ny=ny, nof=9, box=(1, nx, 1, ny, 7, 31))
    rng = np.random.default_rng(4)
    o, eng = make_pair(iris, oracle, op)
    for t in (1, 2, 517, 9999):
        E0, H0 = rfield(rng, o.field_shape), rfield(rng, o.field_shape)
        o.set_field(o.E_CUR, E0)
        o.set_field(o.H_CUR, H0)
        eng.set_field(iris.E, E0)
        eng.set_field(iris.H, H0)
        o.op("dft", t)
        eng.scattering_fourier(t)
    for j in (1, 2, 3):
        fg = eng.get_fdata(0, j)
        # face pairs scattering_fourier accumulates (code/dataprocess.f90:138-205)
        if nx != 1 and ny != 1:
            on = True
        else:
            on = {1: ny == 1 and nx != 1, 2: nx == 1 and ny != 1, 3: True}[j]
        if not on:
            assert fg.shape[1] == 0
            continue
        fo = o.fdata(0, j)
        assert fg.shape == fo.shape
        assert rel_err(fg, fo) <= TOL, j
    assert rel_err(eng.flux(0), o.flux(0)) <= 1e-11


def test_two_boxes(iris, oracle, tmp_path):
    op = small_case(oracle, tmp_path, nx=6, ny=4, nz=48, box=(1, 6, 1, 4, 9, 39), nof=5)
    op.box2 = (2, 5, 1, 3, 12, 30)
    o, eng = make_pair(iris, oracle, op)
    o.L.orc_set_threads(o.h, 1)
    its = [20, 40, 60]
    Jo, ito = o.run(1, 60, max_out=0)
    blocks_g = run_engine_blocks(eng, op, [60])
    Jg1 = eng.flux(1)
    assert rel_err(blocks_g[0], o.flux(0)) <= TOL
    assert rel_err(Jg1, o.flux(1)) <= TOL
    for j in (1, 2, 3):
        assert rel_err(eng.get_fdata(1, j), o.fdata(1, j)) <= TOL


def assert_spectra(Jg, Jo, tol=TOL):
    """Flux blocks [block, face, iw]: norm-wise relative error over the whole
    run (early blocks carry only the pulse's leading tail, orders of magnitude
    below the final spectrum), the final block on its own, and its T/R where
    the total flux is not negligible."""
    assert Jg.shape == Jo.shape
    assert rel_err(Jg, Jo) <= tol
    assert rel_err(Jg[-1], Jo[-1]) <= tol
    tot = Jo[-1, 4] + Jo[-1, 5]
    m = np.abs(tot) > 1e-3 * np.max(np.abs(tot))
    if m.any():
        Rg, Ro = Jg[-1, 4][m] / (Jg[-1, 4] + Jg[-1, 5])[m], Jo[-1, 4][m] / tot[m]
        assert np.max(np.abs(Rg - Ro)) <= tol


def field_err(a, b, op):
    """Interior field error relative to the incident amplitude Epump*Q (after a
    long run the pulse has left and the fields sit at the roundoff floor, where
    a norm relative to the fields themselves says nothing)."""
    amp = op.epump * op.Q
    ia, ib = interior(a, op), interior(b, op)
    return float(np.max(np.abs(ia - ib)) / max(amp, np.max(np.abs(ib))))


def full_run(iris, oracle, op, nsteps=None, ak=(0j, 0j, 0j), eps=None, precision=0):
    if nsteps is not None:
        op.texit = nsteps
    o = oracle.Oracle(op, ak=ak, threads=THREADS)
    eng = iris.Engine(engine_params_from_oracle(iris, op, precision=precision, ak=ak), op.fw)
    if eps is not None:
        o.set_eps_inv(eps)
        eng.set_material(eps)
    its = output_steps(op)
    Jo, ito = o.run(1, op.texit, max_out=len(its) + 1)
    assert ito == its
    Jg = run_engine_blocks(eng, op, its)
    return o, eng, Jo, Jg


def test_example1_full_length(iris, oracle):
    op = oracle.setparam(golden("example_1.inputFDTD.dat"))
    o, eng, Jo, Jg = full_run(iris, oracle, op)
    assert Jg.shape == (51, 6, 500)
    assert_spectra(Jg, Jo)
    Eg, Eo = eng.get_field(iris.E), o.get_field(o.E_CUR)
    assert field_err(Eg, Eo, op) <= TOL
    Hg, Ho = eng.get_field(iris.H), o.get_field(o.H_CUR)
    assert field_err(Hg, Ho, op) <= TOL


def test_example2_slit(iris, oracle):
    op = oracle.setparam(golden("example_2.inputFDTD.dat"))
    op.texit = 6000
    o, eng, Jo, Jg = full_run(iris, oracle, op)
    assert_spectra(Jg, Jo)
    assert field_err(eng.get_field(iris.E), o.get_field(o.E_CUR), op) <= TOL


def test_workload1_slab(iris, oracle, tmp_path):
    w = cfg.workload(1)
    op = oracle.setparam(cfg.write_input(str(tmp_path / "w1.dat"), w, no_downloads=4))
    o, eng, Jo, Jg = full_run(iris, oracle, op, nsteps=1500)
    assert_spectra(Jg, Jo)


def test_workload2_slit_reduced(iris, oracle, tmp_path):
    w = cfg.workload(2, nof=12)
    op = oracle.setparam(cfg.write_input(str(tmp_path / "w2.dat"), w, no_downloads=2))
    o, eng, Jo, Jg = full_run(iris, oracle, op, nsteps=400, eps=cfg.slit_material(w))
    assert_spectra(Jg, Jo)
    assert field_err(eng.get_field(iris.H), o.get_field(o.H_CUR), op) <= TOL


def test_bloch_cell_spheres_reduced(iris, oracle, tmp_path):
    """A small 3D Bloch cell with kx != 0, seeded spheres and complex fields."""
    w = cfg.Workload("sph", 24, 20, 96, 8, 89, 30, 36, 1.0, 0, 14, (1, 24, 1, 20, 10, 86), 10, 300,
                     akx=0.3 * np.pi * 24, structure="spheres",
                     extra=dict(nspheres=12, rmin=3, rmax=7, emin=1.5, emax=6.0))
    op = oracle.setparam(cfg.write_input(str(tmp_path / "w3.dat"), w, no_downloads=3))
    ak = (complex(w.akx), 0j, 0j)
    o, eng, Jo, Jg = full_run(iris, oracle, op, ak=ak, eps=cfg.spheres_material(w, seed=7))
    assert_spectra(Jg, Jo)
    assert field_err(eng.get_field(iris.E), o.get_field(o.E_CUR), op) <= TOL


def test_fp32_mode_tr_error(iris, oracle):
    """Precision form: FP32 fields, FP64 incident field and DFT accumulation;
    T/R against the FP64 oracle within 1e-4 (example_1, full length)."""
    op = oracle.setparam(golden("example_1.inputFDTD.dat"))
    o, eng, Jo, Jg = full_run(iris, oracle, op, precision=1)
    Ro, To = oracle.tr_normalise(Jo[-1, 4], Jo[-1, 5])
    Rg, Tg = iris.tr_normalise(Jg[-1, 4], Jg[-1, 5])
    err = max(np.max(np.abs(Rg - Ro)), np.max(np.abs(Tg - To)))
    assert err <= 1e-4, err


@pytest.mark.parametrize("precision,shape", [(0, (8, 6, 48)), (1, (70, 40, 48))])
def test_step_is_deterministic(iris, oracle, tmp_path, precision, shape):
    """Two runs agree bit for bit: FP64 on a small grid (the persistent
    kernel, the default there), and FP32 with the fused pass, the tensor-core
    DFT commit and flux read: no atomics and no order-dependent reduction
    anywhere on the path."""
    nx, ny, nz = shape
    op = small_case(oracle, tmp_path, nx=nx, ny=ny, nz=nz, nof=6)
    stencil = iris.STENCIL_FUSED if precision == iris.FP32 else iris.STENCIL_DEFAULT
    res = []
    for _ in range(2):
        eng = iris.Engine(engine_params_from_oracle(iris, op, precision=precision), op.fw, dft_block=32,
                          stencil=stencil)
        eng.step(1, 120)
        res.append((eng.get_field(iris.E), eng.get_field(iris.H), eng.flux(0), eng.get_fdata(0, 1)))
        eng.close()
    for a, b in zip(*res):
        assert np.array_equal(a, b)
