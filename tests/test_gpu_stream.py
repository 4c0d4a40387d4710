"""The streamed FP32 split passes (IRIS_STENCIL_STREAM: planes staged in
shared memory by bulk copies, z-marching tiles) against the plain split FP32
passes and the FP64 oracle.

Same per-cell expressions on the same operands as the split passes, so the
results equal the split run's to the last bit; 1e-4 against the oracle.  The
cases cover partial x and y tiles, z chunks that do not divide nz, 1-D and
2-D grids, both polarisations, Bloch phases, and a complex material (which
steps with the split passes).
"""
import importlib
import os

import numpy as np
import pytest

from helpers import interior, output_steps, rel_err, run_engine_blocks
from test_gpu_fused import CASES, make_case, material, run

pytestmark = pytest.mark.gpu
THREADS = max(1, min(16, os.cpu_count() or 1))
cfg = importlib.import_module("irisfdtd-academic_gb300.configs")

STREAM = 3
MORE = [
    ("3d_many_chunks", (70, 19, 150, 9, 140, 60, 30, 4.0, 14, (1, 70, 1, 19, 12, 130)), 2,
     (0.9 + 0j, 0j, 0j), "spheres", 220),
]


@pytest.mark.parametrize("case", CASES + MORE, ids=[c[0] for c in CASES + MORE])
def test_stream_against_split_and_oracle(iris, oracle, tmp_path, case):
    name, spec, i_pol, ak, kind, steps = case
    w, op = make_case(oracle, tmp_path, spec, i_pol)
    op.texit = steps
    eps = material(w, op, kind, np.random.default_rng(5))
    es, Js = run(iris, op, 1, ak, eps)
    et, Jt = run(iris, op, STREAM, ak, eps)
    for which in (iris.E, iris.H):
        fs, ft = interior(es.get_field(which), op), interior(et.get_field(which), op)
        assert np.array_equal(ft, fs), (which, rel_err(ft, fs))
    assert np.array_equal(Jt, Js)
    for j in (1, 2, 3):
        assert np.array_equal(et.get_fdata(0, j), es.get_fdata(0, j)), j
    o = oracle.Oracle(op, ak=ak, threads=THREADS)
    if eps is not None:
        o.set_eps_inv(eps)
    Jo, _ = o.run(1, op.texit, max_out=len(output_steps(op)))
    assert rel_err(Jt, Jo) <= 1e-4
    assert rel_err(interior(et.get_field(iris.E), op), interior(o.get_field(o.E_CUR), op)) <= 1e-4


def test_stream_ghosts_match_split(iris, oracle, tmp_path):
    """The Bloch ghost planes the streamed passes write equal the split ones."""
    w, op = make_case(oracle, tmp_path, (37, 21, 64, 8, 57, 24, 14, 2.25, 12, (1, 37, 1, 21, 9, 54)), 2)
    ak = (0.4 + 0j, -0.2 + 0j, 0j)
    eps = cfg.spheres_material(w, seed=3)
    es, _ = run(iris, op, 1, ak, eps)
    et, _ = run(iris, op, STREAM, ak, eps)
    for which in (iris.E, iris.H):
        fs, ft = es.get_field(which), et.get_field(which)
        for sl in (np.s_[:, :, 0], np.s_[:, 0, :], np.s_[0, :, :], np.s_[:, :, -1], np.s_[:, -1, :], np.s_[-1, :, :]):
            if which == iris.H and sl in (np.s_[:, :, -1], np.s_[:, -1, :], np.s_[-1, :, :]):
                continue  # H ghosts at n+1 are never maintained
            assert np.array_equal(ft[sl], fs[sl])


def test_stream_selection_and_fp64_rejected(iris, oracle, tmp_path):
    w, op = make_case(oracle, tmp_path, (16, 8, 40, 6, 35, 15, 10, 4.0, 10, (1, 16, 1, 8, 8, 32)), 2)
    eng = iris.Engine(engine_params_from_oracle_fp(iris, op, 1), op.fw, stencil=STREAM)
    eng.timing_start()
    eng.step(1, 5)
    _, ms, n = eng.timing_read()
    assert n["update_e"] == 5 and n["update_h"] == 5 and n["fused_eh"] == 0
    with pytest.raises(iris.IrisError) as e:
        iris.Engine(engine_params_from_oracle_fp(iris, op, 0), op.fw, stencil=STREAM)
    assert e.value.code == -1


def engine_params_from_oracle_fp(iris, op, precision):
    from helpers import engine_params_from_oracle
    return engine_params_from_oracle(iris, op, precision=precision)



IRIS_EINVAL, IRIS_ETIMEOUT = -1, -7


@pytest.mark.parametrize("stencil", [STREAM, 2])
def test_bounded_wait_gives_up_and_engine_stays_usable(iris, oracle, tmp_path, stencil):
    """A device wait on an mbarrier that nothing completes (IRIS_OP_WAIT_CHECK)
    gives up after its limit and is reported once as IRIS_ETIMEOUT; the engine
    then steps exactly like a twin that never waited."""
    w, op = make_case(oracle, tmp_path, (24, 12, 48, 6, 43, 18, 10, 4.0, 10, (1, 24, 1, 12, 8, 40)), 2)
    op.texit = 40
    eps = cfg.spheres_material(w, seed=3)

    def engine():
        e = iris.Engine(engine_params_from_oracle_fp(iris, op, 1), op.fw, stencil=stencil)
        e.set_material(eps)
        return e

    eng, twin = engine(), engine()
    assert eng.L.iris_apply(eng.h, iris.OP_WAIT_CHECK, 10) == IRIS_ETIMEOUT  # about a millisecond
    assert "wait check" in eng.L.iris_last_error().decode()
    eng.sync()  # reported once: the error word is clear again
    assert eng.L.iris_apply(eng.h, iris.OP_WAIT_CHECK, 31) == IRIS_EINVAL
    J = run_engine_blocks(eng, op, output_steps(op))
    Jt = run_engine_blocks(twin, op, output_steps(op))
    assert np.array_equal(J, Jt)
    for which in (iris.E, iris.H):
        assert np.array_equal(eng.get_field(which), twin.get_field(which))
