"""The batched form (iris_batch_*): every cell of an uneven batch against the
same cell stepped on its own engine and against the FP64 oracle.

The batch runs the same per-cell arithmetic as a single engine (the same
device functions, one launch per operator over all cells), so the cells'
fields agree with their single-engine runs to the last bit in both
precisions, and FP64 spectra with the oracle within 1e-12; FP32 spectra
within 1e-5 (different DFT block boundaries).  Work list 7 is the fused E+H
pass (FP32 only; its fields alternate between two buffer sets).
"""
import importlib
import os

import numpy as np
import pytest

from helpers import engine_params_from_oracle, interior, output_steps, rel_err, run_engine_blocks

pytestmark = pytest.mark.gpu
cfg = importlib.import_module("irisfdtd-academic_gb300.configs")
THREADS = max(1, min(16, os.cpu_count() or 1))

# nx, ny, nz, pmlzi, pmlzf, hi, dh, tfsf_zi, box, akx, structure
CELLS = [
    (12, 7, 60, 8, 53, 24, 10, 14, (1, 12, 1, 7, 10, 50), 0.3, "pattern"),
    (33, 9, 48, 6, 43, 18, 8, 10, (1, 33, 1, 9, 8, 40), 0.0, "pattern"),
    (5, 17, 72, 8, 65, 30, 12, 14, (1, 5, 1, 17, 11, 62), -0.7, "pattern"),
    (40, 1, 64, 8, 57, 26, 10, 14, (1, 40, 1, 1, 10, 54), 0.0, "slab"),
    (1, 1, 90, 10, 81, 40, 15, 16, (1, 1, 1, 1, 12, 78), 0.0, "slab"),
]
STEPS = 150


def make_cells(oracle, tmp_path):
    out = []
    for i, (nx, ny, nz, pi, pf, hi, dh, zi, box, akx, kind) in enumerate(CELLS):
        w = cfg.Workload(f"c{i}", nx, ny, nz, pi, pf, hi, dh, 4.0 if kind == "slab" else 1.0, 0, zi, box, 9, STEPS,
                         structure=kind, extra=dict(seed=100 + i, fill=0.5))
        op = oracle.setparam(cfg.write_input(str(tmp_path / f"c{i}.dat"), w, no_downloads=3))
        eps = cfg.binary_pattern_material(w) if kind == "pattern" else cfg.slit_material(w)
        out.append((w, op, (complex(akx), 0j, 0j), eps))
    return out


def batch_and_singles(iris, cells, precision, tune=False, tile=None):
    params = [engine_params_from_oracle(iris, op, precision=precision, ak=ak) for _, op, ak, _ in cells]
    b = iris.Batch(params, cells[0][1].fw, dft_faces=iris.DFT_Z)
    for c, (_, _, _, eps) in enumerate(cells):
        b.set_material(c, eps)
    if tile is not None:
        b.set_tile(tile)
        assert b.info()["tile"] == iris.TILES[tile]
    if tune:
        tile, ms = b.tune(reps=2)
        assert tile in iris.TILES and len(ms) == len(iris.TILES)
    its = output_steps(cells[0][1])
    it = 1
    for t in its:
        b.step(it, t - it + 1)
        it = t + 1
    singles = []
    for (_, op, ak, eps), p in zip(cells, params):
        q = p.copy()
        q.dft_faces = iris.DFT_Z
        e = iris.Engine(q, op.fw)
        e.set_material(eps)
        J = run_engine_blocks(e, op, its)
        singles.append((e, J[-1]))
    return b, singles


@pytest.mark.parametrize("tile", [0, 3, 5, 6, 7])
@pytest.mark.parametrize("precision,tol", [(0, 0.0), (1, 0.0)])
def test_batch_matches_single_engines(iris, oracle, tmp_path, precision, tol, tile):
    cells = make_cells(oracle, tmp_path)
    if tile == 7 and precision == 0:
        # the fused work list is FP32 only
        params = [engine_params_from_oracle(iris, op, precision=0, ak=ak) for _, op, ak, _ in cells]
        b = iris.Batch(params, cells[0][1].fw, dft_faces=iris.DFT_Z)
        with pytest.raises(iris.IrisError) as e:
            b.set_tile(7)
        assert e.value.code == -1
        return
    b, singles = batch_and_singles(iris, cells, precision, tile=tile)
    assert b.info()["cells"] == len(CELLS)
    for c, (e, Js) in enumerate(singles):
        Jb = b.flux(c)
        # the single engines flush their DFT blocks at every output step, the
        # batch only when its ring is full: in FP32 the partial sums group
        # differently (and the tensor-core DFT's operand split rounds at ~4x
        # FP32's unit), so the spectra agree to 1e-5 while the fields stay at tol
        assert rel_err(Jb, Js) <= (tol if precision == 0 else 1e-5), c
        assert np.all(Jb[:4] == 0)  # only the z planes are accumulated
        for which in (iris.E, iris.H):
            fb = interior(b.get_field(c, which), cells[c][1])
            fs = interior(e.get_field(which), cells[c][1])
            assert rel_err(fb, fs) <= tol, (c, which)


def test_batch_against_oracle(iris, oracle, tmp_path):
    cells = make_cells(oracle, tmp_path)
    b, _ = batch_and_singles(iris, cells, 0, tune=True)
    for c, (w, op, ak, eps) in enumerate(cells):
        o = oracle.Oracle(op, ak=ak, threads=THREADS)
        o.set_eps_inv(eps)
        o.run(1, op.texit)
        Jo = o.flux(0)
        assert rel_err(b.flux(c)[4:], Jo[4:]) <= 1e-12, c


def test_batch_rejects_mixed_timesteps(iris, oracle, tmp_path):
    cells = make_cells(oracle, tmp_path)[:2]
    params = [engine_params_from_oracle(iris, op) for _, op, _, _ in cells]
    params[1].dt *= 1.01
    with pytest.raises(iris.IrisError) as e:
        iris.Batch(params, cells[0][1].fw)
    assert e.value.code == -1


def test_batch_tune_fp32_matches_single_engines(iris, oracle, tmp_path):
    """FP32 tuning times every work list, the fused one included (its second
    buffer sets are dropped again when another list wins), and stepping after
    it still matches the single engines bit for bit."""
    cells = make_cells(oracle, tmp_path)
    b, singles = batch_and_singles(iris, cells, 1, tune=True)
    assert b.info()["tile"] in iris.TILES
    for c, (e, _) in enumerate(singles):
        for which in (iris.E, iris.H):
            fb = interior(b.get_field(c, which), cells[c][1])
            fs = interior(e.get_field(which), cells[c][1])
            assert np.array_equal(fb, fs), (c, which)


def test_batch_fused_complex_material(iris, oracle, tmp_path):
    """The fused work list with a lossy (complex) material in one cell runs
    the complex-material kernel for the whole batch, still bitwise the single
    engines."""
    cells = make_cells(oracle, tmp_path)[:3]
    r = np.random.default_rng(9)
    w, op, ak, eps = cells[1]
    eps = eps.astype(complex) + 1j * r.uniform(-0.05, 0.0, eps.shape)
    cells[1] = (w, op, ak, eps)
    b, singles = batch_and_singles(iris, cells, 1, tile=7)
    for c, (e, _) in enumerate(singles):
        for which in (iris.E, iris.H):
            fb = interior(b.get_field(c, which), cells[c][1])
            fs = interior(e.get_field(which), cells[c][1])
            assert np.array_equal(fb, fs), (c, which)


def test_batch_fused_cell_without_interior_range(iris, oracle, tmp_path):
    """A cell whose UPML slabs leave no planes for the launch without slab
    code (pmlzf = pmlzi + 2) rides in the slab launch of the fused list."""
    cells = make_cells(oracle, tmp_path)[:2]
    w = cfg.Workload("thin", 10, 6, 20, 6, 8, 7, 1, 4.0, 0, 7, (1, 10, 1, 6, 3, 17), 9, STEPS,
                     structure="pattern", extra=dict(seed=77, fill=0.5))
    op = oracle.setparam(cfg.write_input(str(tmp_path / "thin.dat"), w, no_downloads=3))
    cells.append((w, op, (0.2 + 0j, 0j, 0j), cfg.binary_pattern_material(w)))
    b, singles = batch_and_singles(iris, cells, 1, tile=7)
    for c, (e, _) in enumerate(singles):
        for which in (iris.E, iris.H):
            fb = interior(b.get_field(c, which), cells[c][1])
            fs = interior(e.get_field(which), cells[c][1])
            assert np.array_equal(fb, fs), (c, which)


def _batch(iris, cells, precision):
    params = [engine_params_from_oracle(iris, op, precision=precision, ak=ak) for _, op, ak, _ in cells]
    b = iris.Batch(params, cells[0][1].fw, dft_faces=iris.DFT_Z)
    for c, (_, _, _, eps) in enumerate(cells):
        b.set_material(c, eps)
    return b


def test_autotune_cache_by_size_class(iris, oracle, tmp_path):
    """iris_batch_autotune times the work lists once per size class: a second
    batch of the same class takes the cached pick without timing, and steps
    exactly like a batch set to that pick by hand."""
    cells = make_cells(oracle, tmp_path)
    a = _batch(iris, cells, 1)
    t1, c1 = a.autotune(reps=2)
    b = _batch(iris, cells, 1)
    t2, c2 = b.autotune(reps=2)
    assert (t2, c2) == (t1, True)
    if not c1:  # this process had not seen the class before
        assert t1 in iris.TILES
    ref = _batch(iris, cells, 1)
    ref.set_tile(iris.TILES.index(t1))
    for x in (b, ref):
        x.step(1, 20)
    for c in range(len(cells)):
        assert np.array_equal(b.get_field(c, iris.E), ref.get_field(c, iris.E)), c
    for x in (a, b, ref):
        x.close()


CHILD = """
import importlib, os, sys
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, os.path.join(sys.argv[1], "tests"))
import numpy as np
iris = importlib.import_module("irisfdtd-academic_gb300")
cfg = importlib.import_module("irisfdtd-academic_gb300.configs")
params, mats = [], []
for i, (nx, ny, nz) in enumerate([(12, 7, 60), (33, 9, 48), (5, 17, 72)]):
    w = cfg.Workload("t%d" % i, nx, ny, nz, 8, nz - 7, nz // 2 - 5, 10, 1.0, 0, 14, (1, nx, 1, ny, 10, nz - 10), 9, 40,
                     structure="pattern", extra=dict(seed=7 + i, fill=0.5))
    p, fw, _ = iris.setparam(cfg.write_input(os.path.join(sys.argv[2], "t%d.dat" % i), w))
    p.precision = iris.FP32
    params.append(p)
    mats.append(cfg.binary_pattern_material(w))
b = iris.Batch(params, fw, dft_faces=iris.DFT_Z)
for c, m in enumerate(mats):
    b.set_material(c, m)
tile, cached = b.autotune(reps=1)
print("PICK", iris.TILES.index(tile), int(cached))
"""


def test_autotune_cache_file_across_processes(tmp_path):
    """With IRIS_TUNE_CACHE set, the first process times and appends its pick;
    a second process reads the file and takes the pick without timing."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, IRIS_TUNE_CACHE=str(tmp_path / "tune.txt"))
    out = []
    for _ in range(2):
        r = subprocess.run([sys.executable, "-c", CHILD, root, str(tmp_path)], env=env, capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stderr[-3000:]
        tile, cached = r.stdout.split("PICK")[1].split()
        out.append((int(tile), int(cached)))
    assert out[0][1] == 0 and out[1] == (out[0][0], 1)
    lines = (tmp_path / "tune.txt").read_text().split("\n")
    assert len([ln for ln in lines if ln.strip()]) == 1 and "|fp32|real|" in lines[0]
