"""Graph replay (iris_params.graph): whole DFT blocks of steps replayed from
one captured CUDA graph give results identical, bit for bit, to stepping
launch by launch, for the plain engine (FP64 and FP32 split, FP32 fused and
streamed; the persistent kernel of small grids takes no graphs) and
for the batch, including step calls that start and end inside a block, a
DFT start step after step 1, and a material change after the capture."""
import importlib

import numpy as np
import pytest

from helpers import engine_params_from_oracle, interior
from test_gpu_fused import make_case

pytestmark = pytest.mark.gpu
cfg = importlib.import_module("irisfdtd-academic_gb300.configs")
SPEC = (37, 21, 64, 8, 57, 24, 14, 2.25, 12, (1, 37, 1, 21, 9, 54))
CALLS = [(1, 10), (11, 50), (61, 37), (98, 16)]


def engines(iris, oracle, tmp_path, precision, stencil, to_fourier=7):
    w, op = make_case(oracle, tmp_path, SPEC, 2)
    p = engine_params_from_oracle(iris, op, precision=precision, ak=(0.4 + 0j, 0j, 0j))
    p.to_fourier = to_fourier
    eps = cfg.spheres_material(w, seed=3)
    out = []
    for graph in (False, True):
        e = iris.Engine(p, op.fw, dft_block=16, stencil=stencil, graph=graph)
        e.set_material(eps)
        out.append(e)
    return w, op, eps, out


def same(a, b, op, iris):
    for which in (iris.E, iris.H):
        assert np.array_equal(interior(a.get_field(which), op), interior(b.get_field(which), op)), which
    assert np.array_equal(a.flux(0), b.flux(0))


@pytest.mark.parametrize("precision,stencil", [(0, 1), (1, 1), (1, 2), (1, 3)])
def test_graph_steps_identical(iris, oracle, tmp_path, precision, stencil):
    w, op, eps, (plain, graphed) = engines(iris, oracle, tmp_path, precision, stencil)
    for it0, n in CALLS:
        plain.step(it0, n)
        graphed.step(it0, n)
    same(plain, graphed, op, iris)


def test_graph_after_material_change(iris, oracle, tmp_path):
    w, op, eps, (plain, graphed) = engines(iris, oracle, tmp_path, 1, 1)
    for e in (plain, graphed):
        e.step(1, 40)
        e.set_material(eps * 0.9)
        e.step(41, 40)
    same(plain, graphed, op, iris)


def test_graph_not_used_under_per_kernel_timing(iris, oracle, tmp_path):
    w, op, eps, (_, graphed) = engines(iris, oracle, tmp_path, 1, 1, to_fourier=0)
    graphed.timing_start(per_kernel=True)
    graphed.step(1, 32)
    _, _, n = graphed.timing_read()
    assert n["update_e"] == 32


@pytest.mark.parametrize("tile", [5, 7])
def test_batch_graph_identical(iris, oracle, tmp_path, tile):
    from test_gpu_batch import make_cells
    cells = make_cells(oracle, tmp_path)
    params = [engine_params_from_oracle(iris, op, precision=1, ak=ak) for _, op, ak, _ in cells]
    for p in params:
        p.to_fourier = 5
    bs = []
    for graph in (False, True):
        b = iris.Batch(params, cells[0][1].fw, dft_faces=iris.DFT_Z, dft_block=16, graph=graph)
        for c, (_, _, _, eps) in enumerate(cells):
            b.set_material(c, eps)
        b.set_tile(tile)
        for it0, n in CALLS:
            b.step(it0, n)
        bs.append(b)
    for c in range(len(cells)):
        assert np.array_equal(bs[0].flux(c), bs[1].flux(c)), c
        for which in (iris.E, iris.H):
            assert np.array_equal(bs[0].get_field(c, which), bs[1].get_field(c, which)), (c, which)
