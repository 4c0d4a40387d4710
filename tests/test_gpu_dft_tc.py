"""The FP32 DFT block on the tensor cores (IRIS_DFT_KERNEL_TENSOR: tcgen05
kind::tf32 with the hi/lo operand split) against the CUDA-core FP32 block
kernel and against the FP64 oracle.

Both FP32 kernels form the same twiddles and add one FP32 partial sum per
block into FP64 accumulators; they differ in the order of the FP32 partial
sums and in the TF32 split (error ~2^-21 per product), so the accumulators
agree within 1e-5 norm-wise and the flux spectra within 1e-5; against the
FP64 oracle the tolerance is the FP32 mode's 1e-4.  Cases: every face pair in
3D with 300 frequencies (three frequency groups, the last one partial), DFT
blocks of 32 and 256 samples with a partial block flushed at the flux read,
and a 2-D grid.

The FP32 flux read on the tensor cores (k_dft_ws in flux mode) adds the samples still
buffered on the fly and leaves them buffered: it changes no state, and
committing the buffer first gives the same spectra bit for bit (the pending
sums are the same MMAs on the same operands).
"""
import importlib
import os

import numpy as np
import pytest

from helpers import engine_params_from_oracle, interior, output_steps, rel_err, run_engine_blocks

pytestmark = pytest.mark.gpu
cfg = importlib.import_module("irisfdtd-academic_gb300.configs")
THREADS = max(1, min(16, os.cpu_count() or 1))

CASES = [
    ("3d_300freq", (24, 16, 64, 8, 57, 24, 14, 2.25, 12, (1, 24, 1, 16, 9, 54)), 300, 90),
    ("2d_slit", (40, 1, 80, 10, 71, 30, 12, 9.0, 16, (1, 40, 1, 1, 12, 66)), 37, 200),
]


def make(oracle, tmp_path, spec, nof, steps):
    nx, ny, nz, pmlzi, pmlzf, hi, dh, eps, zi, box = spec
    w = cfg.Workload("tc", nx, ny, nz, pmlzi, pmlzf, hi, dh, eps, 8 if nx >= 16 else 0, zi, box, nof, steps,
                     structure="spheres", extra=dict(nspheres=4, rmin=2, rmax=4, emin=1.5, emax=6.0))
    op = oracle.setparam(cfg.write_input(str(tmp_path / "tc.dat"), w, no_downloads=2))
    return w, op


@pytest.mark.parametrize("block", [32, 256])
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_tensor_dft_matches_cuda_core_dft(iris, oracle, tmp_path, case, block):
    name, spec, nof, steps = case
    w, op = make(oracle, tmp_path, spec, nof, steps)
    eps = cfg.spheres_material(w, seed=2)
    out = []
    for kern in (iris.DFT_KERNEL_CUDA, iris.DFT_KERNEL_TENSOR):
        e = iris.Engine(engine_params_from_oracle(iris, op, precision=1, ak=(0.3 + 0j, 0j, 0j)), op.fw,
                        dft_block=block, dft_kernel=kern)
        e.set_material(eps)
        e.step(1, steps)
        out.append(e)
    cc, tc = out
    assert rel_err(tc.flux(0), cc.flux(0)) <= 1e-5
    for j in (1, 2, 3):
        assert rel_err(tc.get_fdata(0, j), cc.get_fdata(0, j)) <= 1e-5, j


def test_tensor_dft_against_oracle(iris, oracle, tmp_path):
    name, spec, nof, steps = CASES[0]
    w, op = make(oracle, tmp_path, spec, 64, 240)
    eps = cfg.spheres_material(w, seed=2)
    e = iris.Engine(engine_params_from_oracle(iris, op, precision=1), op.fw, dft_kernel=iris.DFT_KERNEL_TENSOR)
    e.set_material(eps)
    J = run_engine_blocks(e, op, output_steps(op))
    o = oracle.Oracle(op, threads=THREADS)
    o.set_eps_inv(eps)
    Jo, _ = o.run(1, op.texit, max_out=len(output_steps(op)))
    assert rel_err(J, Jo) <= 1e-4
    assert rel_err(interior(e.get_field(iris.E), op), interior(o.get_field(o.E_CUR), op)) <= 1e-4


@pytest.mark.parametrize("steps,block", [(1, 256), (13, 256), (90, 32), (64, 32)])
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_flux_read_leaves_buffer_and_equals_commit(iris, oracle, tmp_path, case, steps, block):
    name, spec, nof, _ = case
    w, op = make(oracle, tmp_path, spec, nof, steps + 10)
    eps = cfg.spheres_material(w, seed=2)
    p = engine_params_from_oracle(iris, op, precision=1, ak=(0.3 + 0j, 0j, 0j))
    e = iris.Engine(p, op.fw, dft_block=block, dft_kernel=iris.DFT_KERNEL_TENSOR)
    e.set_material(eps)
    e.step(1, steps)
    sampled = sum(1 for it in range(1, steps + 1) if it >= op.to_fourier and it % op.sample_fourier == 0)
    n0 = e.info()["dft_buffered"]
    assert n0 == sampled % block
    J1 = e.flux(0)
    assert e.info()["dft_buffered"] == n0
    assert np.array_equal(e.flux(0), J1)  # a second read: same state, same bits
    e.dft_commit()
    assert e.info()["dft_buffered"] == 0
    J2 = e.flux(0)
    assert np.array_equal(J1, J2)
    # the CUDA-core path commits before it reads: same spectra to FP32's partial-sum rounding
    c = iris.Engine(p, op.fw, dft_block=block, dft_kernel=iris.DFT_KERNEL_CUDA)
    c.set_material(eps)
    c.step(1, steps)
    assert rel_err(J1, c.flux(0)) <= 1e-5
    # stepping on after a flux read: the buffer keeps filling and commits when full
    e.step(steps + 1, 10)
    c.step(steps + 1, 10)
    assert rel_err(e.flux(0), c.flux(0)) <= 1e-5


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_unwritten_accumulators_equal_zeroed(iris, oracle, tmp_path, case):
    """Until the first block is committed the accumulators hold no sum: the
    engine leaves their memory unwritten, the first tensor-core commit writes
    without reading and a flux read before it takes them as zeros.  An engine
    whose accumulators were zeroed in memory first (iris_get_fdata reads them
    as they lie, so it zeroes them) must give the same bits at every stage,
    and so must one that replays its blocks from a CUDA graph (the capture
    zeroes them, since the captured commit reads)."""
    name, spec, nof, _ = case
    block = 32
    w, op = make(oracle, tmp_path, spec, nof, 3 * block + 20)
    eps = cfg.spheres_material(w, seed=2)
    p = engine_params_from_oracle(iris, op, precision=1, ak=(0.3 + 0j, 0j, 0j))
    lazy = iris.Engine(p, op.fw, dft_block=block, dft_kernel=iris.DFT_KERNEL_TENSOR)
    zeroed = iris.Engine(p, op.fw, dft_block=block, dft_kernel=iris.DFT_KERNEL_TENSOR)
    graphed = iris.Engine(p, op.fw, dft_block=block, dft_kernel=iris.DFT_KERNEL_TENSOR, graph=True)
    assert not np.any(zeroed.get_fdata(0, 3))
    engines = (lazy, zeroed, graphed)
    for e in engines:
        e.set_material(eps)
        e.step(1, 13)
    assert lazy.info()["dft_buffered"] > 0
    J = [e.flux(0) for e in engines]  # before any commit
    assert np.all(np.isfinite(J[0])) and np.any(J[0])
    assert np.array_equal(J[0], J[1]) and np.array_equal(J[0], J[2])
    for e in engines:
        e.dft_commit()  # the first commit: written without a read on the lazy engine
    for j in (1, 2, 3):
        F = [e.get_fdata(0, j) for e in engines]
        assert np.array_equal(F[0], F[1]) and np.array_equal(F[0], F[2]), j
    for e in engines:
        e.step(14, 2 * block + 6)  # whole blocks on: committed (and replayed from the graph) on top of the first
    J = [e.flux(0) for e in engines]
    assert np.array_equal(J[0], J[1]) and np.array_equal(J[0], J[2])
    for e in engines:
        e.close()
