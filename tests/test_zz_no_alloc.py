"""The allocation-free DFT entry point (iris_dft_block_noalloc).

It serves callers that cannot allocate device memory while they run (their
memory belongs to a pooling allocator, or allocation after start-up is not
allowed): they pass buffers they already own and the library uses only a
fixed device array for its scratch.  This test gives it samples in
device memory owned by the test (torch tensors, standing in for such a
caller's pool), calls it twice in a row on the same accumulators, and checks
the result against the engine's own FP32 DFT path (iris_create +
iris_apply(IRIS_OP_DFT) + iris_get_fdata) on the same samples, and against
a direct numpy sum in FP64 of samples x dt x exp(i fw t) over the same
samples.

Tolerance 1e-5 norm-wise relative: the paths form the same FP32 products
from the same FP64 twiddles; they differ only in how many samples share one
FP32 partial sum before the FP64 add (one per sample in the engine path,
three and two here, none in numpy's FP64 sum).

This file is collected last, so a run that stops at the first failure has
already run every other test.
"""
import importlib

import numpy as np
import pytest

from helpers import rel_err

pytestmark = pytest.mark.gpu


def test_noalloc_matches_engine_dft(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    iris = importlib.import_module("irisfdtd-academic_gb300")
    cfg = importlib.import_module("irisfdtd-academic_gb300.configs")
    nbx, nby = 6, 5
    w = cfg.Workload("noalloc", nbx, nby, 40, 6, 35, 15, 10, 4.0, 0, 10, (1, nbx, 1, nby, 8, 32), 24, 50)
    p, fw, _ = iris.setparam(cfg.write_input(str(tmp_path / "inputFDTD.dat"), w))
    eng = iris.Engine(p, fw, precision=iris.FP32)
    rng = np.random.default_rng(11)
    nloc = nbx * nby
    npts = 12 * nloc  # face pair 3 (the two z planes), 6 components each
    t0, step = 7, 3
    times = [t0 + k * step for k in range(5)]
    samples = np.zeros((len(times), npts), np.complex64)
    L_idx = np.arange(nloc)
    for k, t in enumerate(times):
        # FP32-representable fields, so the engine's FP32 storage holds them exactly
        E = (rng.standard_normal(eng.field_shape) + 1j * rng.standard_normal(eng.field_shape)).astype(np.complex64)
        H = (rng.standard_normal(eng.field_shape) + 1j * rng.standard_normal(eng.field_shape)).astype(np.complex64)
        eng.set_field(iris.E, E.astype(np.complex128))
        eng.set_field(iris.H, H.astype(np.complex128))
        eng.scattering_fourier(t)
        # the same samples in the reference's point order of face pair 3:
        # i_pts - 1 = side*6*nloc + ip + 6*L, L = (ix-1) + nbx*(iy-1)
        for side, z in enumerate((w.box[4], w.box[5])):
            for ip in range(6):
                F = E if ip < 3 else H
                samples[k, side * 6 * nloc + ip + 6 * L_idx] = F[z, 1:nby + 1, 1:nbx + 1, ip % 3].reshape(-1)
    ref = eng.get_fdata(0, 3)
    eng.close()
    assert ref.shape == (p.nof, npts)

    dev = torch.device("cuda", 0)
    S = torch.from_numpy(samples.view(np.float32).reshape(len(times), npts, 2).copy()).to(dev)
    FW = torch.from_numpy(np.ascontiguousarray(fw, dtype=np.float64)).to(dev)
    FD = torch.zeros((p.nof, npts, 2), dtype=torch.float64, device=dev)
    L = iris.lib()
    stream = torch.cuda.current_stream(dev).cuda_stream
    # two calls in a row on the same accumulators: samples 0..2, then 3..4
    rc1 = L.iris_dft_block_noalloc(S.data_ptr(), 3, npts, times[0], step, FW.data_ptr(), p.nof, p.dt,
                                   FD.data_ptr(), stream)
    assert rc1 == 0, L.iris_last_error()
    rc2 = L.iris_dft_block_noalloc(S[3].data_ptr(), 2, npts, times[3], step, FW.data_ptr(), p.nof, p.dt,
                                   FD.data_ptr(), stream)
    assert rc2 == 0, L.iris_last_error()
    torch.cuda.synchronize(dev)
    got = FD.cpu().numpy()
    got = got[..., 0] + 1j * got[..., 1]
    assert np.all(np.isfinite(got))
    assert rel_err(got, ref) <= 1e-5
    # independent of the engine: fdata[iw, p] = sum_k F_k(p) dt exp(i fw(iw) t_k), in FP64
    tw = p.dt * np.exp(1j * np.outer(np.asarray(fw, np.float64), np.asarray(times, np.float64)))
    direct = tw @ samples.astype(np.complex128)
    assert rel_err(got, direct) <= 1e-5

    # The refusals (a block whose twiddle table would not fit the fixed
    # scratch, null or misaligned pointers) are checked on the CPU in
    # tests/test_abi.py: every argument check precedes the first CUDA call,
    # and a launch of a refused block would write past the scratch array.
