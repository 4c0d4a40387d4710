"""Field transfer in the reference's own storage (iris_get_field_c,
iris_set_field_c, iris_get_pml_c, iris_set_pml_c): complex(8) arrays
e(3, 0:nx+1, 0:ny+1, 0:nz+1) and the UPML auxiliaries (3, 1:nx, 1:ny, planes)
as code/main.f90:166-167 and code/driver.f90:177-188 allocate them, written
and read on the device a few z planes at a time.  They must carry exactly
what the split re/im calls carry, both ways, in both precisions, including
a grid large enough that the transfer runs in several chunks of the 64 MB
staging buffer."""
import importlib

import numpy as np
import pytest

from helpers import engine_params_from_oracle

pytestmark = pytest.mark.gpu
cfg = importlib.import_module("irisfdtd-academic_gb300.configs")


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("grid", [(9, 5, 40), (130, 130, 120)], ids=["small", "chunked"])
def test_complex8_transfer_equals_split_transfer(iris, oracle, tmp_path, precision, grid):
    nx, ny, nz = grid
    w = cfg.Workload("xfer", nx, ny, nz, 6, nz - 5, nz // 3, 8, 4.0, 0, 10, (1, nx, 1, ny, 8, nz - 8), 4, 30)
    op = oracle.setparam(cfg.write_input(str(tmp_path / "x.dat"), w))
    e = iris.Engine(engine_params_from_oracle(iris, op, precision=precision, ak=(0.3 + 0j, 0j, 0j)), op.fw,
                    stencil=iris.STENCIL_SPLIT)
    e.step(1, 25)  # a state that is not zero
    r = np.random.default_rng(1)
    for which in (iris.E, iris.H):
        a = e.get_field(which)
        c = e.get_field_c(which)
        assert c.shape == a.shape == (nz + 2, ny + 2, nx + 2, 3)
        assert np.array_equal(a, c), which
        # set through the interleaved call, read through both
        v = r.standard_normal(a.shape) + 1j * r.standard_normal(a.shape)
        if precision == 1:
            v = v.astype(np.complex64).astype(np.complex128)  # exactly representable in FP32
        e.set_field_c(which, v)
        assert np.array_equal(e.get_field(which), v)
        assert np.array_equal(e.get_field_c(which), v)
    for which in (0, 1):
        for slab in (0, 1):
            a = e.get_pml(which, slab)
            assert np.array_equal(e.get_pml_c(which, slab), a), (which, slab)
            v = r.standard_normal(a.shape) + 1j * r.standard_normal(a.shape)
            if precision == 1:
                v = v.astype(np.complex64).astype(np.complex128)
            e.set_pml_c(which, slab, v)
            assert np.array_equal(e.get_pml(which, slab), v), (which, slab)
    # the state written through the interleaved calls steps like one written through the split calls
    twin = iris.Engine(engine_params_from_oracle(iris, op, precision=precision, ak=(0.3 + 0j, 0j, 0j)), op.fw,
                       stencil=iris.STENCIL_SPLIT)
    for which in (iris.E, iris.H):
        twin.set_field(which, e.get_field(which))
    for which in (0, 1):
        for slab in (0, 1):
            twin.set_pml(which, slab, e.get_pml(which, slab))
    e.step(26, 5)
    twin.step(26, 5)
    assert np.array_equal(e.get_field_c(iris.E), twin.get_field(iris.E))
