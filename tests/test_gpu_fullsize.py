"""Size-independent properties of the hot path on the full 512x512x1024 Bloch
cell of the spheres workload (200 seeded spheres, 24-cell UPML, kx = 0.3
pi/dx), where the FP64 oracle cannot follow:

* the fused FP32 pass (the default) equals the split passes bit for bit;
* the step is linear in the source amplitude: doubling the TF/SF amplitude
  doubles every field value and quadruples the flux.  In FP64 this holds bit
  for bit (scaling by 2 is exact in binary floating point; checked on the
  cell resized to 160 planes, where FP64 steps are quick).  In FP32 it holds
  to a few ulps (normwise 1e-5 of the field's scale asserted): the FP32
  stencil alone is exactly homogeneous, but the Gaussian pulse rises at the
  source through the FP32 subnormal range, whose fixed absolute quantum does
  not scale with the amplitude; once the two runs differ anywhere, their
  later roundings differ too, and the difference settles at FP32 rounding;
* the fluxes are finite, and the x/y faces carry the flux scattered sideways
  by the spheres.
"""
import importlib
import os
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
cfg = importlib.import_module("irisfdtd-academic_gb300.configs")
STEPS = 800  # the pulse reaches the sphere layer (z = 412) and scatters sideways


@pytest.fixture(scope="module")
def full(iris):
    w = cfg.workload(3)
    eps = cfg.material(w)
    path = cfg.write_input(os.path.join(tempfile.mkdtemp(), "inputFDTD.dat"), w)
    p, fw, _ = iris.setparam(path)
    p.precision = iris.FP32
    p.to_fourier = 1  # every face pair sampled from the first step
    return w, p, fw, eps


def run(iris, full, stencil=0, scale=1.0):
    w, p, fw, eps = full
    q = p.copy()
    q.epump = p.epump * scale
    e = iris.Engine(q, fw, stencil=stencil)
    try:
        e.set_material(eps)
        e.step(1, STEPS)
        J = e.flux(0)
        zi = p.tfsf_zi
        planes = [e.get_plane(which, 3, z, (1, p.nx), (1, p.ny))
                  for which, z in ((iris.E, zi), (iris.H, zi - 1), (iris.E, zi - 6), (iris.E, zi + 9), (iris.H, zi + 20),
                                   (iris.E, 320), (iris.H, 340))]  # the last two inside the pulse
    finally:
        e.close()
    return J, planes


@pytest.fixture(scope="module")
def base(iris, full):
    return run(iris, full)


def test_fullsize_flux_finite_and_nonzero(iris, full, base):
    J, planes = base
    assert np.all(np.isfinite(J))
    assert np.any(J[:4] != 0)  # scattered sideways by the spheres
    assert all(np.any(pl != 0) for pl in planes)


def test_fullsize_linear_in_the_source(iris, full, base):
    J, planes = base
    J2, planes2 = run(iris, full, scale=2.0)
    assert np.max(np.abs(J2 - 4.0 * J)) <= 1e-5 * np.max(np.abs(4.0 * J))
    # relative to the field's scale (the planes inside the pulse): behind the
    # pulse a plane holds residuals a million times smaller, which carry the
    # pulse's FP32 rounding
    scale = max(np.max(np.abs(a)) for a in planes)
    for a, b in zip(planes, planes2):
        assert np.max(np.abs(b - 2.0 * a)) <= 1e-5 * 2.0 * scale


def test_linear_in_the_source_fp64_bitwise(iris):
    w = cfg.resized(cfg.workload(3), 512, 512, 160, nof=16)
    eps = cfg.material(w)
    p, fw, _ = iris.setparam(cfg.write_input(os.path.join(tempfile.mkdtemp(), "inputFDTD.dat"), w))
    p.precision = iris.FP64
    p.to_fourier = 1
    out = []
    for scale in (1.0, 2.0):
        q = p.copy()
        q.epump = p.epump * scale
        e = iris.Engine(q, fw)
        try:
            e.set_material(eps)
            e.step(1, 200)
            out.append((e.flux(0), e.get_plane(iris.E, 3, p.tfsf_zi + 3, (1, p.nx), (1, p.ny)),
                        e.get_plane(iris.H, 3, p.tfsf_zi - 2, (1, p.nx), (1, p.ny))))
        finally:
            e.close()
    (J1, e1, h1), (J2, e2, h2) = out
    assert np.any(e1 != 0)
    assert np.array_equal(J2, 4.0 * J1)
    assert np.array_equal(e2, 2.0 * e1) and np.array_equal(h2, 2.0 * h1)


def test_fullsize_fused_equals_split(iris, full, base):
    J, planes = base
    Js, planes_s = run(iris, full, stencil=iris.STENCIL_SPLIT)
    assert np.array_equal(J, Js)
    for a, b in zip(planes, planes_s):
        assert np.array_equal(a, b)
