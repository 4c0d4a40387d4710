"""The gradient form (iris_adjoint_*): the adjoint kernels are the conjugate
transpose of the forward step, the gradient matches central finite
differences of the FP64 forward, does not depend on the checkpoint interval,
and the FP32 adjoint agrees with the FP64 one.

The case is the adjoint workload's shape at test size: a periodic cell with
UPML at both z ends, a TF/SF plane, a layer holding a design region of
continuous eps in [1, 12], DFT planes below and above it, and a Bloch phase
along x.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
cfg = importlib.import_module("irisfdtd-academic_gb300.configs")

NX, NY, NZ = 12, 10, 96
DESIGN = (3, 10, 2, 9, 44, 51)  # x0 x1 y0 y1 z0 z1 = the whole structure layer in z
AKX = 0.7
NSTEPS = 600


def small_case(iris, tmp_path, nsteps=NSTEPS, nof=6, akx=AKX, seed=5):
    x0, x1, y0, y1, z0, z1 = DESIGN
    w = cfg.Workload("adjoint_small", NX, NY, NZ, 8, NZ - 7, z0, z1 - z0 + 1, 1.0, 0, 14, (1, NX, 1, NY, 12, 84),
                     nof, nsteps, structure="design", extra=dict(x0=x0, x1=x1, y0=y0, y1=y1, emin=1.0, emax=12.0))
    p, fw, _ = iris.setparam(cfg.write_input(str(tmp_path / "adjoint.dat"), w))
    p.akx_re = akx
    eps_inv = cfg.design_region_material(w, seed=seed).real
    eta = eps_inv[1:-1, y0:y1 + 1, x0:x1 + 1].copy()
    return p, fw, eps_inv, eta


def rnd(r, shape):
    return r.standard_normal(shape) + 1j * r.standard_normal(shape)


def dot(a, b):
    return float(np.sum((np.conj(a) * b).real))


@pytest.mark.parametrize("precision,tol", [(0, 1e-13), (1, 1e-5)])
@pytest.mark.parametrize("nsteps", [1, 3])
def test_adjoint_is_conjugate_transpose(iris, tmp_path, precision, tol, nsteps):
    """<lam, A^n s> == <(A^H)^n lam, s> over E, H, D and B (no source)."""
    p, fw, eps_inv, _ = small_case(iris, tmp_path)
    p.epump = 0.0
    adj = iris.Adjoint(p, fw, DESIGN, precision=precision)
    adj.set_material(eps_inv)
    F, A = adj.engine(0), adj.engine(1)
    r = np.random.default_rng(11)
    shp = F.field_shape
    inner = (slice(1, NZ + 1), slice(1, NY + 1), slice(1, NX + 1))
    s = {}
    for which in (iris.E, iris.H):
        f = np.zeros(shp, dtype=complex)
        f[inner] = rnd(r, (NZ, NY, NX, 3))
        if which == iris.H:  # the ghosts the E pass reads: Bloch images of interior cells
            f[1:NZ + 1, 1:NY + 1, 0] = np.exp(-1j * AKX) * f[1:NZ + 1, 1:NY + 1, NX]
            f[1:NZ + 1, 0, 1:NX + 1] = f[1:NZ + 1, NY, 1:NX + 1]
            f[0, 1:NY + 1, 1:NX + 1] = f[NZ, 1:NY + 1, 1:NX + 1]
        F.set_field(which, f)
        s[which] = f[inner]
    for which in (0, 1):
        for slab in (0, 1):
            v = rnd(r, F.pml_shape(slab))
            F.set_pml(which, slab, v)
            s[(which, slab)] = v
    F.step(1, nsteps)
    As = {k: (F.get_field(k)[inner] if k in (iris.E, iris.H) else F.get_pml(*k)) for k in s}
    lam = {}
    for which in (iris.E, iris.H):
        f = np.zeros(shp, dtype=complex)
        f[inner] = rnd(r, (NZ, NY, NX, 3))
        A.set_field(which, f)
        lam[which] = f[inner]
    for which in (0, 1):
        for slab in (0, 1):
            v = rnd(r, F.pml_shape(slab))
            A.set_pml(which, slab, v)
            lam[(which, slab)] = v
    adj.apply(nsteps)
    AHl = {k: (A.get_field(k)[inner] if k in (iris.E, iris.H) else A.get_pml(*k)) for k in s}
    lhs = sum(dot(lam[k], As[k]) for k in s)
    rhs = sum(dot(AHl[k], s[k]) for k in s)
    norm = np.sqrt(sum(np.sum(np.abs(lam[k]) ** 2) for k in s) * sum(np.sum(np.abs(As[k]) ** 2) for k in s))
    assert abs(lhs - rhs) <= tol * norm, (lhs, rhs, norm)
    adj.close()


def gradient(iris, p, fw, eps_inv, eta, precision, K=64, weights=None, nsteps=NSTEPS):
    adj = iris.Adjoint(p, fw, DESIGN, checkpoint_every=K, weights=weights, precision=precision)
    adj.set_material(eps_inv)
    adj.set_design(eta)
    L, J = adj.forward(nsteps)
    g = adj.backward()
    return adj, L, J, g


def test_objective_is_weighted_flux(iris, tmp_path):
    p, fw, eps_inv, eta = small_case(iris, tmp_path)
    r = np.random.default_rng(3)
    w5, w6 = r.uniform(0.5, 1.5, p.nof), r.uniform(0.5, 1.5, p.nof)
    adj, L, J, _ = gradient(iris, p, fw, eps_inv, eta, 0, weights=(w5, w6))
    assert L == pytest.approx(float(w5 @ J[4] + w6 @ J[5]), rel=1e-14)
    # the same run through the plain engine gives the same fluxes
    q = p.copy()
    q.dft_faces = iris.DFT_Z
    e = iris.Engine(q, fw, precision=iris.FP64)
    e.set_material(eps_inv)
    e.step(1, NSTEPS)
    assert np.max(np.abs(e.flux(0)[4:] - J[4:])) <= 1e-13 * np.max(np.abs(J[4:]))


def test_gradient_matches_central_differences(iris, tmp_path):
    """FP64 adjoint against (L(eps+h) - L(eps-h)) / 2h, h = 1e-3, at 32 seeded
    voxels, objective weighting both the J5 and the J6 plane."""
    p, fw, eps_inv, eta = small_case(iris, tmp_path)
    r = np.random.default_rng(7)
    weights = (r.uniform(-1.0, 1.0, p.nof), r.uniform(0.5, 1.5, p.nof))
    adj, L, _, g = gradient(iris, p, fw, eps_inv, eta, 0, weights=weights)
    eps = 1.0 / eta
    dL_deps = -g * eta ** 2
    flat = r.choice(eta.size, 32, replace=False)
    h = 1e-3
    fd, ad = [], []
    for q in flat:
        idx = np.unravel_index(q, eta.shape)
        vals = []
        for sgn in (1, -1):
            e2 = eps.copy()
            e2[idx] += sgn * h
            adj.set_design(1.0 / e2)
            vals.append(adj.forward(NSTEPS)[0])
        fd.append((vals[0] - vals[1]) / (2 * h))
        ad.append(dL_deps[idx])
    fd, ad = np.array(fd), np.array(ad)
    err = np.max(np.abs(fd - ad)) / np.max(np.abs(fd))
    assert err <= 1e-4, (err, fd[:4], ad[:4])


def test_gradient_independent_of_checkpoint_interval(iris, tmp_path):
    p, fw, eps_inv, eta = small_case(iris, tmp_path)
    g = [gradient(iris, p, fw, eps_inv, eta, 0, K=K)[3] for K in (7, 64, NSTEPS)]
    assert np.array_equal(g[0], g[2]) and np.array_equal(g[1], g[2])


def test_fp32_adjoint_matches_fp64(iris, tmp_path):
    p, fw, eps_inv, eta = small_case(iris, tmp_path)
    _, L64, _, g64 = gradient(iris, p, fw, eps_inv, eta, 0)
    _, L32, _, g32 = gradient(iris, p, fw, eps_inv, eta, 1)
    assert abs(L32 - L64) <= 1e-4 * abs(L64)
    assert np.max(np.abs(g32 - g64)) / np.max(np.abs(g64)) <= 1e-3


def test_torch_function(iris, tmp_path):
    torch = pytest.importorskip("torch")
    p, fw, eps_inv, eta = small_case(iris, tmp_path)
    adj, L, _, g = gradient(iris, p, fw, eps_inv, eta, 0)
    f = iris.design_objective(adj, NSTEPS)
    eps = torch.tensor(1.0 / eta, dtype=torch.float64, requires_grad=True)
    Lt = f(eps)  # the design is re-set from 1/(1/eta): equal to roundoff
    assert float(Lt.detach()) == pytest.approx(L, rel=1e-12)
    Lt.backward()
    want = -g * eta ** 2
    assert np.max(np.abs(eps.grad.numpy() - want)) <= 1e-9 * np.max(np.abs(want))


def test_rejects_bad_design_and_complex_material(iris, tmp_path):
    p, fw, eps_inv, eta = small_case(iris, tmp_path)
    with pytest.raises(iris.IrisError) as e:
        iris.Adjoint(p, fw, (3, 10, 2, 9, 40, 51))  # below hi
    assert e.value.code == -1
    adj = iris.Adjoint(p, fw, DESIGN)
    with pytest.raises(iris.IrisError):
        adj.set_material(eps_inv * (1 + 0.1j))
