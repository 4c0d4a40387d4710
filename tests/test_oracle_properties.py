"""Size-independent properties of the CPU oracle itself, on the CPU.

The reference can be pinned to the numbers it states (test_oracle_pins.py);
these check the oracle's wrap and source handling where no reference number
exists:

* Bloch wrap with ak = 0 (code/boundary.f90:163-348): a cell repeated twice
  along x or y (material tiled, DFT box over the whole supercell) holds, in
  each copy, the small cell's fields; the flux through the faces normal to
  the repeat axis is the small cell's, through the other faces twice it.
  The deck is read with double-precision literals, so that the normal
  incidence source does not depend on x (with the reference's REAL(4) pi,
  cos(pi/2) is -4.4e-8 and the incident field varies with x at 1e-8).
* Linearity in the source amplitude: doubling Epump doubles every field
  value and quadruples every flux value, bit for bit (scaling by 2 is exact
  in binary floating point).
* The e_fdtd and h_fdtd operators against an independent vectorised numpy
  restatement of code/fdtd.f90:57-248, bit for bit, regions included; the
  Bloch wrap with complex ak on all three axes against numpy; the flux of
  the z faces recomputed in numpy from the oracle's own accumulators;
  UPML_Array_e and UPML_Array_h (with the component-to-profile permutation
  read from code/boundary_II.f90:86-99,170-183) and set_sz against numpy;
  the on-the-fly DFT of two samples over every face pair's sample list.
"""
import importlib
import math

import numpy as np
import pytest

cfg = importlib.import_module("irisfdtd-academic_gb300.configs")
NX, NY, NZ, STEPS = 5, 3, 48, 140


def workload(nx, ny):
    return cfg.Workload("periodic", nx, ny, NZ, 6, 43, 18, 10, 4.0, 0, 10, (1, nx, 1, ny, 8, 38), 9, STEPS,
                        structure="spheres", extra=dict(nspheres=3, rmin=1, rmax=3, emin=1.5, emax=6.0))


def tile(a, reps, axis):
    """Repeat the interior of a ghost-padded [z, y, x] array along axis
    (2: x, 1: y) and refill that axis's ghosts by the periodic wrap."""
    inner = np.take(a, range(1, a.shape[axis] - 1), axis=axis)
    t = np.concatenate([inner] * reps, axis=axis)
    n = t.shape[axis]
    return np.concatenate([np.take(t, [n - 1], axis=axis), t, np.take(t, [0], axis=axis)], axis=axis)


def run(oracle, tmp_path, w, eps, epump=1.0, name="in.dat"):
    p = oracle.setparam(cfg.write_input(str(tmp_path / name), w, epump=epump), single_literals=False)
    o = oracle.Oracle(p)
    try:
        o.set_eps_inv(eps)
        o.run(1, p.texit)
        return o.get_field(o.E_CUR), o.get_field(o.H_CUR), o.flux(0)
    finally:
        o.close()


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("axis", ["x", "y"])
def test_supercell_of_a_periodic_cell(oracle, tmp_path, axis):
    small = workload(NX, NY)
    eps = cfg.spheres_material(small, seed=11)
    reps = 2
    big = workload(NX * reps, NY) if axis == "x" else workload(NX, NY * reps)
    ax = 2 if axis == "x" else 1
    e1, h1, J1 = run(oracle, tmp_path, small, eps, name="small.dat")
    e2, h2, J2 = run(oracle, tmp_path, big, tile(eps, reps, ax), name="big.dat")
    assert np.any(e1[1:-1, 1:-1, 1:-1] != 0)
    n = NX if axis == "x" else NY
    for f1, f2 in ((e1, e2), (h1, h2)):
        want = f1[1:-1, 1:-1, 1:-1]
        for r in range(reps):
            sl = slice(1 + r * n, 1 + (r + 1) * n)
            got = f2[1:-1, 1:-1, sl] if axis == "x" else f2[1:-1, sl, 1:-1]
            assert rel(got, want) <= 1e-12, (axis, r)
    # faces 1, 2 (x), 3, 4 (y), 5, 6 (z): the repeat axis's faces keep their area
    factor = np.array([1, 1, reps, reps, reps, reps] if axis == "x" else [reps, reps, 1, 1, reps, reps])
    for j in range(6):
        assert rel(J2[j], factor[j] * J1[j]) <= 1e-12, j


def test_linear_in_the_source_bitwise(oracle, tmp_path):
    w = workload(NX, NY)
    eps = cfg.spheres_material(w, seed=11)
    e1, h1, J1 = run(oracle, tmp_path, w, eps, 1.0, "a.dat")
    e2, h2, J2 = run(oracle, tmp_path, w, eps, 2.0, "b.dat")
    assert np.any(J1 != 0)
    assert np.array_equal(e2, 2.0 * e1) and np.array_equal(h2, 2.0 * h1)
    assert np.array_equal(J2, 4.0 * J1)


# ---------------------------------------------------------------------------
# e_fdtd / h_fdtd of the oracle against an independent, vectorised numpy
# restatement of code/fdtd.f90:57-248 (same operation order, no FMA on either
# side, real eps_inv): equal to the last bit in every region, and nothing
# written outside the regions.

def _vec_case(oracle, tmp_path):
    w = cfg.Workload("ops", 7, 5, 40, 6, 35, 15, 9, 4.0, 0, 10, (1, 7, 1, 5, 8, 32), 5, 10)
    p = oracle.setparam(cfg.write_input(str(tmp_path / "ops.dat"), w))
    o = oracle.Oracle(p)
    rng = np.random.default_rng(21)
    eps = 1.0 / rng.uniform(1.0, 6.0, (p.hf - p.hi + 3, p.ny + 2, p.nx + 2)) + 0j
    o.set_eps_inv(eps)
    shp = o.field_shape
    fields = [rng.standard_normal(shp) + 1j * rng.standard_normal(shp) for _ in range(4)]
    return p, o, eps, fields


def _sh(a, dz=0, dy=0, dx=0):
    """a[z+dz, y+dy, x+dx] over the interior x, y and all z (z shifted later)."""
    return a[:, 1 + dy:a.shape[1] - 1 + dy, 1 + dx:a.shape[2] - 1 + dx]


def test_e_fdtd_against_numpy(oracle, tmp_path):
    p, o, eps, (e_prev, h_prev, e_cur0, _) = _vec_case(oracle, tmp_path)
    o.set_field(o.E_PREV, e_prev)
    o.set_field(o.H_PREV, h_prev)
    o.set_field(o.E_CUR, e_cur0)
    o.op("e_fdtd")
    got = o.get_field(o.E_CUR)
    H = [h_prev[..., k] for k in range(3)]
    want = e_cur0.copy()
    for z in range(p.pmlzi + 1, p.pmlzf):
        def at(k, dz=0, dy=0, dx=0):
            return _sh(H[k], dy=dy, dx=dx)[z + dz]
        c = [((at(2) - at(2, dy=-1)) - at(1)) + at(1, dz=-1),
             ((at(0) - at(0, dz=-1)) - at(2)) + at(2, dx=-1),
             ((at(1) - at(1, dx=-1)) - at(0)) + at(0, dy=-1)]
        if z < p.hi:
            m = 1.0 / p.eps1
        elif z > p.hf:
            m = 1.0 / p.eps3
        else:
            m = eps[z - p.hi + 1, 1:-1, 1:-1].real
        for k in range(3):
            want[z, 1:-1, 1:-1, k] = e_prev[z, 1:-1, 1:-1, k] + m * c[k]
    assert np.array_equal(got, want)


def test_h_fdtd_against_numpy(oracle, tmp_path):
    p, o, eps, (e_cur, h_prev, _, h_cur0) = _vec_case(oracle, tmp_path)
    o.set_field(o.E_CUR, e_cur)
    o.set_field(o.H_PREV, h_prev)
    o.set_field(o.H_CUR, h_cur0)
    o.op("h_fdtd")
    got = o.get_field(o.H_CUR)
    c0, Q, dt = p.consts["c0"], p.Q, p.dt
    coef = (dt * c0 / Q) * (dt * c0 / Q)
    E = [e_cur[..., k] for k in range(3)]
    want = h_cur0.copy()
    zmx = p.hf if p.pmlzf < p.hf else p.pmlzf - 1
    for z in range(p.pmlzi, zmx + 1):
        def at(k, dz=0, dy=0, dx=0):
            return _sh(E[k], dy=dy, dx=dx)[z + dz]
        c = [((at(2, dy=1) - at(2)) - at(1, dz=1)) + at(1),
             ((at(0, dz=1) - at(0)) - at(2, dx=1)) + at(2),
             ((at(1, dx=1) - at(1)) - at(0, dy=1)) + at(0)]
        for k in range(3):
            want[z, 1:-1, 1:-1, k] = h_prev[z, 1:-1, 1:-1, k] - coef * c[k]
    assert np.array_equal(got, want)


def test_bloch_wrap_against_numpy(oracle, tmp_path):
    """bc_{x,y,z}max_bloch / bc_{x,y,z}min_bloch (code/boundary.f90:163-348):
    the max ghosts of E and H take exp(+i ak) times the first interior plane,
    the min ghosts exp(-i ak) times the last, axis by axis over the interior
    of the other two axes (edges and corners untouched)."""
    w = cfg.Workload("bloch", 6, 4, 12, 3, 10, 5, 2, 4.0, 0, 4, (1, 6, 1, 4, 4, 8), 3, 10)
    p = oracle.setparam(cfg.write_input(str(tmp_path / "bloch.dat"), w))
    ak = (0.7 - 0.05j, -1.3 + 0.02j, 0.4 + 0j)
    o = oracle.Oracle(p, ak=ak)
    rng = np.random.default_rng(8)
    shp = o.field_shape
    for op, sign in (("bloch_max", +1), ("bloch_min", -1)):
        e0 = rng.standard_normal(shp) + 1j * rng.standard_normal(shp)
        h0 = rng.standard_normal(shp) + 1j * rng.standard_normal(shp)
        o.set_field(o.E_CUR, e0)
        o.set_field(o.H_CUR, h0)
        o.op(op)
        for f0, got in ((e0, o.get_field(o.E_CUR)), (h0, o.get_field(o.H_CUR))):
            want = f0.copy()
            fx, fy, fz = (np.exp(sign * 1j * a) for a in ak)
            if sign > 0:
                want[1:-1, 1:-1, -1] = fx * want[1:-1, 1:-1, 1]
                want[1:-1, -1, 1:-1] = fy * want[1:-1, 1, 1:-1]
                want[-1, 1:-1, 1:-1] = fz * want[1, 1:-1, 1:-1]
            else:
                want[1:-1, 1:-1, 0] = fx * want[1:-1, 1:-1, -2]
                want[1:-1, 0, 1:-1] = fy * want[1:-1, -2, 1:-1]
                want[0, 1:-1, 1:-1] = fz * want[-2, 1:-1, 1:-1]
            assert np.max(np.abs(got - want)) <= 1e-14 * np.max(np.abs(want)), op
            assert np.array_equal(got[1:-1, 1:-1, 1:-1], f0[1:-1, 1:-1, 1:-1])


def test_flux_from_the_accumulated_samples(oracle, tmp_path):
    """scattering_fourier_out (code/dataprocess.f90:246-277) restated in numpy
    on the oracle's own accumulators and sample list: J5 = -sum Re(Ex Hy* -
    Ey Hx*) over the z = szi face, J6 = +sum over z = szf, both times
    eps0 Q / (2 dt)."""
    w = workload(NX, NY)
    p = oracle.setparam(cfg.write_input(str(tmp_path / "flux.dat"), w), single_literals=False)
    o = oracle.Oracle(p)
    o.set_eps_inv(cfg.spheres_material(w, seed=11))
    o.run(1, 90)
    J = o.flux(0)
    fd = o.fdata(0, 3)             # [iw, point]
    pto = o.pto(0, 3)              # (component 1..6, ix, iy, iz) per point
    scale = p.consts["eps0"] * p.Q / (2.0 * p.dt)
    szi, szf = p.box1[4], p.box1[5]
    for j, z, sign in ((4, szi, -1.0), (5, szf, 1.0)):
        def comp(c):
            sel = (pto[:, 0] == c) & (pto[:, 3] == z)
            order = np.lexsort((pto[sel, 1], pto[sel, 2]))
            return fd[:, sel][:, order]
        ex, ey, hx, hy = comp(1), comp(2), comp(4), comp(5)
        want = sign * np.sum((ex * np.conj(hy) - ey * np.conj(hx)).real, axis=1) * scale
        assert np.any(want != 0)
        assert np.max(np.abs(J[j] - want)) <= 1e-12 * np.max(np.abs(want)), j


def test_upml_e_against_numpy(oracle, tmp_path):
    """UPML_Array_e (code/boundary_II.f90:60-138) restated in numpy: per slab
    curl * eps0^2, D_k decays with profile (2, 3, 1)[k] and E_k with profile
    (3, 1, 2)[k] (1-based, as in the reference), bit for bit."""
    p, o, eps, (e_prev, h_prev, e_cur0, _) = _vec_case(oracle, tmp_path)
    rng = np.random.default_rng(5)
    dprev = [rng.standard_normal(o.pml_shape(s)) + 1j * rng.standard_normal(o.pml_shape(s)) for s in (0, 1)]
    o.set_field(o.E_PREV, e_prev)
    o.set_field(o.H_PREV, h_prev)
    o.set_field(o.E_CUR, e_cur0)
    for s in (0, 1):
        o.set_pml(0, 0, s, dprev[s])
    o.op("upml_e")
    got_e = o.get_field(o.E_CUR)
    fpn, fmn, fpx, fmx = o.get_sz()
    eps0 = p.consts["eps0"]
    H = [h_prev[..., k] for k in range(3)]
    want_e = e_cur0.copy()
    pd, pe = (1, 2, 0), (2, 0, 1)
    for s, (z0, z1, fp, fm, eb) in enumerate(((1, p.pmlzi, fpn, fmn, p.eps1), (p.pmlzf, p.nz, fpx, fmx, p.eps3))):
        want_d = np.empty_like(dprev[s])
        for z in range(z0, z1 + 1):
            zr = z - z0

            def at(k, dz=0, dy=0, dx=0):
                return _sh(H[k], dy=dy, dx=dx)[z + dz]
            c = [((at(2) - at(2, dy=-1)) - at(1)) + at(1, dz=-1),
                 ((at(0) - at(0, dz=-1)) - at(2)) + at(2, dx=-1),
                 ((at(1) - at(1, dx=-1)) - at(0)) + at(0, dy=-1)]
            c = [(eps0 * eps0) * ck for ck in c]
            for k in range(3):
                dold = dprev[s][zr, :, :, k]
                dn = (fm[zr, pd[k]] / fp[zr, pd[k]]) * dold + ((2 * eb) / fp[zr, pd[k]]) * c[k]
                want_d[zr, :, :, k] = dn
                v = (fm[zr, pe[k]] / fp[zr, pe[k]]) * e_prev[z, 1:-1, 1:-1, k]
                wv = fp[zr, k] * dn - fm[zr, k] * dold
                want_e[z, 1:-1, 1:-1, k] = v + (1 / (eps0 * eb * fp[zr, pe[k]])) * wv
        assert np.array_equal(o.get_pml(0, 1, s), want_d), s
    assert np.array_equal(got_e, want_e)


def test_set_sz_against_numpy(oracle, tmp_path):
    """set_sz (code/boundary_II.f90:224-276) restated in numpy: only the third
    profile is graded, sigma and kappa - 1 grow as ((pmlzi - i)/(pmlzi - 1))^n
    into the bottom slab and ((i - pmlzf)/(nz - pmlzf))^n into the top one,
    with the REAL(4) literal 1.8 for kappa."""
    p, o, _, _ = _vec_case(oracle, tmp_path)
    k = p.consts
    got = o.get_sz()
    n = p.npml
    want = []
    for eb, r in ((p.eps1, np.array([(p.pmlzi - i) ** n / float(p.pmlzi - 1) ** n for i in range(1, p.pmlzi + 1)])),
                  (p.eps3, np.array([(i - p.pmlzf) ** n / float(p.nz - p.pmlzf) ** n
                                     for i in range(p.pmlzf, p.nz + 1)]))):
        sg = np.zeros((r.size, 3))
        kap = np.ones((r.size, 3))
        sg[:, 2] = math.sqrt(eb) * p.wzpml * r
        kap[:, 2] = 1 + math.sqrt(eb) * k["pmlalfa"] * r
        want += [2 * k["eps0"] * eb * kap + p.dt * sg, 2 * k["eps0"] * eb * kap - p.dt * sg]
    for g, wv in zip(got, want):
        assert g.shape == wv.shape
        assert np.max(np.abs(g - wv)) <= 1e-14 * np.max(np.abs(wv))
    assert k["pmlalfa"] == 1.7999999523162842


def test_upml_h_against_numpy(oracle, tmp_path):
    """UPML_Array_h (code/boundary_II.f90:142-220) restated in numpy, bit for
    bit: B_k = (fm/fp)[(2, 3, 1)[k]] B_prev - ((2 eps / fp) dtq2) curl E,
    H_k decays with profile (3, 1, 2)[k], mu0 in the B-to-H step."""
    p, o, eps, (e_cur, h_prev, _, h_cur0) = _vec_case(oracle, tmp_path)
    rng = np.random.default_rng(6)
    bprev = [rng.standard_normal(o.pml_shape(s)) + 1j * rng.standard_normal(o.pml_shape(s)) for s in (0, 1)]
    o.set_field(o.E_CUR, e_cur)
    o.set_field(o.H_PREV, h_prev)
    o.set_field(o.H_CUR, h_cur0)
    for s in (0, 1):
        o.set_pml(1, 0, s, bprev[s])
    o.op("upml_h")
    got_h = o.get_field(o.H_CUR)
    fpn, fmn, fpx, fmx = o.get_sz()
    mu0 = p.consts["mu0"]
    dtq2 = (p.dt / p.Q) * (p.dt / p.Q)
    E = [e_cur[..., k] for k in range(3)]
    want_h = h_cur0.copy()
    pd, pe = (1, 2, 0), (2, 0, 1)
    for s, (z0, z1, fp, fm, eb) in enumerate(((1, p.pmlzi, fpn, fmn, p.eps1), (p.pmlzf, p.nz, fpx, fmx, p.eps3))):
        want_b = np.empty_like(bprev[s])
        for z in range(z0, z1 + 1):
            zr = z - z0

            def at(k, dz=0, dy=0, dx=0):
                return _sh(E[k], dy=dy, dx=dx)[z + dz]
            c = [((at(2, dy=1) - at(2)) - at(1, dz=1)) + at(1),
                 ((at(0, dz=1) - at(0)) - at(2, dx=1)) + at(2),
                 ((at(1, dx=1) - at(1)) - at(0, dy=1)) + at(0)]
            for k in range(3):
                bold = bprev[s][zr, :, :, k]
                bn = (fm[zr, pd[k]] / fp[zr, pd[k]]) * bold - (((2 * eb) / fp[zr, pd[k]]) * dtq2) * c[k]
                want_b[zr, :, :, k] = bn
                v = (fm[zr, pe[k]] / fp[zr, pe[k]]) * h_prev[z, 1:-1, 1:-1, k]
                wv = fp[zr, k] * bn - fm[zr, k] * bold
                want_h[z, 1:-1, 1:-1, k] = v + (1 / (mu0 * fp[zr, pe[k]])) * wv
        assert np.array_equal(o.get_pml(1, 1, s), want_b), s
    assert np.array_equal(got_h, want_h)


def test_dft_samples_against_numpy(oracle, tmp_path):
    """scattering_fourier (code/dataprocess.f90:109-209) with the sample list
    of init_store_pts_fourier (:793-903): after two samples at steps t1, t2
    every accumulator is dt * (F(t1) e^{i w t1} + F(t2) e^{i w t2}) of its
    point's field component (E for components 1-3, H for 4-6)."""
    p, o, eps, (e1, h1, e2, h2) = _vec_case(oracle, tmp_path)
    fw = np.asarray(p.fw, dtype=np.float64)
    want = {}
    for (e, h), t in (((e1, h1), 7), ((e2, h2), 12)):
        o.set_field(o.E_CUR, e)
        o.set_field(o.H_CUR, h)
        o.op("dft", t)
        for j in (1, 2, 3):
            pto = o.pto(0, j)
            comp, x, y, z = pto[:, 0], pto[:, 1], pto[:, 2], pto[:, 3]
            f = np.where(comp <= 3, e[z, y, x, np.minimum(comp, 3) - 1], h[z, y, x, np.maximum(comp, 4) - 4])
            want[j] = want.get(j, 0) + (p.dt * f)[None, :] * np.exp(1j * fw[:, None] * t)
    for j in (1, 2, 3):
        got = o.fdata(0, j)
        assert got.shape == want[j].shape and got.shape[1] > 0
        assert np.max(np.abs(got - want[j])) <= 1e-14 * np.max(np.abs(want[j])), j
