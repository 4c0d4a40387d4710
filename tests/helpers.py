"""Shared helpers for the parity tests."""
import importlib
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def iris_mod():
    return importlib.import_module("irisfdtd-academic_gb300")


def rel_err(a, b):
    """Norm-wise relative error max|a-b| / max|b|."""
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    if b.size == 0:
        return 0.0
    den = np.max(np.abs(b))
    if den == 0:
        return float(np.max(np.abs(a)))
    return float(np.max(np.abs(a - b)) / den)


def interior(f, p):
    """Interior cells [1..n] of a [z, y, x, c] field."""
    return f[1:p.nz + 1, 1:p.ny + 1, 1:p.nx + 1]


def oracle_params_from_file(oracle, path, **over):
    p = oracle.setparam(path)
    for k, v in over.items():
        setattr(p, k, v)
    return p


def engine_params_from_oracle(iris, op, precision=0, ak=(0j, 0j, 0j)):
    """iris_params carrying exactly the oracle's derived values."""
    k = op.consts
    p = iris.IrisParams()
    p.i_pol, p.nx, p.ny, p.nz = op.i_pol, op.nx, op.ny, op.nz
    p.pmlzi, p.pmlzf, p.npml, p.pml_taflove = op.pmlzi, op.pmlzf, op.npml, op.pml_taflove
    p.q_nm, p.Q, p.cfl, p.dt, p.wzpml = op.q_nm, op.Q, op.cfl, op.dt, op.wzpml
    p.no_downloads, p.output_time_step, p.texit, p.texit_fs = op.no_downloads, op.output_time_step, op.texit, op.texit_fs
    p.hi, p.hf = op.hi, op.hf
    p.eps1, p.eps3 = op.eps1, op.eps3
    p.eps_bbox_re, p.eps_bbox_im = op.eps_bbox.real, op.eps_bbox.imag
    for i in range(6):
        p.box1[i] = op.box1[i]
        p.box2[i] = op.box2[i]
    p.nof, p.dlamda, p.lno = op.nof, op.dlamda, op.lno
    p.to_fourier, p.sample_fourier = op.to_fourier, op.sample_fourier
    p.plane_wave, p.tfsf_zi, p.tfsf_zf, p.cosine = op.plane_wave, op.tfsf_zi, op.tfsf_zi + 5, op.cosine
    p.epump, p.wlpump, p.pump_dt, p.def_pulse = op.epump, op.wlpump, op.pump_dt, op.def_pulse
    p.gpump, p.zopump, p.tincr, p.tdecay = op.gpump, op.zopump, op.tincr, op.tdecay
    p.gap, p.ratio_angle = 0.0, 1.0
    p.dh, p.dx, p.aix, p.afx = op.dh, op.dx, op.aix, op.afx
    p.pi, p.c0, p.eps0, p.mu0, p.f_abohr = k["pi"], k["c0"], k["eps0"], k["mu0"], k["f_abohr"]
    p.uat, p.f_e, p.pmlalfa = k["uat"], k["f_e"], k["pmlalfa"]
    p.akx_re, p.akx_im = ak[0].real, ak[0].imag
    p.aky_re, p.aky_im = ak[1].real, ak[1].imag
    p.akz_re, p.akz_im = ak[2].real, ak[2].imag
    p.system_model = 0
    p.precision = precision
    return p


def output_steps(p):
    """Output steps of the driver loop (code/driver.f90:455-456)."""
    out, nos = [], 1
    for it in range(1, p.texit + 1):
        if it >= p.to_fourier and (it == p.to_fourier + p.no_downloads * nos or it == p.texit):
            out.append(it)
            nos += 1
    return out


def run_engine_blocks(eng, p, its):
    """Step the engine to each output step and collect the box-1 flux."""
    blocks, it = [], 1
    for t in its:
        eng.step(it, t - it + 1)
        blocks.append(eng.flux(0))
        it = t + 1
    return np.asarray(blocks)
