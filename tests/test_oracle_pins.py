"""Pins of the CPU oracle against what the reference states outright.

The reference ships no tests.  Its checkable numbers are the step size and
step count of example_1 (irisfdtd_movie.py:25) and the analytic film spectrum
it writes next to every run (code/common.f90:104-131, the comparison shown in
example_1/README.md:15).
"""
import json

import numpy as np
import pytest

from conftest import golden


def test_example1_dt_and_step_count(oracle):
    pins = json.load(open(golden("pins.json")))["example_1"]
    p = oracle.setparam(golden("example_1.inputFDTD.dat"))
    k = p.consts
    # log.dat prints dt with F15.8 (code/files.f90:144)
    assert f"{p.dt * k['uat']:.8f}" == f"{pins['dt_fs']:.8f}"
    assert p.texit == pins["itmax_steps"]
    # no_downloads=50 becomes an interval of int(25962/50) = 519 steps
    assert p.no_downloads == 519


def test_struct_limit(oracle):
    # slit limits for the two examples and the slit workload
    assert oracle.struct_limit(1, 0) == (1, 0)      # example_1: empty slit
    assert oracle.struct_limit(100, 20) == (41, 60)  # example_2
    assert oracle.struct_limit(256, 64) == (97, 160)
    assert oracle.struct_limit(7, 3) == (3, 5)
    assert oracle.struct_limit(8, 3) == (3, 5)


def test_single_precision_literals(oracle):
    k = oracle.physconsts(True)
    assert k["pi"] == 3.1415927410125732
    assert k["c0"] == 137.03599548339844
    assert k["f_abohr"] == 18.897260665893555
    assert k["pmlalfa"] == 1.7999999523162842
    # cos(pi_f/2) is not zero: the incident field depends on x at 1e-8
    assert abs(np.cos(k["pi"] / 2.0) + 4.371139000186243e-08) < 1e-20


@pytest.fixture(scope="module")
def ex1_run(oracle):
    p = oracle.setparam(golden("example_1.inputFDTD.dat"))
    o = oracle.Oracle(p)
    J, its = o.run(1, p.texit, max_out=100)
    return p, J, its


def test_example1_against_analytic_film(oracle, ex1_run):
    """T/R of the 750 nm eps=9 film vs the analytic transfer-matrix result the
    reference writes (code/common.f90:104-131): agreement at the level of grid
    dispersion (5 nm cells)."""
    p, J, its = ex1_run
    R, T = oracle.tr_normalise(J[-1, 4], J[-1, 5])
    lp, Ra, Ta = oracle.film_spectrum(p)
    assert np.allclose(R + T, 1.0)
    band = (lp >= 900) & (lp <= 2800)
    assert np.max(np.abs(R - Ra)[band]) < 1e-2
    assert np.mean(np.abs(R - Ra)[band]) < 5e-3
    # shorter wavelengths see more grid dispersion (7.5 cells per wavelength in the film at 400 nm)
    assert np.max(np.abs(R - Ra)[lp >= 400]) < 7e-2


def test_example1_output_schedule(ex1_run):
    p, J, its = ex1_run
    assert len(its) == 51  # 50 intervals of 519 steps plus the last step
    assert its[0] == 519 and its[-2] == 25950 and its[-1] == 25962


def test_example1_regression_anchor(ex1_run):
    p, J, its = ex1_run
    g = np.load(golden("example_1_oracle.npz"))
    keep = [0, len(its) // 2, len(its) - 1]
    assert list(np.asarray(its)[keep]) == list(g["its"])
    assert np.array_equal(J[keep], g["J"])


def test_vacuum_has_no_reflection(oracle, tmp_path):
    """eps_bbox = 1 everywhere: the reflection plane lies in the scattered-field
    region and sees only the leakage of the analytic TF/SF source, which is not
    matched to the grid's numerical dispersion (about 1% of the transmitted
    flux for the 10-cells-per-wavelength pulse of the benchmark workloads)."""
    import importlib
    cfg = importlib.import_module("irisfdtd-academic_gb300.configs")
    w = cfg.Workload("vac", 1, 1, 400, 16, 385, 200, 40, 1.0, 0, 60, (1, 1, 1, 1, 40, 360), 40, 3000)
    path = cfg.write_input(str(tmp_path / "inputFDTD.dat"), w)
    p = oracle.setparam(path)
    o = oracle.Oracle(p)
    J, its = o.run(1, p.texit, max_out=10)
    j5, j6 = J[-1, 4], J[-1, 5]
    assert np.max(np.abs(j5)) < 2e-2 * np.max(np.abs(j6))
    assert np.all(j6 > 0)
