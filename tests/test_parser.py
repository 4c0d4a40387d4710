"""The product's setparam (C++, iris_setparam) against the oracle's restatement."""
import ctypes
import math

import numpy as np
import pytest

from conftest import golden


def _compare(iris, oracle, path):
    p, fw, desc = iris.setparam(path)
    q = oracle.setparam(path)
    k = q.consts
    ints = ["i_pol", "nx", "ny", "nz", "pmlzi", "pmlzf", "npml", "no_downloads", "texit", "hi", "hf", "nof",
            "to_fourier", "sample_fourier", "plane_wave", "tfsf_zi", "cosine", "dh", "dx", "aix", "afx"]
    for n in ints:
        assert getattr(p, n) == getattr(q, n), n
    reals = {"Q": q.Q, "dt": q.dt, "wzpml": q.wzpml, "eps1": q.eps1, "eps3": q.eps3, "dlamda": q.dlamda,
             "lno": q.lno, "epump": q.epump, "pump_dt": q.pump_dt, "gpump": q.gpump, "zopump": q.zopump,
             "tincr": q.tincr, "tdecay": q.tdecay, "pi": k["pi"], "c0": k["c0"], "eps0": k["eps0"],
             "mu0": k["mu0"], "f_abohr": k["f_abohr"], "pmlalfa": k["pmlalfa"]}
    for n, v in reals.items():
        assert getattr(p, n) == v, n  # bit-identical
    assert p.eps_bbox_re == q.eps_bbox.real
    assert list(p.box1) == list(q.box1) and list(p.box2) == list(q.box2)
    assert p.tfsf_zf == q.tfsf_zi + 5
    assert np.array_equal(fw, np.asarray(q.fw))
    return p, desc


@pytest.mark.parametrize("name", ["example_1", "example_2"])
def test_examples(iris, oracle, name):
    p, desc = _compare(iris, oracle, golden(f"{name}.inputFDTD.dat"))
    assert desc.startswith(name)


@pytest.mark.parametrize("n", [1, 2, 3, 5])
def test_workloads(iris, oracle, tmp_path, n):
    cfg = __import__("importlib").import_module("irisfdtd-academic_gb300.configs")
    w = cfg.workload(n)
    path = cfg.write_input(str(tmp_path / "inputFDTD.dat"), w)
    p, _ = _compare(iris, oracle, path)
    assert p.texit == w.nsteps
    # Courant number 0.5 and 60-step pulse width = 7.5 cells
    assert math.isclose(p.c0 * p.dt / p.Q, 0.5, rel_tol=1e-12)
    assert math.isclose(p.gpump, 7.5, rel_tol=1e-6)


def test_single_literal_switch(iris, oracle):
    p1, _, _ = iris.setparam(golden("example_1.inputFDTD.dat"), single_literals=True)
    p2, _, _ = iris.setparam(golden("example_1.inputFDTD.dat"), single_literals=False)
    q2 = oracle.setparam(golden("example_1.inputFDTD.dat"), single_literals=False)
    assert p2.dt == q2.dt and p2.c0 == 137.036
    assert p1.dt != p2.dt
    assert p1.texit == p2.texit == 25962


def test_missing_section_is_an_error(iris, tmp_path):
    src = open(golden("example_1.inputFDTD.dat")).read()
    bad = tmp_path / "inputFDTD.dat"
    bad.write_text(src.replace('"Source options"', '"Nothing here"'))
    with pytest.raises(iris.IrisError) as e:
        iris.setparam(str(bad))
    assert e.value.code == -4


def test_garbled_values_are_an_error(iris, tmp_path):
    src = open(golden("example_1.inputFDTD.dat")).read().splitlines()
    i = src.index('"Mesh options"')
    src[i + 3] = "one"  # ixmax
    bad = tmp_path / "inputFDTD.dat"
    bad.write_text("\n".join(src))
    with pytest.raises(iris.IrisError) as e:
        iris.setparam(str(bad))
    assert e.value.code == -4


def test_truncated_file_is_an_error(iris, tmp_path):
    src = open(golden("example_1.inputFDTD.dat")).read()
    bad = tmp_path / "inputFDTD.dat"
    bad.write_text(src[: src.index('"Dielectric constants"') + 30])
    with pytest.raises(iris.IrisError):
        iris.setparam(str(bad))


def test_list_directed_details(iris, oracle, tmp_path):
    """Tabs, commas, continuation over records, D exponents, parenthesised complex."""
    src = open(golden("example_1.inputFDTD.dat")).read().splitlines()
    i = src.index('"Dielectric constants"')
    src[i + 2] = "(9.0d0, 0.0)  eps_bbox as a complex constant"
    j = src.index('"Job options"')
    src[j + 1] = "50,\t1000 , comment"
    src[j + 2] = "2.0D2"
    bad = tmp_path / "inputFDTD.dat"
    bad.write_text("\n".join(src))
    _compare(iris, oracle, str(bad))


def _loop_deck(tmp_path, name, header):
    body = open(golden("example_1.inputFDTD.dat")).read().split("\n", 1)[1]  # without the description line
    d = tmp_path / name
    d.mkdir()
    (d / "inputFDTD.dat").write_text("<<LOOP>>\n" + header + body)
    return d


def test_loop_mode_header(iris, tmp_path):
    """program.f90:36-57: after <<LOOP>> come io_main, if_main and delta_x/y/z;
    do i = io_main, if_main runs no iteration when io_main > if_main (no
    engine, no files), and a header that is not numbers is a parse error."""
    d = _loop_deck(tmp_path, "empty", "3\n2\n0.0\n0.0\n0.0\n")
    iris.run_input(str(d), iris.FP64)
    assert not (d / "log.dat").exists()
    bad = _loop_deck(tmp_path, "bad", "three\n2\n")
    with pytest.raises(iris.IrisError) as e:
        iris.run_input(str(bad), iris.FP64)
    assert e.value.code == -4
    # setparam's section scan still finds every section after the loop header
    ok = _loop_deck(tmp_path, "one", "1\n1\n0.0\n0.0\n0.0\n")
    p, fw, desc = iris.setparam(str(ok / "inputFDTD.dat"))
    q, _, _ = iris.setparam(golden("example_1.inputFDTD.dat"))
    assert (p.nx, p.ny, p.nz, p.texit, p.nof) == (q.nx, q.ny, q.nz, q.texit, q.nof)
