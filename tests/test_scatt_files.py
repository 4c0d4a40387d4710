"""The spectra files and their post-processing, on the CPU: the records
iris_write_scatt appends (scattering_fourier_out, code/dataprocess.f90:279-299)
and the T/R normalisation (irisfdtd_scatt.py:37-42) with the wavelength axis
(IrisFDTD_scattering.py:74-99) against fixtures that the reference's own
Python reader made from the same records (tests/golden/make_scatt_fixture.py)."""
import os

import numpy as np

from conftest import golden


def fixture():
    return np.load(golden("scatt_reference.npz"))


def write_all(iris, d, g):
    for b, it in enumerate(g["its"]):
        iris.write_scatt(str(d), 0, int(it), g["J"][b])


def test_writer_records_byte_for_byte(iris, tmp_path):
    g = fixture()
    write_all(iris, tmp_path, g)
    for f in ("1_scatt5.dat", "1_scatt6.dat"):
        with open(golden(os.path.join("scatt", f)), "rb") as a, open(tmp_path / f, "rb") as b:
            assert a.read() == b.read(), f


def test_records_round_trip_every_face_and_the_sum(iris, tmp_path):
    g = fixture()
    J, nof = g["J"], int(g["nof"])
    write_all(iris, tmp_path, g)
    for j in range(6):
        blocks = iris.read_scatt(str(tmp_path / f"1_scatt{j + 1}.dat"), nof)
        assert np.array_equal(blocks, J[:, j, :])  # 17 significant digits: doubles survive exactly
    s = J[:, 0, :]
    for j in range(1, 6):
        s = s + J[:, j, :]  # the writer's order of summation
    assert np.array_equal(iris.read_scatt(str(tmp_path / "1_scatt.dat"), nof), s)
    # the step numbers of the '# it' lines
    its = [int(line.split()[1]) for line in open(tmp_path / "1_scatt5.dat") if line.split()[0] == "#"]
    assert its == list(g["its"])


def test_tr_and_wavelength_axis_match_the_reference_reader(iris):
    g = fixture()
    nof = int(g["nof"])
    r5 = iris.read_scatt(golden(os.path.join("scatt", "1_scatt5.dat")), nof)
    r6 = iris.read_scatt(golden(os.path.join("scatt", "1_scatt6.dat")), nof)
    x = iris.wavelength_axis(float(g["lno"]), float(g["dlamda"]), nof)
    for it in range(len(g["its"])):
        R, T = iris.tr_normalise(r5[it], r6[it])
        assert np.array_equal(x, g["x"][it])
        assert np.array_equal(R, g["R"][it]) and np.array_equal(T, g["T"][it])


def test_oracle_tr_matches_the_reference_reader(iris, oracle):
    g = fixture()
    nof = int(g["nof"])
    r5 = iris.read_scatt(golden(os.path.join("scatt", "1_scatt5.dat")), nof)
    r6 = iris.read_scatt(golden(os.path.join("scatt", "1_scatt6.dat")), nof)
    for it in range(len(g["its"])):
        R, T = oracle.tr_normalise(r5[it], r6[it])
        assert np.array_equal(R, g["R"][it]) and np.array_equal(T, g["T"][it])
    assert np.array_equal(oracle.wavelength_axis(float(g["lno"]), float(g["dlamda"]), nof), g["x"][0])


def test_writer_rejects_bad_arguments(iris, tmp_path):
    import pytest
    with pytest.raises(ValueError):
        iris.write_scatt(str(tmp_path), 0, 1, np.zeros((5, 4)))
    with pytest.raises(iris.IrisError):
        iris.write_scatt(str(tmp_path / "no_such_dir"), 0, 1, np.zeros((6, 4)))
