"""The drop-in main program end to end: iris_run_input on the reference's own
example decks against the oracle's run of the same deck.

iris_run_input reads dir/inputFDTD.dat, steps the engine and writes, every
no_downloads steps and at the last step, one block per output step to
<box>_scatt1..6.dat (the six faces' fluxes) and <box>_scatt.dat (their sum),
as scattering_fourier_out appends them (code/dataprocess.f90:279-299,
called from code/driver.f90:455-466), plus log.dat and the analytic film
spectrum dielectric_layer_spectra.dat (code/common.f90:104-131).  The blocks
are read back from the files (17 significant digits: the doubles round-trip
exactly) and compared with the oracle's flux blocks at the same steps within
1e-12 in FP64; log.dat's step size and step count with the numbers the
reference quotes for example_1 (irisfdtd_movie.py:25); the deck's snapshot
plane gives one file per output step, numbered as the movie script expects.

<<LOOP>> mode (code/program.f90:36-57) runs main() once per index with the
same input; the scatt files are opened for appending, so a two-index deck
leaves every block twice, the second run's equal to the first's.
"""
import json
import os
import shutil

import numpy as np
import pytest

from conftest import golden
from helpers import output_steps, rel_err

pytestmark = pytest.mark.gpu
THREADS = max(1, min(16, os.cpu_count() or 1))
TOL = 1e-12


def read_blocks(path, nof):
    """(steps, values [block, nof]) of a <box>_scatt*.dat file."""
    its, vals = [], []
    with open(path) as fh:
        for line in fh:
            v = line.split()
            if not v:
                continue
            if v[0] == "#":
                its.append(int(v[1]))
            else:
                vals.append(float(v[0]))
    a = np.asarray(vals)
    assert a.size == len(its) * nof, (path, a.size, len(its))
    return its, a.reshape(len(its), nof)


@pytest.fixture(scope="module")
def example1_oracle(oracle):
    op = oracle.setparam(golden("example_1.inputFDTD.dat"))
    o = oracle.Oracle(op, threads=THREADS)
    its = output_steps(op)
    Jo, ito = o.run(1, op.texit, max_out=len(its) + 1)
    assert ito == its
    lp, R, T = oracle.film_spectrum(op)
    return op, its, Jo, (lp, R, T)


def check_scatt(d, op, its, Jo, repeats=1):
    for j in range(1, 7):
        fits, v = read_blocks(os.path.join(d, f"1_scatt{j}.dat"), op.nof)
        assert fits == its * repeats, j
        for r in range(repeats):
            blk = v[r * len(its):(r + 1) * len(its)]
            assert rel_err(blk, Jo[:, j - 1]) <= TOL, (j, r)
            assert rel_err(blk[-1], Jo[-1, j - 1]) <= TOL, (j, r)
            if r:
                assert np.array_equal(blk, v[:len(its)]), j
    tits, tot = read_blocks(os.path.join(d, "1_scatt.dat"), op.nof)
    assert tits == its * repeats
    assert rel_err(tot[:len(its)], Jo.sum(axis=1)) <= TOL
    # one box: no second box's files (code/driver.f90:463)
    assert not os.path.exists(os.path.join(d, "2_scatt1.dat"))


def test_run_input_example1_against_oracle(iris, example1_oracle, tmp_path, capfd):
    op, its, Jo, (lp, R, T) = example1_oracle
    shutil.copy(golden("example_1.inputFDTD.dat"), tmp_path / "inputFDTD.dat")
    iris.run_input(str(tmp_path), iris.FP64)
    check_scatt(str(tmp_path), op, its, Jo)
    # the screen progress of code/driver.f90:339-354: one block each time a
    # multiple of OUTPUT_TIME_STEP (1000 here) was passed, at the output steps
    out = capfd.readouterr().out.splitlines()
    steps = [int(ln.split()[1]) for ln in out if ln.strip().startswith("Iteration ") and " of %d" % op.texit in ln]
    assert len(steps) == op.texit // op.output_time_step
    assert steps == sorted(steps) and all(s in its for s in steps)
    assert sum(1 for ln in out if ln.strip().startswith("Iteration/second = ")) == len(steps)
    assert sum(1 for ln in out if ln.strip().startswith("Completed ")) == len(steps)
    # log.dat: the step size and step count the reference quotes for example_1
    pins = json.load(open(golden("pins.json")))
    log = open(tmp_path / "log.dat").read().splitlines()
    dt = [ln for ln in log if ln.startswith("# dt(fs)=")]
    nit = [ln for ln in log if ln.startswith("# Iteration max. number =")]
    assert len(dt) == 1 and len(nit) == 1
    assert abs(float(dt[0].split("=")[1]) - pins["example_1"]["dt_fs"]) < 5e-9
    assert int(nit[0].split("=")[1].split()[0]) == pins["example_1"]["itmax_steps"]
    assert log[-1].strip() == "...done! status=0"
    # example_1's snapshot plane (y = 1, z = 75..325, copied 300 times, |E|): one
    # file per output step, numbered from 2 as the movie script reads them
    # (irisfdtd_movie.py:21-31); their values are checked in tests/test_gpu_sdl.py
    snaps = sorted(int(n[len("Y_SDL_E"):-2]) for n in os.listdir(tmp_path) if n.startswith("Y_SDL_E"))
    assert snaps == list(range(2, len(its) + 2))
    assert os.path.getsize(tmp_path / "Y_SDL_E2.e") == 300 * 251 * 4 + 8
    # the analytic film spectrum written next to every run
    f = np.loadtxt(tmp_path / "dielectric_layer_spectra.dat")
    assert f.shape == (op.nof, 3)
    assert rel_err(f[:, 0], lp) <= TOL and rel_err(f[:, 1], R) <= 1e-11 and rel_err(f[:, 2], T) <= 1e-11


def test_run_input_loop_two_indices(iris, example1_oracle, tmp_path):
    op, its, Jo, _ = example1_oracle
    body = open(golden("example_1.inputFDTD.dat")).read().split("\n", 1)[1]  # no description line in loop mode
    (tmp_path / "inputFDTD.dat").write_text("<<LOOP>>\n1\n2\n0.0\n0.0\n0.0\n" + body)
    iris.run_input(str(tmp_path), iris.FP64)
    check_scatt(str(tmp_path), op, its, Jo, repeats=2)
    log = open(tmp_path / "log.dat").read().splitlines()
    # log.dat is replaced by every main(i) and carries an empty description (code/main.f90:108-115)
    assert log[0].rstrip() == " Description     :"
    assert log[-1].strip() == "...done! status=0"


def test_run_input_example2_fp32_tr(iris, oracle, tmp_path):
    """The slit-array example in FP32 through the drop-in program (the default
    stepping, the persistent kernel on this grid; the tensor-core DFT and its
    flux read): T/R of every output block
    within 1e-4 of the FP64 oracle, steps trimmed to 6000."""
    src = open(golden("example_2.inputFDTD.dat")).read()
    d = tmp_path / "ex2"
    d.mkdir()
    (d / "inputFDTD.dat").write_text(src)
    op = oracle.setparam(str(d / "inputFDTD.dat"))
    steps = 6000
    # the step count enters through itmax (fs): (steps + 0.5) dt, as the workload decks set it
    lines = src.split("\n")
    k = lines.index('"Job options"')
    lines[k + 2] = repr(float((steps + 0.5) * op.dt * op.consts["uat"]))
    (d / "inputFDTD.dat").write_text("\n".join(lines))
    op = oracle.setparam(str(d / "inputFDTD.dat"))
    assert op.texit == steps
    iris.run_input(str(d), iris.FP32)
    o = oracle.Oracle(op, threads=THREADS)
    its = output_steps(op)
    Jo, ito = o.run(1, op.texit, max_out=len(its) + 1)
    assert ito == its
    _, j5 = read_blocks(str(d / "1_scatt5.dat"), op.nof)
    _, j6 = read_blocks(str(d / "1_scatt6.dat"), op.nof)
    R, T = iris.tr_normalise(j5[-1], j6[-1])
    Ro, To = oracle.tr_normalise(Jo[-1, 4], Jo[-1, 5])
    assert max(np.max(np.abs(R - Ro)), np.max(np.abs(T - To))) <= 1e-4
