"""SDL field snapshots of the drop-in main program (iris_run_input) against
the oracle's restatement of SDL_output (code/sdl.f90:68-483, the driver's
calls at code/driver.f90:468-494), which tests/test_sdl_oracle.py pins to
the reference's own reader.

Every snapshot file the engine writes must be one the oracle writes (same
names: orientation, layer, mode suffix, file number nos + 1, extension)
with the same REAL(4) record, from the oracle's own run of the same deck: E
of the output step and H of the step before it, over q*Epump.  Tolerance:
one REAL(4) rounding step of the file's largest value plus 1e-12 of the
incident amplitude (the FP64 fields agree to ~1e-15 of it and can straddle
a rounding boundary).  Cases: example_1's slab with its y plane copied three
times (E modulus, Ex real, Ey imaginary, Hy with the mode of Ey's entry), and
a 3D cell with x, y and z planes, two extra z layers, copies on both axes of
the z planes, the |H| modulus and the other modes.
"""
import os
import struct

import numpy as np
import pytest

from conftest import golden
from helpers import output_steps

pytestmark = pytest.mark.gpu
THREADS = max(1, min(16, os.cpu_count() or 1))

DECK_3D = """SDL snapshot deck: 3D cell, three planes, extra z layers

"Mesh options"
2
5.0
10
8
48
0.8
0.09
2
6
43

"Source options"
1
20.0 180.0
1.0 200.0 1.0 4.0
10
0

"Job options"
4 1000
1.0
20
1 1 1

"Dielectric constants"
1.0
4.0
1.0

"Fourier transformation options"
1 1
10 10
1 1
8 8
8 8
40 40
8
5.0
150.0
0 1

"Time evolution options"
1 2         SDL_copy_flag, SDL_copy_no
3 1   1     xi
3 10  10    xf
1 2   1     yi
8 2   8     yf
5 5   20    zi
40 40 20    zf
2           |H|
3           Ex
0           Ey
4           Ez
1           Hx
0           Hy
1           Hz

"Extra parameters-SDLextended"
1 1 2
0
0
0
7

"Slit Array"
10
0
"""


def read_record(path):
    raw = open(path, "rb").read()
    n = struct.unpack("<i", raw[:4])[0]
    assert struct.unpack("<i", raw[-4:])[0] == n and len(raw) == n + 8
    return np.frombuffer(raw[4:-4], dtype="<f4")


def oracle_files(oracle, path):
    p = oracle.setparam(path)
    q = oracle.setparam_sdl(path)
    o = oracle.Oracle(p, threads=THREADS)
    norm = p.Q * p.epump
    out, it = {}, 1
    for nos, t in enumerate(output_steps(p), start=1):
        o.run(it, t - it + 1)
        it = t + 1
        snap = oracle.sdl_snapshot(nos + 1, o.get_field(o.E_CUR), o.get_field(o.H_PREV), q, p.sdl_plane_on, norm)
        out.update({k[2:]: v for k, v in snap.items()})
    return out


@pytest.mark.parametrize("deck", ["example_1_plane", "3d_planes"])
def test_sdl_files_against_oracle(iris, oracle, tmp_path, deck):
    d = tmp_path / "run"
    d.mkdir()
    if deck == "example_1_plane":
        (d / "inputFDTD.dat").write_text(open(golden("sdl_deck.inputFDTD.dat")).read())
    else:
        (d / "inputFDTD.dat").write_text(DECK_3D)
    iris.run_input(str(d), iris.FP64)
    want = oracle_files(oracle, str(d / "inputFDTD.dat"))
    assert want
    got = sorted(n for n in os.listdir(d) if "_SDL" in n)
    assert got == sorted(want), (got, sorted(want))
    for n, v in want.items():
        g = read_record(d / n).astype(np.float64)
        assert g.shape == v.shape, n
        # the values are over q*Epump, so the incident field is O(1): one REAL(4)
        # rounding step of the file's largest value, plus the FP64 modes' 1e-12
        # (components at the roundoff floor, such as Ez here, differ there)
        err = np.max(np.abs(g - v))
        assert err <= 2.0 ** -22 * np.max(np.abs(v)) + 1e-12, (n, err)
    # the 3D deck reaches every plane orientation, both z layers and the copies on both axes
    if deck == "3d_planes":
        assert any(n.startswith("X_SDL3layer") for n in got) and any(n.startswith("Y_SDL2layer") for n in got)
        assert any(n.startswith("Z_SDL20layer") for n in got) and any(n.startswith("Z_SDL27layer") for n in got)
        assert any(n.startswith("Z_SDL20layer_H") for n in got)
        z = read_record(d / [n for n in got if n.startswith("Z_SDL20layer_H")][0])
        assert z.size == (2 * 10) * (2 * 8)
