"""SDL field snapshots of the drop-in main program (code/sdl.f90 SDL_output,
called from code/driver.f90:468-494): file names, the Fortran unformatted
REAL(4) record, the copies, and the values (E of the output step, H of the
step before it, both over q*Epump) against an engine stepped to the same
steps."""
import os
import struct

import numpy as np
import pytest

from helpers import output_steps

pytestmark = pytest.mark.gpu

DECK = """SDL snapshot test deck (1x1x400 slab)

"Mesh options"
2
5.0
1
1
400
0.8
0.09
2
75
325

"Source options"
1
20.0 180.0
1.0 689.0 2.0 4.0
105
0

"Job options"
3 1000
3.0
150
0 1 0

"Dielectric constants"
1.0
9.0
1.0

"Fourier transformation options"
1 1
1 1
1 1
1 1
90 90
320 320
50
5.0
400.0
0 1

"Time evolution options"
1 3         SDL_copy_flag, SDL_copy_no
0 1   0     sxi
0 1   0     sxf
0 1   0     syi
0 1   0     syf
0 75  0     szi
0 325 0     szf
1           E
1           Ex
0           Ey
0           Ez
0           Hx
2           Hy
0           Hz

"Slit Array"
150
0
"""


def read_record(path):
    raw = open(path, "rb").read()
    n = struct.unpack("<i", raw[:4])[0]
    assert struct.unpack("<i", raw[-4:])[0] == n and len(raw) == n + 8
    return np.frombuffer(raw[4:-4], dtype="<f4")


def test_sdl_files(iris, tmp_path):
    d = tmp_path / "run"
    d.mkdir()
    (d / "inputFDTD.dat").write_text(DECK)
    iris.run_input(str(d), iris.FP64)
    p, fw, _ = iris.setparam(str(d / "inputFDTD.dat"))
    its = output_steps(p)
    assert len(its) >= 2
    norm = p.Q * p.epump
    eng = iris.Engine(p, fw)
    it = 1
    for nos, t in enumerate(its, start=1):
        if t - 1 >= it:
            eng.step(it, t - it)
        h_prev = eng.get_plane(iris.H, 2, 1, (1, 1), (75, 325))[:, 0, :]  # [z, comp]
        eng.step(t, 1)
        it = t + 1
        e = eng.get_plane(iris.E, 2, 1, (1, 1), (75, 325))[:, 0, :]
        files = {"E": f"Y_SDL_E{nos}.e", "Ex": f"Y_SDL_R{nos}.e1", "Hy": f"Y_SDL_I{nos}.h2"}
        for f in files.values():
            assert os.path.exists(d / f), f
        want = {"E": np.sqrt(np.sum(np.abs(e) ** 2, axis=1)) / norm, "Ex": e[:, 0].real / norm,
                "Hy": h_prev[:, 1].imag / norm}
        for key, f in files.items():
            v = read_record(d / f).reshape(251, 3)  # Output(1:3 copies, 75:325), first index fastest
            for c in range(3):
                np.testing.assert_allclose(v[:, c], want[key].astype(np.float32), rtol=1e-6, atol=1e-30)
    # the flux files are still written alongside
    assert os.path.exists(d / "1_scatt.dat") or any(n.endswith("_scatt.dat") for n in os.listdir(d))
