"""The oracle's restatement of the SDL field snapshots (SDL_output and
setparam_SDL of code/sdl.f90, the driver's calls at code/driver.f90:468-494)
pinned to the reference's own reader.

tests/golden/sdl_oracle.npz (written by tests/golden/make_sdl_fixture.py)
holds the snapshot files the oracle wrote for sdl_deck.inputFDTD.dat
(example_1's slab and snapshot plane, 389 steps) and the matrices that the
reference's reader, IrisFDTD_time_evolution.py fdtdEMt.setpyplotformat,
returned for them.  The oracle writes the same files again here, byte for
byte, and the reader's matrices are the planes of the oracle's fields in
the orientation the reference's movie script expects (irisfdtd_movie.py:29:
nx = copies x the plane's x extent, nz = its z extent), numbered from 2
(the driver passes nos + 1).  The engine's own files are checked against
this restatement on the GPU (tests/test_gpu_sdl.py).
"""
import os
import sys

import numpy as np

from conftest import golden

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_sdl_fixture as F  # noqa: E402


def test_oracle_writes_the_fixture_files(oracle, tmp_path):
    names, p, q = F.oracle_snapshots(str(tmp_path))
    d = np.load(golden("sdl_oracle.npz"))
    assert names == [str(n) for n in d["names"]]
    for n in names:
        assert open(tmp_path / n, "rb").read() == d["rec:" + n].tobytes(), n


def test_reference_reader_sees_the_oracle_planes(oracle):
    d = np.load(golden("sdl_oracle.npz"))
    nx, ny = int(d["nx"]), int(d["ny"])
    names = [str(n) for n in d["names"]]
    assert (nx, ny) == (3, 251)
    for key in d.files:
        if not key.startswith("reader:"):
            continue
        series = key[len("reader:"):]
        prefix, ext = series.rsplit(".", 1)
        first = int(d["first:" + series])
        assert first == 2  # the first output step's files carry nos + 1 = 2
        Z = d[key]
        files = [n for n in names if n.startswith(prefix) and n.endswith("." + ext)
                 and n[len(prefix):-len(ext) - 1].isdigit()]
        assert len(files) == Z.shape[0] - 1  # the reader appends one empty matrix
        for n in files:
            k = int(n[len(prefix):-len(ext) - 1]) - first
            raw = d["rec:" + n].tobytes()
            assert np.frombuffer(raw[:4], "<i4")[0] == nx * ny * 4 == np.frombuffer(raw[-4:], "<i4")[0]
            vals = np.frombuffer(raw[4:-4], "<f4").reshape(ny, nx)
            assert np.array_equal(Z[k], vals.astype(np.float64)), n


def test_snapshot_values_from_the_fields(oracle, tmp_path):
    """The modulus file of the first output step against |E| computed here
    from the oracle's field at that step: the plane y = 1, z = 75..325,
    copied three times along x, over q*Epump, REAL(4) as the reference
    rounds it (real() before the division, real() again on writing)."""
    p = oracle.setparam(F.DECK)
    q = oracle.setparam_sdl(F.DECK)
    assert (q.copy_flag, q.copy_no, q.module_e, q.field) == (1, 3, 1, (1, 2, 0, 0, 1, 0))
    o = oracle.Oracle(p)
    o.run(1, p.no_downloads)
    e = o.get_field(o.E_CUR)[75:326, 1, 1, :]
    want = np.sqrt(np.sum(np.abs(e) ** 2, axis=1)).astype(np.float32).astype(np.float64) / (p.Q * p.epump)
    d = np.load(golden("sdl_oracle.npz"))
    Z = d["reader:Y_SDL_E.e"][0]
    for c in range(3):
        np.testing.assert_array_equal(Z[:, c], want.astype(np.float32).astype(np.float64))
    # Hy's file takes its mode from SDLField(2) (Ey's entry, 2: imaginary part)
    h = o.get_field(o.H_PREV)[75:326, 1, 1, 1]
    Zh = d["reader:Y_SDL_I.h2"][0]
    np.testing.assert_array_equal(Zh[:, 0], (h.imag.astype(np.float32).astype(np.float64) / (p.Q * p.epump))
                                  .astype(np.float32).astype(np.float64))
