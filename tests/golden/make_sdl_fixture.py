"""Writes tests/golden/sdl_oracle.npz: the SDL snapshot files that the
oracle's restatement of SDL_output writes for a run of sdl_deck.inputFDTD.dat
(example_1's slab and snapshot plane, 389 steps, 5 outputs), and what the
reference's own reader (IrisFDTD_time_evolution.py, fdtdEMt.setpyplotformat)
returns for each file series.  tests/test_sdl_oracle.py checks the oracle's
writer against both on any machine.

Usage: make_sdl_fixture.py <path of the IrisFDTD-Academic checkout>
"""
import contextlib
import io
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import iris_oracle as O  # noqa: E402

DECK = os.path.join(HERE, "sdl_deck.inputFDTD.dat")


def oracle_snapshots(directory):
    """Run the oracle over the deck and write its snapshot files into directory;
    returns (the files' names in order, the plane shape (ny, nx) per file)."""
    p = O.setparam(DECK)
    q = O.setparam_sdl(DECK)
    o = O.Oracle(p)
    norm = p.Q * p.epump
    names = []
    it, nos = 1, 1
    for t in range(1, p.texit + 1):
        if t >= p.to_fourier and (t == p.to_fourier + p.no_downloads * nos or t == p.texit):
            o.run(it, t - it + 1)
            it = t + 1
            e, h_prev = o.get_field(o.E_CUR), o.get_field(o.H_PREV)
            for name, v in O.sdl_snapshot(nos + 1, e, h_prev, q, p.sdl_plane_on, norm).items():
                O.write_sdl_record(os.path.join(directory, name), v)
                names.append(name[2:])
            nos += 1
    o.close()
    return names, p, q


def main(ref):
    sys.path.insert(0, ref)
    import IrisFDTD_time_evolution as T
    O.build()
    with tempfile.TemporaryDirectory() as d:
        names, p, q = oracle_snapshots(d)
        records = {n: np.frombuffer(open(os.path.join(d, n), "rb").read(), dtype=np.uint8) for n in names}
        # the reader, once per file series (prefix, extension), over the file numbers written
        series = sorted({(n[:n.index("SDL") + 3] + "".join(ch for ch in n[n.index("SDL") + 3:].split(".")[0]
                                                             if not ch.isdigit()), "." + n.split(".")[1])
                         for n in names})
        nx = q.copy_no * (q.xf[1] - q.xi[1] + 1)
        ny = q.zf[1] - q.zi[1] + 1
        out = {"names": np.asarray(names), "nx": nx, "ny": ny}
        for n in names:
            out["rec:" + n] = records[n]
        for prefix, ext in series:
            nums = sorted(int("".join(ch for ch in n[len(prefix):].split(".")[0])) for n in names
                          if n.startswith(prefix) and n.endswith(ext))
            with contextlib.redirect_stdout(io.StringIO()):
                Z = T.fdtdEMt(nums[0], nums[-1] + 1, nx, ny, d + "/", prefix, ext).setpyplotformat()
            out[f"reader:{prefix}{ext}"] = Z
            out[f"first:{prefix}{ext}"] = nums[0]
        np.savez_compressed(os.path.join(HERE, "sdl_oracle.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_sdl_fixture.py <path of the IrisFDTD-Academic checkout>")
    main(sys.argv[1])
