"""Regenerate the committed golden fixtures (run in a tree that has the
reference checkout; the fixtures themselves are what the tests read).

    python tests/golden/make_fixtures.py /path/to/IrisFDTD-Academic

Writes:
* example_1.inputFDTD.dat, example_2.inputFDTD.dat — the two reference input
  decks (example_{1,2}/inputFDTD.dat) re-emitted value for value through this
  project's own writer: the same section headers and the same leading values
  on every line setparam() and setparam_SDL() read, without the reference's
  comments.
* example_1_oracle.npz — three of the CPU oracle's flux blocks for example_1
  at full length (25962 steps): a regression anchor for the oracle itself.
* pins.json — numbers the reference states outright: dt and step count of
  example_1 (irisfdtd_movie.py:25).
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import iris_oracle as O  # noqa: E402


def raw_values(path):
    """The raw (unconverted) values setparam() reads, in file order."""
    p = O.setparam(path)
    b1, b2 = p.box1, p.box2
    return p, [
        ("Mesh options", [[p.i_pol], [p.q_nm], [p.nx], [p.ny], [p.nz], [p.cfl], [p.wzpml_in], [p.pml_taflove],
                          [p.pmlzi], [p.pmlzf]]),
        ("Source options", [[p.plane_wave], [p.tincr_in, p.tdecay_in],
                            [p.epump_in, p.wlpump, p.pump_dt_in, p.def_pulse], [p.tfsf_zi], [p.cosine]]),
        ("Job options", [[p.no_downloads_in, p.output_time_step], [p.texit_fs], [p.hi], list(p.sdl_plane_on)]),
        ("Dielectric constants", [[p.eps1], [p.eps_bbox.real], [p.eps3]]),
        ("Fourier transformation options", [[b1[i], b2[i]] for i in range(6)] +
         [[p.nof], [p.dlamda], [p.lno], [p.to_fourier, p.sample_fourier]]),
        ("Slit Array", [[p.dh], [p.dx]]),
    ] + sdl_values(path, p)


def sdl_values(path, p):
    """The snapshot section setparam_SDL reads (code/sdl.f90:365-400), when the
    deck turns a snapshot plane on."""
    if not any(p.sdl_plane_on):
        return []
    q = O.setparam_sdl(path)
    rows = [[q.copy_flag, q.copy_no], list(q.xi), list(q.xf), list(q.yi), list(q.yf), list(q.zi), list(q.zf),
            [q.module_e]] + [[v] for v in q.field]
    return [("Time evolution options", rows)]


def emit(values, description, out):
    lines = [description, ""]
    for header, rows in values:
        lines.append(f'"{header}"')
        for r in rows:
            lines.append(" ".join(repr(v) if isinstance(v, float) else str(v) for v in r))
        lines.append("")
    with open(out, "w") as fh:
        fh.write("\n".join(lines))


def main(ref):
    pins = {}
    for ex in ("example_1", "example_2"):
        src = os.path.join(ref, ex, "inputFDTD.dat")
        p, vals = raw_values(src)
        out = os.path.join(HERE, f"{ex}.inputFDTD.dat")
        emit(vals, f"{ex} of IrisFDTD-Academic, re-emitted value for value", out)
        q = O.setparam(out)
        assert (q.texit, q.nof, q.hf, q.aix, q.afx) == (p.texit, p.nof, p.hf, p.aix, p.afx)
    pins["example_1"] = {"dt_fs": 0.00770333, "itmax_steps": 25962, "source": "irisfdtd_movie.py:25"}
    with open(os.path.join(HERE, "pins.json"), "w") as fh:
        json.dump(pins, fh, indent=1)
    p = O.setparam(os.path.join(HERE, "example_1.inputFDTD.dat"))
    o = O.Oracle(p)
    J, its = o.run(1, p.texit, max_out=100)
    keep = [0, len(its) // 2, len(its) - 1]
    np.savez_compressed(os.path.join(HERE, "example_1_oracle.npz"), J=J[keep], its=np.asarray(its)[keep])


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_fixtures.py <path of the IrisFDTD-Academic checkout>")
    main(sys.argv[1])
