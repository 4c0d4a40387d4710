"""Writes tests/golden/slit_256x4x768_oracle.npz: the FP64 oracle's flux
spectra for the 256x4x768 slit-array workload (eps 4.0, 80 cells thick,
one 64-cell air slit per period, 16-cell UPML, TF/SF at z = 40, DFT planes
z = 30 and z = 738) over its full 8000 steps, with 24 of its 300
frequencies (every 12th wavelength of the workload's grid); the oracle's
run takes about eleven minutes on 8 cores.  tests/test_gpu_slit.py
compares the GPU engine's FP32 and FP64 spectra with it per spectrum.

Usage: make_slit_fixture.py [threads]
"""
import importlib
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import iris_oracle as O  # noqa: E402

cfg = importlib.import_module("irisfdtd-academic_gb300.configs")
NOF, EVERY = 24, 12


def deck(directory):
    """The workload's deck with the frequency grid thinned (the same first
    wavelength, a step EVERY times longer)."""
    w = cfg.workload(2, nof=NOF)
    lam0 = cfg.LAMBDA0
    return cfg.write_input(os.path.join(directory, "inputFDTD.dat"), w, no_downloads=8,
                           lno=0.75 * lam0, dlamda=EVERY * 0.75 * lam0 / 300), w


def main(threads):
    O.build()
    with tempfile.TemporaryDirectory() as d:
        path, w = deck(d)
        p = O.setparam(path)
        o = O.Oracle(p, threads=threads)
        o.set_eps_inv(cfg.slit_material(w))
        t0 = time.time()
        its = [t for t in range(1, p.texit + 1)
               if t >= p.to_fourier and (t == p.texit or (t - p.to_fourier) % p.no_downloads == 0)]
        J, ito = o.run(1, p.texit, max_out=len(its) + 2)
        print(f"oracle: {p.texit} steps in {time.time() - t0:.1f} s, {len(ito)} output blocks")
        np.savez_compressed(os.path.join(HERE, "slit_256x4x768_oracle.npz"), J=J, its=np.asarray(ito),
                            fw=np.asarray(p.fw), steps=p.texit, nof=p.nof)


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1))
