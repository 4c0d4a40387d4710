"""Regenerate the spectra-file fixtures (run in a tree that has the reference
checkout and this project's library built; the tests read only the output):

    python tests/golden/make_scatt_fixture.py /path/to/IrisFDTD-Academic

Writes, from seeded synthetic fluxes J[block, 6, nof] (4 output blocks, 16
frequencies, magnitudes spread over many decades, a few negative values):

* scatt/1_scatt5.dat, scatt/1_scatt6.dat — the reflection and transmission
  records this project's writer (iris_write_scatt) appends, as
  scattering_fourier_out does (code/dataprocess.f90:279-299);
* scatt_reference.npz — J, and for every output block what the reference's
  own post-processing makes of those two files: its reader
  (IrisFDTD_scattering.py fdtdscatt.load_spectra / get_single_spectra, imported
  from the checkout) gives the wavelength axis x and the spectra, and
  irisfdtd_scatt.py:37-42 normalises them to R and T.
"""
import importlib
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
NOF, NBLOCKS, LNO, DLAMDA = 16, 4, 400.0, 5.0
ITS = (1000, 2000, 3000, 4000)


def synthetic_flux(seed=7):
    r = np.random.default_rng(seed)
    mag = 10.0 ** r.uniform(-9, 3, size=(NBLOCKS, 6, NOF))
    sign = np.where(r.random((NBLOCKS, 6, NOF)) < 0.1, -1.0, 1.0)
    J = sign * mag
    J[:, 4:6, :] = np.abs(J[:, 4:6, :])  # reflected and transmitted power positive, as in a physical run
    return J


def main(ref):
    sys.path.insert(0, ROOT)
    iris = importlib.import_module("irisfdtd-academic_gb300")
    sys.path.insert(0, ref)
    import IrisFDTD_scattering as scatt  # the reference's reader

    J = synthetic_flux()
    tmp = tempfile.mkdtemp()
    for b in range(NBLOCKS):
        iris.write_scatt(tmp, 0, ITS[b], J[b])
    out = os.path.join(HERE, "scatt")
    os.makedirs(out, exist_ok=True)
    for f in ("1_scatt5.dat", "1_scatt6.dat"):
        shutil.copy(os.path.join(tmp, f), os.path.join(out, f))
    path = tmp + "/"
    r = scatt.fdtdscatt(path, "1_scatt5.dat", "wavelength_list.dat", NOF, NBLOCKS - 1, DLAMDA, LNO)
    t = scatt.fdtdscatt(path, "1_scatt6.dat", "wavelength_list.dat", NOF, NBLOCKS - 1, DLAMDA, LNO)
    ref_r, ref_t = r.load_spectra(), t.load_spectra()
    xs, Rs, Ts = [], [], []
    for it in range(NBLOCKS):
        x, y = r.get_single_spectra(ref_r, it)
        xx, yy = t.get_single_spectra(ref_t, it)
        total = y + yy  # irisfdtd_scatt.py:37-42
        xs.append(x)
        Rs.append(y / total)
        Ts.append(yy / total)
        assert np.array_equal(x, xx)
    np.savez(os.path.join(HERE, "scatt_reference.npz"), J=J, its=np.array(ITS), x=np.array(xs), R=np.array(Rs),
             T=np.array(Ts), nof=NOF, lno=LNO, dlamda=DLAMDA)
    shutil.rmtree(tmp)


if __name__ == "__main__":
    main(sys.argv[1])
