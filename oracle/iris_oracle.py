"""TEST INFRASTRUCTURE ONLY — the parity oracle for the GB300 FDTD engine.

Python half of the CPU FP64 restatement of IrisFDTD-Academic's hot path:

* ``physconsts`` — code/physconst.f90:31-53.  Literals written without a
  ``d0`` suffix are default REAL (single precision) in Fortran and are widened
  to double only after rounding; ``single_literals=True`` (the default, the
  standard-Fortran reading) reproduces the step size and step count the
  reference quotes for example_1 (irisfdtd_movie.py:25: dt = 0.00770333 fs,
  25962 steps).
* ``setparam`` — code/files.f90:39-344: the section-scanning, list-directed
  reader of ``inputFDTD.dat`` plus the unit conversions.
* ``struct_limit`` — code/files.f90:385-409.
* ``Oracle`` — ctypes wrapper of ``iris_oracle.cpp`` (the numerics: Yee E/H,
  UPML, Bloch, TF/SF, on-the-fly DFT, flux).
* ``tr_normalise``, ``wavelength_axis`` — irisfdtd_scatt.py:37-42 and
  IrisFDTD_scattering.py:111,143, checked bit for bit against fixtures the
  reference's own reader produced (tests/test_scatt_files.py).
* ``setparam_sdl``, ``sdl_output``, ``sdl_snapshot`` — the field snapshots:
  setparam_SDL (code/sdl.f90:365-400) with the SDLextended layers
  (code/files.f90:291-320), SDL_output (code/sdl.f90:68-483) and the driver's
  calls (code/driver.f90:468-494), from the oracle's own field arrays; the
  files it writes are read back by the reference's reader in
  tests/test_sdl_oracle.py.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, as the checker or as the timed CPU baseline.  The product never
imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")


def _f32(x: float) -> float:
    return float(np.float32(x))


def physconsts(single_literals: bool = True) -> dict:
    """code/physconst.f90:31-53 (and the other default-REAL literals the hot path reads)."""
    r = _f32 if single_literals else float
    pi = r(3.14159265358979323846)
    c0 = r(137.0360)
    if single_literals:
        # 10/0.529177249: integer/REAL -> REAL division, rounded to single
        f_abohr = float(np.float32(10) / np.float32(0.529177249))
    else:
        f_abohr = 10 / 0.529177249
    eps0 = 1.0 / (4.0 * pi)
    mu0 = 1.0 / (eps0 * (c0 * c0))
    return dict(
        pi=pi, c0=c0, eps0=eps0, mu0=mu0, f_abohr=f_abohr,
        uat=r(24.188843265e-3),
        f_e=r(514.2208281e9),
        one_e_m5=r(1e-5),            # files.f90:281
        pmlalfa=r(1.8),              # boundary_II.f90:233
    )


# ---------------------------------------------------------------------------
# list-directed reading (Fortran ``read(unit,*)``)

class _Records:
    def __init__(self, lines):
        self.lines = lines
        self.pos = 0

    def rewind(self):
        self.pos = 0

    def eof(self):
        return self.pos >= len(self.lines)

    @staticmethod
    def _tokens(line):
        out = []
        i, n = 0, len(line)
        while i < n:
            ch = line[i]
            if ch in " \t\r\n,":
                i += 1
                continue
            if ch == "/":
                out.append("/")
                break
            if ch in "'\"":
                j = line.find(ch, i + 1)
                if j < 0:
                    j = n
                out.append(("str", line[i + 1:j]))
                i = j + 1
                continue
            if ch == "(":
                j = line.find(")", i)
                if j < 0:
                    j = n
                out.append(("cplx", line[i + 1:j]))
                i = j + 1
                continue
            j = i
            while j < n and line[j] not in " \t\r\n,/":
                j += 1
            out.append(line[i:j])
            i = j
        return out

    def read(self, nitems):
        """One ``read(u,*)`` of nitems: continues over records until satisfied."""
        items = []
        while len(items) < nitems:
            if self.eof():
                raise EOFError("end of file in list-directed read")
            toks = self._tokens(self.lines[self.pos])
            self.pos += 1
            for t in toks:
                if t == "/":
                    return items + [None] * (nitems - len(items))
                items.append(t)
                if len(items) == nitems:
                    break
        return items


def _as_str(t):
    return t[1] if isinstance(t, tuple) else t


def _as_int(t):
    s = _as_str(t)
    return int(s)


def _as_real(t):
    s = _as_str(t).replace("d", "e").replace("D", "e")
    return float(s)


def _as_complex(t):
    if isinstance(t, tuple) and t[0] == "cplx":
        a, b = t[1].split(",")
        return complex(_as_real(a.strip()), _as_real(b.strip()))
    return complex(_as_real(t), 0.0)


def struct_limit(n: int, a: int):
    """code/files.f90:385-409: slit limits [ai, af] of width a centred in 1..n."""
    if a % 2 == 0:
        if n % 2 == 0:
            return n // 2 - (a // 2 - 1), n // 2 + a // 2
        return (n + 1) // 2 - a // 2, (n + 1) // 2 + a // 2 - 1
    if n % 2 == 0:
        return n // 2 - ((a + 1) // 2 - 1), n // 2 + (a - 1) // 2
    return (n + 1) // 2 - (a - 1) // 2, (n + 1) // 2 + (a - 1) // 2


@dataclass
class Params:
    description: str = ""
    i_pol: int = 2
    q_nm: float = 0.0
    nx: int = 1
    ny: int = 1
    nz: int = 1
    cfl: float = 0.0
    wzpml_in: float = 0.0
    pml_taflove: int = 2
    npml: int = 2
    pmlzi: int = 0
    pmlzf: int = 0
    no_downloads_in: int = 1
    output_time_step: int = 1
    texit_fs: float = 0.0
    hi: int = 1
    sdl_plane_on: tuple = (0, 0, 0)
    eps1: float = 1.0
    eps_bbox: complex = 1.0
    eps3: float = 1.0
    box1: tuple = (1, 1, 1, 1, 1, 1)
    box2: tuple = (1, 1, 1, 1, 1, 1)
    nof: int = 1
    dlamda: float = 0.0
    lno: float = 0.0
    to_fourier: int = 0
    sample_fourier: int = 1
    plane_wave: int = 1
    tincr_in: float = 0.0
    tdecay_in: float = 0.0
    epump_in: float = 0.0
    wlpump: float = 0.0
    pump_dt_in: float = 0.0
    def_pulse: float = 0.0
    tfsf_zi: int = 0
    cosine: int = 0
    dh: int = 0
    dx: int = 0
    # derived (code/files.f90)
    Q: float = 0.0
    dt: float = 0.0
    wzpml: float = 0.0
    texit: int = 0
    no_downloads: int = 1
    fw: list = field(default_factory=list)
    lnf: float = 0.0
    hf: int = 0
    aix: int = 1
    afx: int = 0
    epump: float = 0.0
    pump_dt: float = 0.0
    gpump: float = 0.0
    zopump: float = 0.0
    tincr: float = 0.0
    tdecay: float = 0.0
    iz_min: int = 0
    iz_max: int = 0
    consts: dict = field(default_factory=dict)


def setparam(path: str, single_literals: bool = True) -> Params:
    """Restatement of setparam() (code/files.f90:39-344) and the description read
    (code/main.f90:111)."""
    with open(path, "r", encoding="latin-1") as fh:
        lines = fh.read().splitlines()
    k = physconsts(single_literals)
    R = _Records(lines)
    p = Params(consts=k)
    p.description = lines[0][:100] if lines else ""

    def seek(header, guarded):
        R.rewind()
        while True:
            if guarded and R.eof():
                return False
            msg = _as_str(R.read(1)[0])
            if msg == header:
                return True

    seek("Mesh options", False)
    p.i_pol = _as_int(R.read(1)[0])
    if p.i_pol not in (1, 2, 3, 4):
        raise ValueError("Invalid input file: i_pol")
    p.q_nm = _as_real(R.read(1)[0])
    if p.q_nm <= 0:
        raise ValueError("Invalid input file: q")
    p.nx = _as_int(R.read(1)[0])
    p.ny = _as_int(R.read(1)[0])
    p.nz = _as_int(R.read(1)[0])
    if min(p.nx, p.ny, p.nz) < 1:
        raise ValueError("Invalid input file: grid size")
    Q = k["f_abohr"] * p.q_nm
    p.Q = Q
    p.cfl = _as_real(R.read(1)[0])
    if p.cfl <= 0:
        raise ValueError("Invalid input file: CFL")
    p.dt = p.cfl / (k["c0"] * np.sqrt(3.0 / (Q * Q)))
    p.wzpml_in = _as_real(R.read(1)[0])
    if p.wzpml_in < 0:
        raise ValueError("Invalid input file: wzPML")
    p.wzpml = k["f_abohr"] * (p.wzpml_in / Q)
    p.pml_taflove = _as_int(R.read(1)[0])
    p.npml = 2
    p.pmlzi = _as_int(R.read(1)[0])
    p.pmlzf = _as_int(R.read(1)[0])

    seek("Job options", False)
    a, b = R.read(2)
    p.no_downloads_in, p.output_time_step = _as_int(a), _as_int(b)
    p.texit_fs = _as_real(R.read(1)[0])
    p.texit = int(p.texit_fs / (p.dt * k["uat"]))
    p.no_downloads = int(p.texit // p.no_downloads_in)
    p.hi = _as_int(R.read(1)[0])
    p.sdl_plane_on = tuple(_as_int(t) for t in R.read(3))

    seek("Dielectric constants", False)
    p.eps1 = _as_real(R.read(1)[0])
    p.eps_bbox = _as_complex(R.read(1)[0])
    p.eps3 = _as_real(R.read(1)[0])

    if not seek("Fourier transformation options", True):
        raise ValueError("Invalid input file: no Fourier transformation options")
    box = []
    for _ in range(6):
        s_, m_ = R.read(2)
        box.append((_as_int(s_), _as_int(m_)))
    p.box1 = tuple(b[0] for b in box)
    p.box2 = tuple(b[1] for b in box)
    p.nof = _as_int(R.read(1)[0])
    p.dlamda = _as_real(R.read(1)[0])
    p.lno = _as_real(R.read(1)[0])
    lno_aux = p.lno
    fw = []
    for _ in range(p.nof):
        fw.append(2.0 * k["pi"] * k["c0"] * p.dt / (k["f_abohr"] * lno_aux))
        lno_aux = lno_aux + p.dlamda
    p.fw = fw
    p.lnf = lno_aux
    a, b = R.read(2)
    p.to_fourier, p.sample_fourier = _as_int(a), _as_int(b)

    if not seek("Source options", True):
        raise ValueError("Invalid input file: no Source options")
    p.plane_wave = _as_int(R.read(1)[0])
    a, b = R.read(2)
    p.tincr_in, p.tdecay_in = _as_real(a), _as_real(b)
    a, b, c, d = R.read(4)
    p.epump_in, p.wlpump, p.pump_dt_in, p.def_pulse = (_as_real(a), _as_real(b), _as_real(c), _as_real(d))
    p.tfsf_zi = _as_int(R.read(1)[0])
    p.cosine = _as_int(R.read(1)[0])
    p.tincr = p.tincr_in / k["uat"]
    p.tdecay = p.tdecay_in / k["uat"]
    p.epump = p.epump_in / (k["f_e"] * k["one_e_m5"])
    p.pump_dt = p.pump_dt_in / k["uat"]
    p.gpump = k["c0"] * p.pump_dt / (2.0 * Q * np.sqrt(p.eps1 * p.def_pulse))
    p.zopump = -(np.sqrt(p.def_pulse) * p.gpump) - p.tfsf_zi
    p.iz_min = p.tfsf_zi
    p.iz_max = p.tfsf_zi + 5

    seek("Slit Array", False)
    p.dh = _as_int(R.read(1)[0])
    p.hf = (p.hi + p.dh) - 1
    p.dx = _as_int(R.read(1)[0])
    p.aix, p.afx = struct_limit(p.nx, p.dx)
    return p


# ---------------------------------------------------------------------------
# ctypes binding of iris_oracle.cpp

class OrcParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("pmlzi", ctypes.c_int), ("pmlzf", ctypes.c_int), ("npml", ctypes.c_int),
        ("hi", ctypes.c_int), ("hf", ctypes.c_int),
        ("i_pol", ctypes.c_int), ("plane_wave", ctypes.c_int), ("cosine", ctypes.c_int),
        ("iz_min", ctypes.c_int), ("iz_max", ctypes.c_int),
        ("nof", ctypes.c_int), ("to_fourier", ctypes.c_int), ("sample_fourier", ctypes.c_int),
        ("box1", ctypes.c_int * 6), ("box2", ctypes.c_int * 6),
        ("system_model", ctypes.c_int), ("texit", ctypes.c_int), ("no_downloads", ctypes.c_int),
        ("Q", ctypes.c_double), ("dt", ctypes.c_double), ("c0", ctypes.c_double), ("pi", ctypes.c_double),
        ("eps0", ctypes.c_double), ("mu0", ctypes.c_double), ("f_abohr", ctypes.c_double),
        ("eps1", ctypes.c_double), ("eps3", ctypes.c_double),
        ("eps_bbox_re", ctypes.c_double), ("eps_bbox_im", ctypes.c_double),
        ("wzpml", ctypes.c_double), ("pmlalfa", ctypes.c_double),
        ("epump", ctypes.c_double), ("wlpump", ctypes.c_double), ("gpump", ctypes.c_double),
        ("zopump", ctypes.c_double),
        ("eoxy", ctypes.c_double), ("tincr", ctypes.c_double), ("tdecay", ctypes.c_double),
        ("gap", ctypes.c_double), ("ratio_angle", ctypes.c_double),
        ("akx_re", ctypes.c_double), ("akx_im", ctypes.c_double),
        ("aky_re", ctypes.c_double), ("aky_im", ctypes.c_double),
        ("akz_re", ctypes.c_double), ("akz_im", ctypes.c_double),
    ]


def build(force: bool = False) -> str:
    """Compile iris_oracle.cpp with the committed Makefile recipe."""
    src = os.path.join(HERE, "iris_oracle.cpp")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)
        L.orc_create.argtypes = [ctypes.POINTER(OrcParams), dp, ctypes.POINTER(vp)]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_threads.argtypes = [vp, ip]
        L.orc_set_eps_inv.argtypes = [vp, dp, dp]
        L.orc_slit.argtypes = [vp, ip, ip]
        L.orc_run.argtypes = [vp, ip, ip, dp, ctypes.POINTER(ctypes.c_int), ip,
                              ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        for name in ("orc_op_swap", "orc_op_e_fdtd", "orc_op_upml_e", "orc_op_bloch_max",
                     "orc_op_h_fdtd", "orc_op_upml_h", "orc_op_bloch_min"):
            getattr(L, name).argtypes = [vp]
        L.orc_op_tfsf.argtypes = [vp, ip]
        L.orc_op_dft.argtypes = [vp, ip]
        L.orc_flux.argtypes = [vp, ip, dp]
        L.orc_get_field.argtypes = [vp, ip, dp, dp]
        L.orc_set_field.argtypes = [vp, ip, dp, dp]
        L.orc_pml_size.argtypes = [vp, ip]
        L.orc_pml_size.restype = ctypes.c_long
        L.orc_get_pml.argtypes = [vp, ip, ip, ip, dp, dp]
        L.orc_set_pml.argtypes = [vp, ip, ip, ip, dp, dp]
        L.orc_get_sz.argtypes = [vp, dp, dp, dp, dp]
        L.orc_npts.argtypes = [vp, ip, ip]
        L.orc_npts.restype = ctypes.c_long
        L.orc_fdata_len.argtypes = [vp, ip, ip]
        L.orc_fdata_len.restype = ctypes.c_long
        L.orc_get_fdata.argtypes = [vp, ip, ip, dp, dp]
        L.orc_get_pto.argtypes = [vp, ip, ip, ctypes.POINTER(ctypes.c_int)]
        L.orc_tfsf_len.argtypes = [vp]
        L.orc_tfsf_len.restype = ctypes.c_long
        L.orc_get_tfsf.argtypes = [vp, dp, dp]
        L.orc_run_timed.argtypes = [vp, ip, ip, dp, dp]
        L.orc_total_points.argtypes = [vp]
        L.orc_total_points.restype = ctypes.c_long
        L.orc_film_spectrum.argtypes = [ctypes.POINTER(OrcParams), ctypes.c_double, ctypes.c_double,
                                        ip, ip, ip, dp, dp, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def to_orc_params(p: Params, ak=(0j, 0j, 0j)) -> OrcParams:
    k = p.consts
    o = OrcParams()
    o.nx, o.ny, o.nz = p.nx, p.ny, p.nz
    o.pmlzi, o.pmlzf, o.npml = p.pmlzi, p.pmlzf, p.npml
    o.hi, o.hf = p.hi, p.hf
    o.i_pol, o.plane_wave, o.cosine = p.i_pol, p.plane_wave, p.cosine
    o.iz_min, o.iz_max = p.iz_min, p.iz_max
    o.nof, o.to_fourier, o.sample_fourier = p.nof, p.to_fourier, p.sample_fourier
    o.box1 = (ctypes.c_int * 6)(*p.box1)
    o.box2 = (ctypes.c_int * 6)(*p.box2)
    o.system_model = 0
    o.texit, o.no_downloads = p.texit, p.no_downloads
    o.Q, o.dt = p.Q, p.dt
    o.c0, o.pi, o.eps0, o.mu0, o.f_abohr = k["c0"], k["pi"], k["eps0"], k["mu0"], k["f_abohr"]
    o.eps1, o.eps3 = p.eps1, p.eps3
    o.eps_bbox_re, o.eps_bbox_im = p.eps_bbox.real, p.eps_bbox.imag
    o.wzpml, o.pmlalfa = p.wzpml, k["pmlalfa"]
    o.epump, o.wlpump, o.gpump, o.zopump = p.epump, p.wlpump, p.gpump, p.zopump
    o.eoxy, o.tincr, o.tdecay, o.gap = p.epump, p.tincr, p.tdecay, 0.0
    o.ratio_angle = 1.0
    o.akx_re, o.akx_im = ak[0].real, ak[0].imag
    o.aky_re, o.aky_im = ak[1].real, ak[1].imag
    o.akz_re, o.akz_im = ak[2].real, ak[2].imag
    return o


class Oracle:
    """One reference run: main() + driver() state (code/main.f90, code/driver.f90)."""

    E_CUR, H_CUR, E_PREV, H_PREV = 0, 1, 2, 3

    def __init__(self, p: Params, ak=(0j, 0j, 0j), threads: int = 1, slit: bool = True):
        self.p = p
        self.L = lib()
        self.oparams = to_orc_params(p, ak)
        fw = np.ascontiguousarray(np.asarray(p.fw, dtype=np.float64))
        self._fw = fw
        h = ctypes.c_void_p()
        rc = self.L.orc_create(ctypes.byref(self.oparams), _dp(fw), ctypes.byref(h))
        if rc != 0:
            raise RuntimeError("orc_create failed")
        self.h = h
        self.L.orc_set_threads(h, threads)
        if slit:
            self.L.orc_slit(h, p.aix, p.afx)
        self.nos = ctypes.c_int(1)

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def field_shape(self):
        p = self.p
        return (p.nz + 2, p.ny + 2, p.nx + 2, 3)

    def set_eps_inv(self, eps_inv: np.ndarray):
        """eps_inv over (hi-1:hf+1, 0:ny+1, 0:nx+1) as a complex array [z, y, x]."""
        a = np.ascontiguousarray(eps_inv, dtype=np.complex128)
        re = np.ascontiguousarray(a.real)
        im = np.ascontiguousarray(a.imag)
        self.L.orc_set_eps_inv(self.h, _dp(re), _dp(im))

    def get_field(self, which: int) -> np.ndarray:
        """Field in the reference layout, returned as complex [z, y, x, comp]."""
        n = int(np.prod(self.field_shape))
        re = np.empty(n)
        im = np.empty(n)
        self.L.orc_get_field(self.h, which, _dp(re), _dp(im))
        return (re + 1j * im).reshape(self.field_shape)

    def set_field(self, which: int, f: np.ndarray):
        a = np.ascontiguousarray(f, dtype=np.complex128).reshape(-1)
        re = np.ascontiguousarray(a.real)
        im = np.ascontiguousarray(a.imag)
        self.L.orc_set_field(self.h, which, _dp(re), _dp(im))

    def pml_shape(self, slab: int):
        p = self.p
        n = p.pmlzi if slab == 0 else p.nz - p.pmlzf + 1
        return (n, p.ny, p.nx, 3)

    def get_pml(self, which: int, cur: int, slab: int) -> np.ndarray:
        n = int(self.L.orc_pml_size(self.h, slab))
        re = np.empty(n)
        im = np.empty(n)
        self.L.orc_get_pml(self.h, which, cur, slab, _dp(re), _dp(im))
        return (re + 1j * im).reshape(self.pml_shape(slab))

    def set_pml(self, which: int, cur: int, slab: int, v: np.ndarray):
        a = np.ascontiguousarray(v, dtype=np.complex128).reshape(-1)
        re = np.ascontiguousarray(a.real)
        im = np.ascontiguousarray(a.imag)
        self.L.orc_set_pml(self.h, which, cur, slab, _dp(re), _dp(im))

    def get_sz(self):
        p = self.p
        nb, nt = p.pmlzi, p.nz - p.pmlzf + 1
        a, b, c, d = np.empty(3 * nb), np.empty(3 * nb), np.empty(3 * nt), np.empty(3 * nt)
        self.L.orc_get_sz(self.h, _dp(a), _dp(b), _dp(c), _dp(d))
        return a.reshape(nb, 3), b.reshape(nb, 3), c.reshape(nt, 3), d.reshape(nt, 3)

    def run(self, it0: int, n: int, max_out: int = 0):
        p = self.p
        J = np.zeros(max(max_out, 1) * 6 * p.nof)
        its = (ctypes.c_int * max(max_out, 1))()
        nout = ctypes.c_int(0)
        self.L.orc_run(self.h, it0, n, _dp(J) if max_out else None, its, max_out,
                       ctypes.byref(nout), ctypes.byref(self.nos))
        k = nout.value
        return J[: k * 6 * p.nof].reshape(k, 6, p.nof), list(its[:k])

    def run_timed(self, it0: int, n: int):
        """Run n steps; returns (seconds in the DFT, seconds in everything else)."""
        td, tr = ctypes.c_double(0), ctypes.c_double(0)
        self.L.orc_run_timed(self.h, it0, n, ctypes.byref(td), ctypes.byref(tr))
        return td.value, tr.value

    def total_points(self) -> int:
        """DFT sample points accumulated per sampled step (all boxes and faces)."""
        return int(self.L.orc_total_points(self.h))

    def flux(self, box: int = 0) -> np.ndarray:
        J = np.zeros(6 * self.p.nof)
        self.L.orc_flux(self.h, box, _dp(J))
        return J.reshape(6, self.p.nof)

    def fdata(self, box: int, j: int) -> np.ndarray:
        """emg(j)%fdata(i_pts, iw) of face pair j = 1..3 as complex [iw, i_pts]."""
        n = int(self.L.orc_fdata_len(self.h, box, j - 1))
        re = np.empty(n)
        im = np.empty(n)
        self.L.orc_get_fdata(self.h, box, j - 1, _dp(re), _dp(im))
        npts = n // self.p.nof
        return (re + 1j * im).reshape(self.p.nof, npts)

    def pto(self, box: int, j: int) -> np.ndarray:
        """spts(j)%pto(i_pts, 1:4) of face pair j = 1..3."""
        n = int(self.L.orc_fdata_len(self.h, box, j - 1)) // self.p.nof
        out = np.empty(4 * n, dtype=np.int32)
        self.L.orc_get_pto(self.h, box, j - 1, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        return out.reshape(n, 4)

    def tfsf_data(self) -> np.ndarray:
        n = int(self.L.orc_tfsf_len(self.h))
        re = np.empty(n)
        im = np.empty(n)
        self.L.orc_get_tfsf(self.h, _dp(re), _dp(im))
        p = self.p
        return (re + 1j * im).reshape(p.iz_max - p.iz_min + 3, p.ny + 4, p.nx + 4, 6)

    # single reference operators (no buffer swap)
    def op(self, name: str, *args):
        getattr(self.L, "orc_op_" + name)(self.h, *args)


def film_spectrum(p: Params):
    """spectra_lossless_dielectric(), code/common.f90:104-131: analytic (lp, R, T)."""
    L = lib()
    o = to_orc_params(p)
    n = p.nof
    lp, R, T = np.empty(n), np.empty(n), np.empty(n)
    L.orc_film_spectrum(ctypes.byref(o), p.lno, p.dlamda, p.dh, 1, n, _dp(lp), _dp(R), _dp(T))
    return lp, R, T


def tr_normalise(j5: np.ndarray, j6: np.ndarray):
    """irisfdtd_scatt.py:40-42: R = J5/(J5+J6), T = J6/(J5+J6)."""
    tot = j5 + j6
    return j5 / tot, j6 / tot


def wavelength_axis(lno: float, dlamda: float, nof: int) -> np.ndarray:
    """IrisFDTD_scattering.py:111,143: linspace(iwav, iwav + dlambda*nof, nof)."""
    return np.linspace(lno, lno + dlamda * nof, nof)


# ---------------------------------------------------------------------------
# SDL field snapshots (code/sdl.f90)

@dataclass
class SdlParams:
    copy_flag: int = 0
    copy_no: int = 1
    xi: tuple = (0, 0, 0)
    xf: tuple = (0, 0, 0)
    yi: tuple = (0, 0, 0)
    yf: tuple = (0, 0, 0)
    zi: tuple = (0, 0, 0)
    zf: tuple = (0, 0, 0)
    module_e: int = 0     # SDLModuleE: 1 |E|, 2 |H|
    field: tuple = (0, 0, 0, 0, 0, 0)  # SDLField(1:6): Ex Ey Ez Hx Hy Hz
    delta: tuple = ((0,), (0,), (0,))  # SDL_deltaX/Y/Z (code/files.f90:291-320)


def setparam_sdl(path: str) -> SdlParams:
    """setparam_SDL (code/sdl.f90:365-400): after the "Time evolution options"
    header, SDL_copy_flag and SDL_copy_no, the six rows xi, xf, yi, yf, zi, zf
    (one value per plane orientation), SDLModuleE and SDLField(1:6); then the
    optional "Extra parameters-SDLextended" section (code/files.f90:291-320)."""
    with open(path, "r", encoding="latin-1") as fh:
        lines = fh.read().splitlines()
    R = _Records(lines)

    def seek(header):
        R.rewind()
        while not R.eof():
            if _as_str(R.read(1)[0]) == header:
                return True
        return False

    if not seek("Time evolution options"):
        raise ValueError("no Time evolution options")
    q = SdlParams()
    a, b = R.read(2)
    q.copy_flag, q.copy_no = _as_int(a), _as_int(b)
    rows = [tuple(_as_int(t) for t in R.read(3)) for _ in range(6)]
    q.xi, q.xf, q.yi, q.yf, q.zi, q.zf = rows
    q.module_e = _as_int(R.read(1)[0])
    q.field = tuple(_as_int(R.read(1)[0]) for _ in range(6))
    if seek("Extra parameters-SDLextended"):
        n = [_as_int(t) for t in R.read(3)]
        q.delta = tuple(tuple(_as_int(R.read(1)[0]) for _ in range(n[a])) for a in range(3))
    return q


def inttoascii(n: int) -> str:
    """inttoASCII (code/common.f90:40-101): the decimal digits of 0 <= n < 100000."""
    if not 0 <= n < 100000:
        raise ValueError("inttoASCII covers 0..99999")
    return str(n)


def _f4(x):
    """REAL(4) rounding of a REAL(8) value (Fortran real() without a kind)."""
    return np.asarray(x, dtype=np.float64).astype(np.float32)


def sdl_output(ino: int, comp: int, em: int, f: np.ndarray, q: SdlParams, layer: int, ranges, norm: float):
    """SDL_output (code/sdl.f90:68-483) for one plane: returns the file name
    and the record's REAL(4) values in file order (first index fastest).

    f: the field (e or h) as complex [z, y, x, component] over 0..n+1.
    comp: NoComponente (1..3, 0 for the modulus), em: 1 E, 2 H, 0 modulus.
    layer: 1, 2, 3 (x, y, z = const); ranges: (index, lo1, hi1, lo2, hi2) with
    the plane index and the two in-plane ranges (y, z / x, z / x, y).
    norm: SDLnorm = q*Epump with the TF/SF source on (:358-362), 1 if 0.
    The files of the "cluster" path are the ones this version writes
    (RUTA_SDL = 'cluster', :373), named './X_SDL...' (:178-193, :207-215)."""
    index, lo1, hi1, lo2, hi2 = ranges
    # EXT and EXT2 (:115-156)
    if em == 0:
        ext = ".e"
        ext2 = "_E" if q.module_e == 1 else "_H"
    else:
        ext = (".e" if em == 1 else ".h") + str(comp)
        # select case(SDLField(NoComponente)) (:140-153, :202-212): the mode of
        # an H component is read from the E entries SDLField(1:3) too; with no
        # matching case the name has no suffix and Output stays unassigned
        # (0 here)
        mode = q.field[comp - 1]
        ext2 = {1: "_R", 2: "_I", 3: "_MC", 4: "_MR", 5: "_MI"}.get(mode, "")
    axis = "XYZ"[layer - 1]
    one_layer = all(len(d) == 1 for d in q.delta)
    if one_layer:
        name = f"./{axis}_SDL{ext2}{inttoascii(ino)}{ext}"
    else:
        name = f"./{axis}_SDL{inttoascii(index)}layer{ext2}{inttoascii(ino)}{ext}"
    # Output(i1, i2) over the plane (:195-330)
    n1, n2 = hi1 - lo1 + 1, hi2 - lo2 + 1
    out = np.zeros((n2, n1))  # [i2, i1]
    for b in range(n2):
        for a in range(n1):
            u, v = lo1 + a, lo2 + b
            x, y, z = (index, u, v) if layer == 1 else (u, index, v) if layer == 2 else (u, v, index)
            if em == 0:
                g = 0.0
                for k in range(3):
                    c = f[z, y, x, k]
                    g = g + (c.conjugate() * c).real
                out[b, a] = np.sqrt(abs(g)) if layer == 2 else np.sqrt(g)
            else:
                c = f[z, y, x, comp - 1]
                if mode == 1:
                    out[b, a] = c.real
                elif mode == 2:
                    out[b, a] = c.imag
                elif mode == 3:
                    out[b, a] = np.sqrt((c.conjugate() * c).real)
                elif mode == 4:
                    out[b, a] = np.sqrt(c.real * c.real)
                elif mode == 5:
                    out[b, a] = np.sqrt(c.imag * c.imag)
    if norm == 0.0:
        norm = 1.0
    # output = real(output)/SDLnorm (:363): REAL(4) first, then the REAL(8)
    # quotient, written as REAL(4) again (:449-456)
    out = _f4(_f4(out).astype(np.float64) / norm)
    if not q.copy_flag:
        return name, out.reshape(-1)
    # the copies (:391-421): output_aux(ixo : SDL_copy_no*(ixf+1-ixo), iyo : ...)
    # (both axes for z planes); this restatement covers lo1 = 1 (and lo2 = 1 for
    # z planes), where every cell of output_aux is written
    c2 = q.copy_no if layer == 3 else 1
    if lo1 != 1 or (layer == 3 and lo2 != 1):
        raise ValueError("copies are restated for planes starting at index 1")
    aux = np.tile(out, (c2, q.copy_no))
    return name, aux.reshape(-1)


def sdl_snapshot(ino: int, e: np.ndarray, h_prev: np.ndarray, q: SdlParams, planes_on, norm: float) -> dict:
    """The driver's snapshot at one output step (code/driver.f90:468-494): for
    each plane orientation switched on and each extra layer, setSDL_FILE
    (code/sdl.f90:404-448) with e_cur and h_prev; ino is the file number the
    driver passes (nos + 1).  Returns {file name: REAL(4) values}."""
    out = {}
    for layer in (1, 2, 3):
        if not planes_on[layer - 1]:
            continue
        j = layer - 1
        for d in q.delta[j]:
            if layer == 1:
                r = (q.xi[j] + d, q.yi[j], q.yf[j], q.zi[j], q.zf[j])
            elif layer == 2:
                r = (q.yi[j] + d, q.xi[j], q.xf[j], q.zi[j], q.zf[j])
            else:
                r = (q.zi[j] + d, q.xi[j], q.xf[j], q.yi[j], q.yf[j])
            if q.module_e == 1:
                k, v = sdl_output(ino, 0, 0, e, q, layer, r, norm)
                out[k] = v
            if q.module_e == 2:
                k, v = sdl_output(ino, 0, 0, h_prev, q, layer, r, norm)
                out[k] = v
            for c in (1, 2, 3):
                if q.field[c - 1] >= 1:
                    k, v = sdl_output(ino, c, 1, e, q, layer, r, norm)
                    out[k] = v
            for c in (1, 2, 3):
                if q.field[c + 2] >= 1:
                    k, v = sdl_output(ino, c, 2, h_prev, q, layer, r, norm)
                    out[k] = v
    return out


def write_sdl_record(path: str, values: np.ndarray):
    """One Fortran unformatted sequential record: a 4-byte length, the REAL(4)
    values, the length again."""
    v = np.asarray(values, dtype="<f4")
    n = np.asarray([v.size * 4], dtype="<i4").tobytes()
    with open(path, "wb") as fh:
        fh.write(n + v.tobytes() + n)
