"""GB300-native FDTD engine with IrisFDTD-Academic's hot-path interface.

Python host mirror of the reference's operator interface, over the C ABI in
include/iris_fdtd.h (libiris_fdtd.so, CUDA kernels for sm_103a):

=====================  =========================================================
this module            reference (IrisFDTD-Academic, Fortran)
=====================  =========================================================
``setparam``           setparam(), code/files.f90:39-344
``set_emconstants``    set_emconstants(), code/mesh.f90:75-109 (+ slit(), :57-69)
``Engine``             main()/driver() state, code/main.f90:164-170, driver.f90:174-335
``Engine.step``        the time-loop body, code/driver.f90:356-451
``Engine.e_fdtd``      e_fdtd + UPML_Array_e + bc_*max_bloch (driver.f90:388-400)
``Engine.h_fdtd``      h_fdtd + UPML_Array_h + bc_*min_bloch (driver.f90:405-415)
``Engine.tfsf``        tfsf_gauss/tfsf_plane_wave + tfsf_update_* (driver.f90:420-442)
``Engine.scattering_fourier``      scattering_fourier, code/dataprocess.f90:109-209
``Engine.scattering_fourier_out``  flux of scattering_fourier_out, :213-277
``run_input``          program IrisFDTD, code/program.f90:25-61
``tr_normalise``       irisfdtd_scatt.py:40-42
=====================  =========================================================

Errors raise :class:`IrisError` carrying the C status code (the reference
STOPs in err(), code/files.f90:352-381).  There is no CPU fallback: without
the native library (or without a GPU) the engine entry points raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import native
from .native import IrisError, IrisParams, build, check, lib

FP64, FP32 = 0, 1
STENCIL_DEFAULT, STENCIL_SPLIT, STENCIL_FUSED, STENCIL_STREAM, STENCIL_PERSISTENT = 0, 1, 2, 3, 4
PERSISTENT_MAX_CELLS = 1048576  # IRIS_PERSISTENT_MAX_CELLS: the persistent kernel's default limit in FP64
PERSISTENT_MAX_CELLS_FP32 = 8388608  # IRIS_PERSISTENT_MAX_CELLS_FP32: the same in FP32
DFT_KERNEL_AUTO, DFT_KERNEL_CUDA, DFT_KERNEL_TENSOR = 0, 1, 2
E, H = 0, 1
OP_E, OP_H, OP_TFSF, OP_DFT, OP_WAIT_CHECK, OP_BARRIER_CHECK = 1, 2, 3, 4, 5, 6

__all__ = [
    "FP64", "FP32", "E", "H", "IrisError", "IrisParams", "Engine", "build", "lib", "setparam",
    "set_emconstants", "run_input", "tr_normalise", "wavelength_axis", "frequencies", "physconsts",
    "write_scatt", "read_scatt",
]


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _split_material(eps_inv):
    """(re, im) float64 C-contiguous arrays; im None for a real material (a
    real array is passed on without a copy)."""
    a = np.asarray(eps_inv)
    if not np.iscomplexobj(a):
        return np.ascontiguousarray(a, dtype=np.float64), None
    im = np.ascontiguousarray(a.imag, dtype=np.float64)
    return np.ascontiguousarray(a.real, dtype=np.float64), (im if np.any(im) else None)


def physconsts(single_literals: bool = True) -> IrisParams:
    p = IrisParams()
    lib().iris_physconsts(ctypes.byref(p), 1 if single_literals else 0)
    return p


def frequencies(p: IrisParams) -> np.ndarray:
    fw = np.zeros(max(p.nof, 1))
    check(lib().iris_frequencies(ctypes.byref(p), _dp(fw), len(fw)), "iris_frequencies")
    return fw[: p.nof]


def setparam(path: str, single_literals: bool = True):
    """Read inputFDTD.dat: returns (params, fw, description)."""
    L = lib()
    p = IrisParams()
    desc = ctypes.create_string_buffer(128)
    check(L.iris_setparam(os.fsencode(path), 1 if single_literals else 0, ctypes.byref(p), None, 0, desc, 128),
          "iris_setparam")
    return p, frequencies(p), desc.value.decode("latin-1")


def set_emconstants(p: IrisParams) -> np.ndarray:
    """eps_inv over (hi-1:hf+1, 0:ny+1, 0:nx+1) as complex [z, y, x], with the
    slit of slit() applied (code/mesh.f90:57-109)."""
    nz = p.hf - p.hi + 3
    eb = complex(p.eps_bbox_re, p.eps_bbox_im)
    a = np.full((nz, p.ny + 2, p.nx + 2), 1.0 / eb, dtype=np.complex128)
    a[0] = 1.0 / p.eps1
    a[-1] = 1.0 / p.eps3
    if p.afx >= p.aix:
        a[1:-1, :, p.aix:p.afx + 1] = 1.0
    return a


class Engine:
    """One run: device state of main()+driver() behind iris_create."""

    def __init__(self, p: IrisParams, fw=None, precision: int | None = None, dft_block: int = 0, device: int = 0,
                 stencil: int = 0, graph: bool = False, dft_kernel: int = 0):
        self.L = lib()
        q = p.copy()
        if precision is not None:
            q.precision = precision
        q.dft_block = dft_block
        q.stencil = stencil
        q.device = device
        q.graph = 1 if graph else 0
        q.dft_kernel = dft_kernel
        self.p = q
        self.fw = np.ascontiguousarray(frequencies(q) if fw is None else np.asarray(fw, dtype=np.float64))
        h = ctypes.c_void_p()
        check(self.L.iris_create(ctypes.byref(self.p), _dp(self.fw), ctypes.byref(h)), "iris_create")
        self.h = h

    @classmethod
    def _view(cls, handle, p: IrisParams, fw, owner) -> "Engine":
        """A borrowed engine handle (owned and destroyed by owner)."""
        e = cls.__new__(cls)
        e.L, e.p, e.fw, e.h, e._owner = lib(), p, fw, handle, owner
        return e

    # -- lifetime
    def close(self):
        if getattr(self, "_owner", None) is not None:
            self.h = None
            return
        if getattr(self, "h", None):
            self.L.iris_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- shapes
    @property
    def field_shape(self):
        p = self.p
        return (p.nz + 2, p.ny + 2, p.nx + 2, 3)

    def pml_shape(self, slab: int):
        p = self.p
        return ((p.pmlzi if slab == 0 else p.nz - p.pmlzf + 1), p.ny, p.nx, 3)

    # -- material
    def set_material(self, eps_inv: np.ndarray):
        """eps_inv over (hi-1:hf+1, 0:ny+1, 0:nx+1) as [z, y, x], real or complex."""
        p = self.p
        want = (p.hf - p.hi + 3, p.ny + 2, p.nx + 2)
        if np.shape(eps_inv) != want:
            raise ValueError(f"eps_inv shape {np.shape(eps_inv)} != {want}")
        re, im = _split_material(eps_inv)
        check(self.L.iris_set_material(self.h, _dp(re), _dp(im) if im is not None else None), "iris_set_material")

    # -- material generated on the device (the same values as the host voxelisers in configs.py)
    def material_spheres(self, spheres: np.ndarray):
        """Rows (cx, cy, cz, r, eps) over 1/eps_bbox, later rows win (iris_material_spheres)."""
        a = np.ascontiguousarray(np.asarray(spheres, dtype=np.float64).reshape(-1, 5))
        check(self.L.iris_material_spheres(self.h, a.shape[0], _dp(a)), "iris_material_spheres")

    def material_pattern(self, seed: int, fill: float, eps_in: float = 4.0, eps_out: float = 1.0):
        check(self.L.iris_material_pattern(self.h, seed, fill, eps_in, eps_out), "iris_material_pattern")

    def material_design(self, seed: int, region, emin: float, emax: float):
        r = (ctypes.c_int * 4)(*[int(v) for v in region])
        check(self.L.iris_material_design(self.h, seed, r, emin, emax), "iris_material_design")

    def get_material(self) -> np.ndarray:
        """The stored eps_inv, planes hi..hf, as complex [z, y, x] over 0..n+1."""
        p = self.p
        shape = (max(0, p.hf - p.hi + 1), p.ny + 2, p.nx + 2)
        n = int(np.prod(shape))
        re, im = np.zeros(max(n, 1)), np.zeros(max(n, 1))
        check(self.L.iris_get_material(self.h, _dp(re), _dp(im)), "iris_get_material")
        return (re[:n] + 1j * im[:n]).reshape(shape)

    # -- stepping
    def step(self, it0: int, n: int):
        check(self.L.iris_step(self.h, it0, n), "iris_step")

    def sync(self):
        check(self.L.iris_sync(self.h), "iris_sync")

    def e_fdtd(self):
        check(self.L.iris_apply(self.h, OP_E, 0), "iris_apply(E)")

    def h_fdtd(self):
        check(self.L.iris_apply(self.h, OP_H, 0), "iris_apply(H)")

    def tfsf(self, it: int):
        check(self.L.iris_apply(self.h, OP_TFSF, it), "iris_apply(TFSF)")

    def scattering_fourier(self, t: int):
        check(self.L.iris_apply(self.h, OP_DFT, t), "iris_apply(DFT)")

    def scattering_fourier_out(self, box: int = 0) -> np.ndarray:
        return self.flux(box)

    def flux(self, box: int = 0) -> np.ndarray:
        J = np.zeros(6 * self.p.nof)
        check(self.L.iris_flux(self.h, box, _dp(J)), "iris_flux")
        return J.reshape(6, self.p.nof)

    # -- state access in the reference layout
    def get_field(self, which: int) -> np.ndarray:
        n = int(np.prod(self.field_shape))
        re, im = np.empty(n), np.empty(n)
        check(self.L.iris_get_field(self.h, which, _dp(re), _dp(im)), "iris_get_field")
        return (re + 1j * im).reshape(self.field_shape)

    def set_field(self, which: int, f: np.ndarray):
        a = np.asarray(f, dtype=np.complex128).reshape(-1)
        re, im = np.ascontiguousarray(a.real), np.ascontiguousarray(a.imag)
        check(self.L.iris_set_field(self.h, which, _dp(re), _dp(im)), "iris_set_field")

    def get_field_c(self, which: int) -> np.ndarray:
        """The field as the reference stores it, complex(8) (3, 0:nx+1, 0:ny+1,
        0:nz+1) in Fortran order, i.e. a C-order complex128 array [z, y, x, c]
        filled in place by the device (iris_get_field_c)."""
        a = np.empty(self.field_shape, dtype=np.complex128)
        check(self.L.iris_get_field_c(self.h, which, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
              "iris_get_field_c")
        return a

    def set_field_c(self, which: int, f: np.ndarray):
        a = np.ascontiguousarray(np.asarray(f, dtype=np.complex128).reshape(self.field_shape))
        check(self.L.iris_set_field_c(self.h, which, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
              "iris_set_field_c")

    def get_pml_c(self, which: int, slab: int) -> np.ndarray:
        a = np.empty(self.pml_shape(slab), dtype=np.complex128)
        check(self.L.iris_get_pml_c(self.h, which, slab, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
              "iris_get_pml_c")
        return a

    def set_pml_c(self, which: int, slab: int, v: np.ndarray):
        a = np.ascontiguousarray(np.asarray(v, dtype=np.complex128).reshape(self.pml_shape(slab)))
        check(self.L.iris_set_pml_c(self.h, which, slab, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
              "iris_set_pml_c")

    def get_pml(self, which: int, slab: int) -> np.ndarray:
        n = int(np.prod(self.pml_shape(slab)))
        re, im = np.empty(n), np.empty(n)
        check(self.L.iris_get_pml(self.h, which, slab, _dp(re), _dp(im)), "iris_get_pml")
        return (re + 1j * im).reshape(self.pml_shape(slab))

    def set_pml(self, which: int, slab: int, v: np.ndarray):
        a = np.asarray(v, dtype=np.complex128).reshape(-1)
        re, im = np.ascontiguousarray(a.real), np.ascontiguousarray(a.imag)
        check(self.L.iris_set_pml(self.h, which, slab, _dp(re), _dp(im)), "iris_set_pml")

    def get_plane(self, which: int, axis: int, index: int, r1, r2) -> np.ndarray:
        """One plane (axis 1, 2, 3 = x, y, z = index) over the in-plane ranges
        r1 = (lo, hi), r2 = (lo, hi), as complex [i2, i1, component]."""
        n1, n2 = r1[1] - r1[0] + 1, r2[1] - r2[0] + 1
        re, im = np.empty(3 * n1 * n2), np.empty(3 * n1 * n2)
        check(self.L.iris_get_plane(self.h, which, axis, index, r1[0], r1[1], r2[0], r2[1], _dp(re), _dp(im)),
              "iris_get_plane")
        return (re + 1j * im).reshape(n2, n1, 3)

    # -- instrumentation
    KERNELS = ("update_e", "update_h", "tfsf", "dft_gather", "dft_block", "flux", "fused_eh", "persistent")

    def timing_start(self, per_kernel: bool = True):
        check(self.L.iris_timing(self.h, 1 if per_kernel else 0), "iris_timing")

    def timing_read(self):
        """(region_ms, {kernel: ms}, {kernel: launches}) of the timed region."""
        reg = ctypes.c_double(0)
        ms = np.zeros(len(self.KERNELS))
        n = (ctypes.c_long * len(self.KERNELS))()
        check(self.L.iris_timing_read(self.h, ctypes.byref(reg), _dp(ms), n), "iris_timing_read")
        return reg.value, dict(zip(self.KERNELS, ms.tolist())), dict(zip(self.KERNELS, list(n)))

    def info(self) -> dict:
        a = (ctypes.c_long * 7)()
        check(self.L.iris_info(self.h, a), "iris_info")
        return dict(dft_points=a[0], dft_block=a[1], bytes_per_complex=a[2], comp_elems=a[3],
                    complex_material=bool(a[4]), boxes=a[5], dft_buffered=a[6])

    def dft_commit(self):
        """Accumulate the buffered DFT samples into fdata now (iris_dft_commit)."""
        check(self.L.iris_dft_commit(self.h), "iris_dft_commit")

    def get_fdata(self, box: int, j: int) -> np.ndarray:
        """emg(j)%fdata in the reference order as complex [iw, i_pts]."""
        n = ctypes.c_long(0)
        check(self.L.iris_get_fdata(self.h, box, j, None, None, ctypes.byref(n)), "iris_get_fdata")
        npts = n.value
        if npts == 0:
            return np.zeros((self.p.nof, 0), dtype=np.complex128)
        re, im = np.empty(npts * self.p.nof), np.empty(npts * self.p.nof)
        check(self.L.iris_get_fdata(self.h, box, j, _dp(re), _dp(im), ctypes.byref(n)), "iris_get_fdata")
        return (re + 1j * im).reshape(self.p.nof, npts)


DFT_ALL, DFT_Z = 0, 1
TILES = ((32, 8, 1), (32, 4, 2), (64, 4, 1), (16, 16, 1), (32, 2, 4), ("flat", 256), ("flat", 256, "uncapped"),
         ("fused", 32, 16))


class Batch:
    """Many independent cells stepped together (iris_batch_*): each cell its own
    grid, structure, source and Bloch phases; shared precision, dt, frequencies."""

    def __init__(self, params, fw, precision: int | None = None, dft_faces: int = DFT_Z, device: int = 0,
                 dft_block: int = 0, graph: bool = False):
        self.L = lib()
        arr = (IrisParams * len(params))()
        for i, p in enumerate(params):
            q = p.copy()
            if precision is not None:
                q.precision = precision
            q.device = device
            q.dft_block = dft_block
            q.graph = 1 if graph else 0
            arr[i] = q
        self.params = arr
        self.n = len(params)
        self.fw = np.ascontiguousarray(np.asarray(fw, dtype=np.float64))
        h = ctypes.c_void_p()
        check(self.L.iris_batch_create(self.n, arr, _dp(self.fw), dft_faces, ctypes.byref(h)), "iris_batch_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.iris_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_material(self, cell: int, eps_inv: np.ndarray):
        re, im = _split_material(eps_inv)
        check(self.L.iris_batch_set_material(self.h, cell, _dp(re), _dp(im) if im is not None else None),
              "iris_batch_set_material")

    def material_pattern(self, cell: int, seed: int, fill: float, eps_in: float = 4.0, eps_out: float = 1.0):
        check(self.L.iris_batch_material_pattern(self.h, cell, seed, fill, eps_in, eps_out),
              "iris_batch_material_pattern")

    def step(self, it0: int, n: int):
        check(self.L.iris_batch_step(self.h, it0, n), "iris_batch_step")

    def flux(self, cell: int) -> np.ndarray:
        J = np.zeros(6 * self.params[cell].nof)
        check(self.L.iris_batch_flux(self.h, cell, _dp(J)), "iris_batch_flux")
        return J.reshape(6, -1)

    def get_field(self, cell: int, which: int) -> np.ndarray:
        p = self.params[cell]
        shape = (p.nz + 2, p.ny + 2, p.nx + 2, 3)
        n = int(np.prod(shape))
        re, im = np.empty(n), np.empty(n)
        check(self.L.iris_batch_get_field(self.h, cell, which, _dp(re), _dp(im)), "iris_batch_get_field")
        return (re + 1j * im).reshape(shape)

    def tune(self, reps: int = 3):
        """Time every work list (split-pass tiles, flat runs and, in FP32, the
        fused pass) on this batch and keep the fastest; call before the first
        step.  Returns (the chosen entry of TILES, {entry: ms per E+H pass},
        -1 for a list the precision or memory does not allow)."""
        best = ctypes.c_int(0)
        ms = np.zeros(len(TILES))
        check(self.L.iris_batch_tune(self.h, reps, ctypes.byref(best), _dp(ms)), "iris_batch_tune")
        return TILES[best.value], dict(zip(TILES, ms.tolist()))

    def autotune(self, reps: int = 3):
        """iris_batch_autotune: the cached pick for this batch's size class, or
        tune() and cache its pick.  Returns (the chosen entry of TILES, whether
        it came from the cache)."""
        best, cached = ctypes.c_int(0), ctypes.c_int(0)
        check(self.L.iris_batch_autotune(self.h, reps, ctypes.byref(best), ctypes.byref(cached)),
              "iris_batch_autotune")
        return TILES[best.value], bool(cached.value)

    def set_tile(self, tile_index: int):
        check(self.L.iris_batch_set_tile(self.h, tile_index), "iris_batch_set_tile")

    def timing_start(self, per_kernel: bool = True):
        check(self.L.iris_batch_timing(self.h, 1 if per_kernel else 0), "iris_batch_timing")

    def timing_read(self):
        reg = ctypes.c_double(0)
        ms = np.zeros(len(Engine.KERNELS))
        n = (ctypes.c_long * len(Engine.KERNELS))()
        check(self.L.iris_batch_timing_read(self.h, ctypes.byref(reg), _dp(ms), n), "iris_batch_timing_read")
        return reg.value, dict(zip(Engine.KERNELS, ms.tolist())), dict(zip(Engine.KERNELS, list(n)))

    def info(self) -> dict:
        a = (ctypes.c_long * 8)()
        check(self.L.iris_batch_info(self.h, a), "iris_batch_info")
        return dict(cells=a[0], grid_cells=a[1], dft_points=a[2], dft_block=a[3], tile=TILES[a[4]], items=a[5],
                    launches_per_pass=a[6], dft_buffered=a[7])

    def dft_commit(self):
        """Accumulate the buffered DFT samples of every cell (iris_batch_dft_commit)."""
        check(self.L.iris_batch_dft_commit(self.h), "iris_batch_dft_commit")


from .adjoint import Adjoint, design_objective  # noqa: E402


def bounds_check():
    """(enabled, first) of iris_bounds_check: whether the loaded library is the
    bounds-checking build (IRIS_BOUNDS_CHECK=1 in the environment before the
    first call loads it), and the first out-of-range access its kernels met
    since the last call as (site, index), or None; the record is cleared."""
    v = ctypes.c_ulonglong(0)
    enabled = lib().iris_bounds_check(ctypes.byref(v))
    if enabled < 0:
        check(enabled, "iris_bounds_check")
    first = None if v.value == 0 else (int(v.value >> 48), int(v.value & 0xFFFFFFFFFFFF))
    return bool(enabled), first


def run_input(directory: str, precision: int = FP64):
    """The drop-in main program: reads directory/inputFDTD.dat, writes log.dat and
    the <box>_scatt*.dat files there."""
    check(lib().iris_run_input(os.fsencode(directory), precision), "iris_run_input")


def tr_normalise(j5: np.ndarray, j6: np.ndarray):
    """R = J5/(J5+J6), T = J6/(J5+J6) (irisfdtd_scatt.py:40-42), in FP64."""
    j5 = np.asarray(j5, dtype=np.float64)
    j6 = np.asarray(j6, dtype=np.float64)
    tot = j5 + j6
    return j5 / tot, j6 / tot


def wavelength_axis(lno: float, dlamda: float, nof: int) -> np.ndarray:
    """The plotting axis of IrisFDTD_scattering.py:111,143."""
    return np.linspace(lno, lno + dlamda * nof, nof)


def write_scatt(directory: str, box: int, it: int, J: np.ndarray):
    """Append one output block (step it, J[6, nof] as returned by Engine.flux)
    to <box+1>_scatt1..6.dat and <box+1>_scatt.dat in directory, in the
    records scattering_fourier_out writes (code/dataprocess.f90:279-299)."""
    J = np.ascontiguousarray(J, dtype=np.float64)
    if J.ndim != 2 or J.shape[0] != 6:
        raise ValueError("J must be [6, nof]")
    check(lib().iris_write_scatt(os.fsencode(directory), box, it, J.shape[1], _dp(J)), "iris_write_scatt")


def read_scatt(path: str, nof: int) -> np.ndarray:
    """Blocks of a <box>_scatt<j>.dat file as [block, nof] (IrisFDTD_scattering.py:74-99)."""
    vals = []
    with open(path) as fh:
        for line in fh:
            v = line.split()
            if v and v[0] != "#":
                vals.append(float(v[0]))
    a = np.asarray(vals)
    return a.reshape(-1, nof)
