"""Build and load the native engine (libiris_fdtd.so) — CUDA kernels for
sm_103a plus the C ABI declared in include/iris_fdtd.h.

The library is built in-tree next to this file.  There is no fallback: if it
is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB_PLAIN = os.path.join(PKG, "libiris_fdtd.so")
# the bounds-checking build (-DIRIS_BOUNDS_CHECK); IRIS_BOUNDS_CHECK=1 loads it
LIB_BC = os.path.join(PKG, "libiris_fdtd_bc.so")
LIB = LIB_BC if os.environ.get("IRIS_BOUNDS_CHECK") == "1" else LIB_PLAIN
SOURCES = ["iris_engine.cu", "iris_batch.cu", "iris_adjoint.cu", "iris_host.cpp"]
HEADERS = [os.path.join(INCLUDE, "iris_fdtd.h")] + [os.path.join(CSRC, h) for h in
                                                   ("iris_internal.h", "iris_device.cuh", "iris_engine.h",
                                                    "iris_fused.cuh")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _stale(lib_path: str = None) -> bool:
    paths = [lib_path] if lib_path else [LIB_PLAIN, LIB_BC]
    deps = [os.path.join(CSRC, s) for s in SOURCES] + HEADERS
    for path in paths:
        if not os.path.exists(path):
            return True
        t = os.path.getmtime(path)
        if any(os.path.getmtime(d) > t for d in deps):
            return True
    return False


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the engine for sm_103a (nvcc cross-compiles without a GPU):
    libiris_fdtd.so and its bounds-checking twin libiris_fdtd_bc.so, all
    translation units in parallel."""
    if not force and not _stale():
        return LIB
    jobs = []  # (library, objects)
    procs = []
    for lib_path, defs, tag in ((LIB_PLAIN, [], ""), (LIB_BC, ["-DIRIS_BOUNDS_CHECK"], "_bc")):
        objs = []
        for s in SOURCES:
            src = os.path.join(CSRC, s)
            obj = os.path.join(CSRC, os.path.splitext(s)[0] + tag + ".o")
            cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", *defs,
                   "-I", INCLUDE, "-c", src, "-o", obj]
            if verbose:
                print(" ".join(cmd))
            procs.append(subprocess.Popen(cmd))
            objs.append(obj)
        jobs.append((lib_path, objs))
    for pr in procs:
        if pr.wait() != 0:
            raise RuntimeError("nvcc failed building the engine")
    for lib_path, objs in jobs:
        tmp = lib_path + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, lib_path)
        for o in objs:
            os.remove(o)
    return LIB


# ---------------------------------------------------------------------------
# ctypes mirror of iris_params (include/iris_fdtd.h)

_I, _D = ctypes.c_int, ctypes.c_double


class IrisParams(ctypes.Structure):
    _fields_ = [
        ("i_pol", _I), ("nx", _I), ("ny", _I), ("nz", _I), ("pmlzi", _I), ("pmlzf", _I),
        ("npml", _I), ("pml_taflove", _I),
        ("q_nm", _D), ("Q", _D), ("cfl", _D), ("dt", _D), ("wzpml", _D),
        ("no_downloads", _I), ("output_time_step", _I), ("texit", _I), ("texit_fs", _D),
        ("hi", _I), ("hf", _I), ("sdl_plane_on", _I * 3),
        ("eps1", _D), ("eps3", _D), ("eps_bbox_re", _D), ("eps_bbox_im", _D),
        ("box1", _I * 6), ("box2", _I * 6), ("nof", _I), ("dlamda", _D), ("lno", _D),
        ("to_fourier", _I), ("sample_fourier", _I),
        ("plane_wave", _I), ("tfsf_zi", _I), ("tfsf_zf", _I), ("cosine", _I),
        ("epump", _D), ("wlpump", _D), ("pump_dt", _D), ("def_pulse", _D), ("gpump", _D), ("zopump", _D),
        ("tincr", _D), ("tdecay", _D), ("gap", _D), ("ratio_angle", _D),
        ("dh", _I), ("dx", _I), ("aix", _I), ("afx", _I),
        ("pi", _D), ("c0", _D), ("eps0", _D), ("mu0", _D), ("f_abohr", _D), ("uat", _D), ("f_e", _D),
        ("pmlalfa", _D),
        ("akx_re", _D), ("akx_im", _D), ("aky_re", _D), ("aky_im", _D), ("akz_re", _D), ("akz_im", _D),
        ("system_model", _I), ("precision", _I), ("dft_block", _I), ("device", _I), ("stencil", _I),
        ("dft_faces", _I), ("graph", _I), ("dft_kernel", _I),
    ]

    def copy(self) -> "IrisParams":
        c = IrisParams()
        ctypes.memmove(ctypes.byref(c), ctypes.byref(self), ctypes.sizeof(IrisParams))
        return c


EXPORTS = [
    "iris_strerror", "iris_last_error", "iris_setparam", "iris_physconsts", "iris_frequencies",
    "iris_create", "iris_destroy", "iris_set_material", "iris_step", "iris_sync", "iris_flux",
    "iris_dft_commit", "iris_material_spheres", "iris_material_pattern", "iris_material_design",
    "iris_get_material", "iris_batch_material_pattern", "iris_write_scatt", "iris_get_field", "iris_set_field", "iris_get_pml", "iris_set_pml",
    "iris_get_field_c", "iris_set_field_c", "iris_get_pml_c", "iris_set_pml_c",
    "iris_get_fdata", "iris_get_plane", "iris_apply", "iris_run_input", "iris_timing", "iris_timing_read", "iris_info",
    "iris_bounds_check",
    "iris_dft_block_noalloc", "iris_batch_create", "iris_batch_destroy", "iris_batch_set_material",
    "iris_batch_step", "iris_batch_flux", "iris_batch_dft_commit", "iris_batch_get_field", "iris_batch_tune",
    "iris_batch_autotune", "iris_batch_set_tile",
    "iris_batch_timing", "iris_batch_timing_read", "iris_batch_info",
    "iris_adjoint_create", "iris_adjoint_destroy", "iris_adjoint_set_material", "iris_adjoint_set_design",
    "iris_adjoint_forward", "iris_adjoint_backward", "iris_adjoint_engine", "iris_adjoint_apply",
    "iris_adjoint_timing",
]

_lib = None


def lib():
    """Load libiris_fdtd.so (building it if the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB) or _stale(LIB):
        build()
    L = ctypes.CDLL(LIB)
    vp, ip, dp, cp = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_char_p
    P = ctypes.POINTER(IrisParams)
    L.iris_strerror.argtypes = [ip]
    L.iris_strerror.restype = cp
    L.iris_last_error.argtypes = []
    L.iris_last_error.restype = cp
    L.iris_setparam.argtypes = [cp, ip, P, dp, ip, cp, ip]
    L.iris_physconsts.argtypes = [P, ip]
    L.iris_physconsts.restype = None
    L.iris_frequencies.argtypes = [P, dp, ip]
    L.iris_create.argtypes = [P, dp, ctypes.POINTER(vp)]
    L.iris_destroy.argtypes = [vp]
    L.iris_destroy.restype = None
    L.iris_set_material.argtypes = [vp, dp, dp]
    L.iris_step.argtypes = [vp, ip, ip]
    L.iris_sync.argtypes = [vp]
    L.iris_flux.argtypes = [vp, ip, dp]
    L.iris_dft_commit.argtypes = [vp]
    u64 = ctypes.c_ulonglong
    L.iris_material_spheres.argtypes = [vp, ip, dp]
    L.iris_material_pattern.argtypes = [vp, u64, ctypes.c_double, ctypes.c_double, ctypes.c_double]
    L.iris_material_design.argtypes = [vp, u64, ctypes.POINTER(ctypes.c_int), ctypes.c_double, ctypes.c_double]
    L.iris_get_material.argtypes = [vp, dp, dp]
    L.iris_batch_material_pattern.argtypes = [vp, ip, u64, ctypes.c_double, ctypes.c_double, ctypes.c_double]
    L.iris_write_scatt.argtypes = [cp, ip, ip, ip, dp]
    L.iris_get_field.argtypes = [vp, ip, dp, dp]
    L.iris_set_field.argtypes = [vp, ip, dp, dp]
    L.iris_get_pml.argtypes = [vp, ip, ip, dp, dp]
    L.iris_set_pml.argtypes = [vp, ip, ip, dp, dp]
    L.iris_get_field_c.argtypes = [vp, ip, dp]
    L.iris_set_field_c.argtypes = [vp, ip, dp]
    L.iris_get_pml_c.argtypes = [vp, ip, ip, dp]
    L.iris_set_pml_c.argtypes = [vp, ip, ip, dp]
    L.iris_get_fdata.argtypes = [vp, ip, ip, dp, dp, ctypes.POINTER(ctypes.c_long)]
    L.iris_get_plane.argtypes = [vp, ip, ip, ip, ip, ip, ip, ip, dp, dp]
    L.iris_apply.argtypes = [vp, ip, ip]
    L.iris_run_input.argtypes = [cp, ip]
    L.iris_timing.argtypes = [vp, ip]
    L.iris_timing_read.argtypes = [vp, dp, dp, ctypes.POINTER(ctypes.c_long)]
    L.iris_info.argtypes = [vp, ctypes.POINTER(ctypes.c_long)]
    L.iris_bounds_check.argtypes = [ctypes.POINTER(ctypes.c_ulonglong)]
    L.iris_dft_block_noalloc.argtypes = [vp, ip, ctypes.c_long, ip, ip, vp, ip, ctypes.c_double, vp, vp]
    lp = ctypes.POINTER(ctypes.c_long)
    L.iris_batch_create.argtypes = [ip, P, dp, ip, ctypes.POINTER(vp)]
    L.iris_batch_destroy.argtypes = [vp]
    L.iris_batch_destroy.restype = None
    L.iris_batch_set_material.argtypes = [vp, ip, dp, dp]
    L.iris_batch_step.argtypes = [vp, ip, ip]
    L.iris_batch_flux.argtypes = [vp, ip, dp]
    L.iris_batch_dft_commit.argtypes = [vp]
    L.iris_batch_get_field.argtypes = [vp, ip, ip, dp, dp]
    L.iris_batch_tune.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_int), dp]
    L.iris_batch_autotune.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.iris_batch_set_tile.argtypes = [vp, ip]
    L.iris_batch_timing.argtypes = [vp, ip]
    L.iris_batch_timing_read.argtypes = [vp, dp, dp, lp]
    L.iris_batch_info.argtypes = [vp, lp]
    L.iris_adjoint_create.argtypes = [P, dp, ctypes.POINTER(ctypes.c_int), ip, dp, ctypes.POINTER(vp)]
    L.iris_adjoint_destroy.argtypes = [vp]
    L.iris_adjoint_destroy.restype = None
    L.iris_adjoint_set_material.argtypes = [vp, dp, dp]
    L.iris_adjoint_set_design.argtypes = [vp, dp]
    L.iris_adjoint_forward.argtypes = [vp, ip, dp, dp]
    L.iris_adjoint_backward.argtypes = [vp, dp]
    L.iris_adjoint_engine.argtypes = [vp, ip, ctypes.POINTER(vp)]
    L.iris_adjoint_apply.argtypes = [vp, ip]
    L.iris_adjoint_timing.argtypes = [vp, dp]
    _lib = L
    return L


class IrisError(RuntimeError):
    def __init__(self, code: int, where: str):
        L = lib()
        msg = L.iris_last_error().decode() or L.iris_strerror(code).decode()
        super().__init__(f"{where}: {L.iris_strerror(code).decode()} ({code}): {msg}")
        self.code = code


def check(rc: int, where: str):
    if rc != 0:
        raise IrisError(rc, where)
