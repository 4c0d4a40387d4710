"""The C-ABI library builds, loads and exports every entry point of
include/iris_fdtd.h; without a GPU the engine refuses loudly."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden


def header_functions():
    src = open(os.path.join(ROOT, "include", "iris_fdtd.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(iris_[a-z_0-9]+)\s*\(", src)))


def test_exports_match_header(iris):
    L = iris.lib()
    names = header_functions()
    assert len(names) >= 18
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(iris.native.EXPORTS)


def header_constants():
    """Integer macros of the header: IRIS_NAME -> value (status codes in
    parentheses included)."""
    src = open(os.path.join(ROOT, "include", "iris_fdtd.h")).read()
    return {m.group(1): int(m.group(2)) for m in re.finditer(r"^#define IRIS_([A-Z0-9_]+)\s+\(?(-?\d+)\)?", src, re.M)}


def test_python_constants_match_header(iris):
    """The Python mirror's constants carry the header's values: every
    IRIS_<NAME> the module also defines as <NAME>, the kernel classes'
    order (IRIS_KC_*) and the batch's work lists (IRIS_BATCH_NTILES)."""
    c = header_constants()
    matched = [n for n in c if hasattr(iris, n)]
    for n in matched:
        assert getattr(iris, n) == c[n], n
    for n in ("FP64", "FP32", "STENCIL_DEFAULT", "STENCIL_PERSISTENT", "PERSISTENT_MAX_CELLS",
              "PERSISTENT_MAX_CELLS_FP32", "DFT_KERNEL_TENSOR", "DFT_Z", "OP_BARRIER_CHECK", "E", "H"):
        assert n in matched, n
    assert c["EINVAL"] == -1 and c["ETIMEOUT"] == -7
    kc = {"update_e": "KC_E", "update_h": "KC_H", "tfsf": "KC_TFSF", "dft_gather": "KC_GATHER",
          "dft_block": "KC_DFT", "flux": "KC_FLUX", "fused_eh": "KC_FUSED", "persistent": "KC_PERSIST"}
    assert len(iris.Engine.KERNELS) == c["NKC"]
    for i, k in enumerate(iris.Engine.KERNELS):
        assert c[kc[k]] == i, k
    assert len(iris.TILES) == c["BATCH_NTILES"]


def test_bounds_checking_twin_exports_the_same_entry_points(iris):
    """libiris_fdtd_bc.so (built with -DIRIS_BOUNDS_CHECK beside the ordinary
    library) loads and exports every header function; the ordinary library
    reports that it does not check and has nothing recorded (no device
    call)."""
    iris.lib()  # builds both when stale
    bc = ctypes.CDLL(iris.native.LIB_BC)
    for n in header_functions():
        assert hasattr(bc, n), n
    v = ctypes.c_ulonglong(7)
    plain = ctypes.CDLL(iris.native.LIB_PLAIN)
    plain.iris_bounds_check.argtypes = [ctypes.POINTER(ctypes.c_ulonglong)]
    assert plain.iris_bounds_check(ctypes.byref(v)) == 0 and v.value == 0


def test_strerror(iris):
    L = iris.lib()
    assert L.iris_strerror(0) == b"success"
    assert L.iris_strerror(-4) == b"invalid input file"


def test_struct_layout_matches_header(iris):
    # the ctypes mirror and the C struct agree field by field: round-trip through the C parser
    p, fw, _ = iris.setparam(golden("example_2.inputFDTD.dat"))
    assert (p.nx, p.ny, p.nz, p.nof, p.aix, p.afx) == (100, 1, 400, 500, 41, 60)
    assert p.tfsf_zf == 110 and p.precision == 0 and p.device == 0


def test_no_gpu_means_error_not_fallback(iris):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    p, fw, _ = iris.setparam(golden("example_1.inputFDTD.dat"))
    with pytest.raises(iris.IrisError) as e:
        iris.Engine(p, fw)
    assert e.value.code in (-8, -3)
    # the batched and gradient forms refuse the same way
    with pytest.raises(iris.IrisError) as e:
        iris.Batch([p, p.copy()], fw, dft_faces=iris.DFT_Z)
    assert e.value.code in (-8, -3)
    with pytest.raises(iris.IrisError) as e:
        iris.Adjoint(p, fw, (1, 1, 1, 1, p.hi, p.hi + 2))
    assert e.value.code in (-8, -3)


def test_invalid_parameters_rejected(iris):
    p, fw, _ = iris.setparam(golden("example_1.inputFDTD.dat"))
    q = p.copy()
    q.pmlzi = 1  # set_sz would divide by zero
    with pytest.raises(iris.IrisError) as e:
        iris.Engine(q, fw)
    assert e.value.code == -1
    q = p.copy()
    q.box1[5] = q.nz + 1
    with pytest.raises(iris.IrisError) as e:
        iris.Engine(q, fw)
    assert e.value.code == -1


C_CLIENT = r"""
#include <stdio.h>
#include <string.h>
#include "iris_fdtd.h"

int main(int argc, char** argv) {
  iris_params p;
  double fw[1024];
  char desc[256];
  int rc = iris_setparam(argv[1], 1, &p, fw, 1024, desc, sizeof desc);
  if (rc != IRIS_OK) { printf("setparam %d %s\n", rc, iris_last_error()); return 1; }
  printf("grid %d %d %d nof %d texit %d\n", p.nx, p.ny, p.nz, p.nof, p.texit);
  iris_engine* e = NULL;
  rc = iris_create(&p, fw, &e);
  printf("create %d %s\n", rc, rc == IRIS_OK ? "ok" : iris_strerror(rc));
  if (rc == IRIS_OK) iris_destroy(e);
  return 0;
}
"""


def test_c_client_links_and_fails_loudly_without_gpu(iris, tmp_path):
    """The header is plain C99: a C host (as a Fortran iso_c_binding host
    would) compiles against it, links the library, parses a reference deck,
    and gets a status code, not a crash or a CPU fallback, when no GPU is
    there (IRIS_OK when one is)."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        pytest.skip("no C compiler")
    lib = iris.build()
    src = tmp_path / "client.c"
    src.write_text(C_CLIENT)
    exe = tmp_path / "client"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe), lib, "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    out = subprocess.run([str(exe), golden("example_1.inputFDTD.dat")], capture_output=True, text=True, check=True)
    lines = out.stdout.splitlines()
    assert lines[0] == "grid 1 1 400 nof 500 texit 25962", lines
    code = int(lines[1].split()[1])
    try:
        import torch
        gpu = torch.cuda.is_available()
    except ImportError:
        gpu = False
    assert code == 0 if gpu else code in (-8, -3), lines


def test_noalloc_refusals_touch_no_device(iris):
    """iris_dft_block_noalloc checks every argument before any CUDA call:
    null or misaligned pointers and blocks beyond the fixed scratch are
    refused with IRIS_EINVAL (the addresses below are never dereferenced)."""
    L = iris.lib()
    a8, a16 = 0x10000, 0x20000
    call = L.iris_dft_block_noalloc
    assert call(None, 1, 1, 0, 1, a8, 1, 1.0, a16, None) == -1
    assert b"null" in L.iris_last_error()
    assert call(a8, 0, 1, 0, 1, a8, 1, 1.0, a16, None) == -1
    assert call(a8 + 4, 1, 1, 0, 1, a8, 1, 1.0, a16, None) == -1
    assert b"aligned" in L.iris_last_error()
    assert call(a8, 1, 1, 0, 1, a8 + 2, 1, 1.0, a16, None) == -1
    assert call(a8, 1, 1, 0, 1, a8, 1, 1.0, a16 + 8, None) == -1
    assert b"aligned" in L.iris_last_error()
    assert call(a8, 65537, 1, 0, 1, a8, 1, 1.0, a16, None) == -1
    assert b"exceeds" in L.iris_last_error()
