"""The bounds-checking build (libiris_fdtd_bc.so, -DIRIS_BOUNDS_CHECK): every
kernel that maps its threads to cells, slab rows, TF/SF rows, DFT points or
flux faces checks the index against its range and records the first one
outside it in a device word (iris_bounds_check).  The odd sizes the parity
tests use (1x1xN columns, 37x21 partial tiles, the thinnest UPML the
parameters allow, a 40x1 cell, uneven batch cells) run through every
stepping path (split, persistent, fused, streamed; FP64 and FP32; all faces
and z faces; the tensor-core DFT's commit and flux read; the batch's work
lists) in a child process that loads the checking build, and the word must
stay clean.  Nothing here is meant to go out of range: the checks only
record and skip, they never fault.
"""
import os
import subprocess
import sys
import textwrap

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent('''
    import importlib, os, sys, tempfile
    sys.path.insert(0, sys.argv[1])
    iris = importlib.import_module("irisfdtd-academic_gb300")
    cfg = importlib.import_module("irisfdtd-academic_gb300.configs")
    enabled, first = iris.bounds_check()
    assert enabled, "the checking build was not loaded"
    assert first is None, first
    d = tempfile.mkdtemp()
    W = cfg.Workload
    CASES = [
        ("col", W("col", 1, 1, 120, 12, 109, 50, 20, 9.0, 0, 20, (1, 1, 1, 1, 15, 100), 11, 40), {}, 0.0, "slab"),
        ("sph", W("sph", 37, 21, 64, 8, 57, 24, 14, 2.25, 0, 12, (1, 37, 1, 21, 9, 54), 9, 40, structure="spheres",
                  extra=dict(nspheres=6, rmin=2, rmax=5, emin=1.5, emax=6.0)), {"i_pol": 1}, 0.4, "spheres"),
        ("thin", W("thin", 19, 3, 40, 2, 39, 10, 6, 4.0, 0, 6, (1, 19, 1, 3, 4, 36), 7, 40, structure="slit"), {},
         0.0, "slit"),
        ("row", W("row", 40, 1, 64, 8, 57, 26, 10, 4.0, 0, 14, (1, 40, 1, 1, 10, 54), 9, 40), {}, -0.3, "slab"),
    ]
    runs = 0
    for name, w, kw, akx, kind in CASES:
        p, fw, _ = iris.setparam(cfg.write_input(os.path.join(d, name + ".dat"), w, no_downloads=2, **kw))
        p.akx_re = akx
        eps = cfg.spheres_material(w, seed=3) if kind == "spheres" else cfg.slit_material(w)
        for prec in (iris.FP64, iris.FP32):
            for st in (iris.STENCIL_SPLIT, iris.STENCIL_PERSISTENT, iris.STENCIL_FUSED, iris.STENCIL_STREAM):
                for faces in (iris.DFT_ALL, iris.DFT_Z):
                    q = p.copy()
                    q.dft_faces = faces
                    try:
                        e = iris.Engine(q, fw, precision=prec, stencil=st, dft_block=16)
                    except iris.IrisError:
                        continue  # a combination the engine refuses (fused/streamed are FP32 only)
                    e.set_material(eps)
                    e.step(1, 23)
                    e.flux(0)
                    e.dft_commit()
                    e.step(24, 9)
                    e.flux(0)
                    e.close()
                    runs += 1
                    en, first = iris.bounds_check()
                    assert first is None, (name, prec, st, faces, first)
    # the batch's work lists over uneven cells
    cells = [(12, 7, 60, 8, 53, 24, 10, 14, (1, 12, 1, 7, 10, 50)), (33, 9, 48, 6, 43, 18, 8, 10, (1, 33, 1, 9, 8, 40)),
             (1, 1, 90, 10, 81, 40, 15, 16, (1, 1, 1, 1, 12, 78))]
    for prec in (iris.FP64, iris.FP32):
        params, mats = [], []
        for i, (nx, ny, nz, pi, pf, hi, dh, zi, box) in enumerate(cells):
            w = W("b%d" % i, nx, ny, nz, pi, pf, hi, dh, 1.0, 0, zi, box, 9, 40, structure="pattern",
                  extra=dict(seed=100 + i, fill=0.5))
            p, fw, _ = iris.setparam(cfg.write_input(os.path.join(d, "b%d.dat" % i), w, no_downloads=3))
            p.precision = prec
            params.append(p)
            mats.append(cfg.binary_pattern_material(w))
        for tile in range(len(iris.TILES)):
            b = iris.Batch(params, fw, dft_faces=iris.DFT_Z)
            for c, m in enumerate(mats):
                b.set_material(c, m)
            try:
                b.set_tile(tile)
            except iris.IrisError:
                b.close()
                continue  # the fused work list is FP32 only
            b.step(1, 21)
            for c in range(len(cells)):
                b.flux(c)
            b.close()
            runs += 1
            en, first = iris.bounds_check()
            assert first is None, ("batch", prec, tile, first)
    print("RUNS", runs)
''')


def test_bounds_checked_build_stays_clean():
    env = dict(os.environ, IRIS_BOUNDS_CHECK="1")
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    runs = int(r.stdout.split("RUNS")[1].split()[0])
    assert runs >= 40, r.stdout
