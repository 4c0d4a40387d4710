"""Workload definitions and geometry front-end.

* ``write_input`` writes an inputFDTD.dat with the reference's section layout
  (the file setparam() reads, code/files.f90:39-344).
* ``WORKLOADS`` restates the five named benchmark workloads as run
  parameters: grid, UPML, structure, source, DFT planes and step count.
  Shared choices: cell q = 5 nm; Courant number S = c0*dt/Q = 0.5, i.e.
  CFL = 0.5*sqrt(3) in the reference's convention dt = CFL*Q/(c0*sqrt(3))
  (code/files.f90:88); pulse centre 0.05 cycles/step, i.e. wavelength
  S*q/0.05 = 50 nm; 60-step pulse width, i.e. pump_DT = 60*dt with
  def_pulse = 4 (Gpump = 7.5 cells); wavelength grid lno = 0.75*lambda0,
  dlambda = 0.75*lambda0/nof; i_pol = 2, complex source, wzPML = 0.09; the
  simulated time is (N + 0.5)*dt so that int() truncation gives exactly N
  steps (code/files.f90:142).
* ``spheres_material``, ``binary_pattern_material``, ``design_region_material``:
  seeded voxelisers that build eps_inv over (hi-1:hf+1, 0:ny+1, 0:nx+1), the
  array slit() fills in the reference (code/mesh.f90:57-69).  The engine
  builds the same arrays on the device (iris_material_spheres,
  iris_material_pattern, iris_material_design), value for value: the
  spheres' parameters are drawn here (``sphere_params``) and passed, the
  per-voxel draws of the patterns and design regions are the i-th outputs of
  a SplitMix64 stream started at the seed (``splitmix_uniform``), which both
  sides compute from the voxel's index.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

Q_NM = 5.0
COURANT = 0.5
CFL = COURANT * math.sqrt(3.0)
LAMBDA0 = COURANT * Q_NM / 0.05  # 50 nm


@dataclass
class Workload:
    name: str
    nx: int
    ny: int
    nz: int
    pmlzi: int
    pmlzf: int
    hi: int
    dh: int
    eps_bbox: float
    dx: int
    tfsf_zi: int
    box: tuple  # sxi sxf syi syf szi szf
    nof: int
    nsteps: int
    eps1: float = 1.0
    eps3: float = 1.0
    akx: float = 0.0
    aky: float = 0.0
    structure: str = "slab"  # slab | slit | spheres | pattern | design
    extra: dict = field(default_factory=dict)

    @property
    def cells(self) -> int:
        return self.nx * self.ny * self.nz


def _dt_fs(q_nm: float, cfl: float, single_literals: bool = True) -> float:
    # dt in fs exactly as the reference forms it (code/files.f90:81-88, physconst.f90)
    f32 = (lambda v: float(np.float32(v))) if single_literals else float
    c0 = f32(137.0360)
    f_abohr = float(np.float32(10) / np.float32(0.529177249)) if single_literals else 10 / 0.529177249
    uat = f32(24.188843265e-3)
    Q = f_abohr * q_nm
    dt = cfl / (c0 * math.sqrt(3.0 / (Q * Q)))
    return dt * uat


def write_input(path: str, w: Workload, description: str = "", no_downloads: int = 1,
                pulse_steps: float = 60.0, wlpump: float = LAMBDA0, q_nm: float = Q_NM, cfl: float = CFL,
                sample_fourier: int = 1, to_fourier: int = 0, plane_wave: int = 1, i_pol: int = 2,
                cosine: int = 0, epump: float = 1.0, lno: float | None = None, dlamda: float | None = None):
    dtfs = _dt_fs(q_nm, cfl)
    itmax_fs = (w.nsteps + 0.5) * dtfs
    pump_dt_fs = pulse_steps * dtfs
    lno = 0.75 * wlpump if lno is None else lno
    dlamda = 0.75 * wlpump / w.nof if dlamda is None else dlamda
    b = w.box
    lines = [
        description or f"{w.name}: synthetic workload",
        "",
        '"Mesh options"',
        f"{i_pol}        i_pol",
        f"{q_nm!r}      q (nm)",
        f"{w.nx}        ixmax",
        f"{w.ny}        iymax",
        f"{w.nz}        izmax",
        f"{cfl!r}       CFL",
        "0.09     wzPML",
        "2        nPML line (pml_taflove)",
        f"{w.pmlzi}     pmlzi",
        f"{w.pmlzf}     pmlzf",
        "",
        '"Source options"',
        f"{plane_wave}        plane_wave",
        "20.0 180.0   tincr_PW,tdecay_PW (fs)",
        f"{epump!r} {wlpump!r} {pump_dt_fs!r} 4    Epump(kV/cm) wavelength(nm) width(fs) def_pulse",
        f"{w.tfsf_zi}       tfsf_zi",
        f"{cosine}        cosine",
        "",
        '"Job options"',
        f"{no_downloads} 1000    no_downloads,OUTPUT_TIME_STEP",
        f"{itmax_fs!r}    itmax (fs)",
        f"{w.hi}     hi",
        "0 0 0    SDL planes",
        "",
        '"Dielectric constants"',
        f"{w.eps1!r}    eps cover",
        f"{w.eps_bbox!r}    eps_bbox",
        f"{w.eps3!r}    eps substrate",
        "",
        '"Fourier transformation options"',
        f"{b[0]} {b[0]}   sxi mxi",
        f"{b[1]} {b[1]}   sxf mxf",
        f"{b[2]} {b[2]}   syi myi",
        f"{b[3]} {b[3]}   syf myf",
        f"{b[4]} {b[4]}   szi mzi",
        f"{b[5]} {b[5]}   szf mzf",
        f"{w.nof}      nof",
        f"{dlamda!r}   dlambda (nm)",
        f"{lno!r}   lno (nm)",
        f"{to_fourier} {sample_fourier}    to_Fourier,sample_Fourier",
        "",
        '"Slit Array"',
        f"{w.dh}     Dh",
        f"{w.dx}     dx",
        "",
    ]
    with open(path, "w") as fh:
        fh.write("\n".join(lines))
    return path


def workload(n: int, **over) -> Workload:
    """The named workloads 1..5 (5 adjoint form, 4 batched form: one cell)."""
    if n == 1:
        w = Workload("slab_4x4x512_fp64", 4, 4, 512, 16, 497, 236, 40, 2.25, 0, 40, (1, 4, 1, 4, 30, 480), 200, 4000)
    elif n == 2:
        w = Workload("slit_256x4x768", 256, 4, 768, 16, 753, 344, 80, 4.0, 64, 40, (1, 256, 1, 4, 30, 738), 300,
                     8000, structure="slit")
    elif n == 3:
        w = Workload("spheres_512x512x1024", 512, 512, 1024, 24, 1001, 412, 200, 1.0, 0, 48,
                     (1, 512, 1, 512, 36, 988), 300, 10000, akx=0.3 * math.pi * 512, structure="spheres",
                     extra=dict(nspheres=200, rmin=8, rmax=32, emin=1.5, emax=6.0))
    elif n == 5:
        w = Workload("adjoint_160x160x512", 160, 160, 512, 16, 497, 241, 32, 1.0, 0, 40, (1, 160, 1, 160, 30, 482),
                     64, 6000, structure="design", extra=dict(x0=17, x1=144, y0=17, y1=144, emin=1.0, emax=12.0))
    else:
        raise ValueError("workload 4 is the batched form: use batch_cells()")
    for k, v in over.items():
        setattr(w, k, v)
    return w


def resized(w: Workload, nx: int, ny: int, nz: int, nof: int | None = None) -> Workload:
    """The same workload on another grid: UPML thickness, TF/SF plane and DFT
    planes keep their distance to the z ends, the structure layer keeps its
    relative position and thickness (used for small profiling cases)."""
    f = nz / w.nz
    hi = max(w.tfsf_zi + 8, int(round(w.hi * f)))
    dh = max(1, int(round(w.dh * f)))
    box = (1, nx, 1, ny, w.box[4], nz - (w.nz - w.box[5]))
    out = Workload(f"{w.name}_as_{nx}x{ny}x{nz}", nx, ny, nz, w.pmlzi, nz - (w.nz - w.pmlzf), hi, dh, w.eps_bbox, 0,
                   w.tfsf_zi, box, nof or w.nof, w.nsteps, w.eps1, w.eps3, 0.3 * math.pi * nx if w.akx else 0.0,
                   w.aky, w.structure, dict(w.extra))
    return out


def batch_cells(ncells: int = 256, seed: int = 0, nsteps: int = 6000, nof: int = 128):
    """Batched form: ncells independent Bloch cells of uneven size, cell i
    seeded with seed+i: nx, ny ~ U{32..160}, nz ~ U{256..768}, UPML 16,
    a 64-cell layer centred in z holding a binary eps in {1, 4} pattern."""
    out = []
    for i in range(ncells):
        r = np.random.default_rng(seed + i)
        nx, ny = int(r.integers(32, 161)), int(r.integers(32, 161))
        nz = int(r.integers(256, 769))
        hi = nz // 2 - 32
        w = Workload(f"cell{i}", nx, ny, nz, 16, nz - 15, hi, 64, 1.0, 0, 40, (1, nx, 1, ny, 30, nz - 30), nof,
                     nsteps, structure="pattern", extra=dict(seed=seed + i, fill=float(r.uniform(0.3, 0.7))))
        out.append(w)
    return out


# ---------------------------------------------------------------------------
# voxelisers: eps_inv over (hi-1:hf+1, 0:ny+1, 0:nx+1) as complex [z, y, x]

def _base(w: Workload) -> np.ndarray:
    hf = w.hi + w.dh - 1
    a = np.full((hf - w.hi + 3, w.ny + 2, w.nx + 2), 1.0 / w.eps_bbox, dtype=np.complex128)
    a[0] = 1.0 / w.eps1
    a[-1] = 1.0 / w.eps3
    return a


def slit_material(w: Workload) -> np.ndarray:
    a = _base(w)
    if w.dx > 0:
        n, d = w.nx, w.dx
        if d % 2 == 0:
            ai, af = (n // 2 - (d // 2 - 1), n // 2 + d // 2) if n % 2 == 0 else ((n + 1) // 2 - d // 2, (n + 1) // 2 + d // 2 - 1)
        else:
            ai, af = (n // 2 - ((d + 1) // 2 - 1), n // 2 + (d - 1) // 2) if n % 2 == 0 else ((n + 1) // 2 - (d - 1) // 2, (n + 1) // 2 + (d - 1) // 2)
        a[1:-1, :, ai:af + 1] = 1.0
    return a


SPLITMIX_GAMMA = 0x9E3779B97F4A7C15


def splitmix_uniform(seed: int, idx) -> np.ndarray:
    """The idx-th outputs (idx >= 0) of a SplitMix64 generator started at seed,
    as doubles in [0, 1): state = seed + (idx + 1) * 0x9E3779B97F4A7C15, mixed
    by SplitMix64's finaliser, top 53 bits scaled by 2^-53."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + (np.asarray(idx, dtype=np.uint64) + np.uint64(1)) * \
            np.uint64(SPLITMIX_GAMMA)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def sphere_params(w: Workload, seed: int = 0) -> np.ndarray:
    """The nspheres seeded spheres as rows (cx, cy, cz, radius, eps): radius
    ~U[rmin,rmax] cells, eps ~U[emin,emax], centres in the layer."""
    ex = w.extra
    hf = w.hi + w.dh - 1
    r = np.random.default_rng(seed)
    out = np.empty((int(ex["nspheres"]), 5))
    for i in range(out.shape[0]):
        out[i, 0] = r.uniform(1, w.nx)
        out[i, 1] = r.uniform(1, w.ny)
        out[i, 2] = r.uniform(w.hi, hf)
        out[i, 3] = r.uniform(ex["rmin"], ex["rmax"])
        out[i, 4] = r.uniform(ex["emin"], ex["emax"])
    return out


def spheres_material(w: Workload, seed: int = 0) -> np.ndarray:
    """nspheres seeded spheres (sphere_params), periodic in x and y, later
    spheres win: a cell takes 1/eps of the last sphere whose closed ball,
    over the sphere's bounding box of at most nx by ny cells, holds it."""
    a = _base(w)
    hf = w.hi + w.dh - 1
    for cx, cy, cz, rad, eps in sphere_params(w, seed):
        z = np.arange(max(w.hi, math.floor(cz - rad)), min(hf, math.ceil(cz + rad)) + 1)
        if z.size == 0:
            continue
        # bounding box in x and y, wrapped onto the periodic cell (2r < n)
        x = np.arange(math.floor(cx - rad), math.ceil(cx + rad) + 1)
        y = np.arange(math.floor(cy - rad), math.ceil(cy + rad) + 1)
        x, y = x[: w.nx], y[: w.ny]
        inside = ((z[:, None, None] - cz) ** 2 + (y[None, :, None] - cy) ** 2 + (x[None, None, :] - cx) ** 2
                  <= rad * rad)
        zi = z - w.hi + 1
        yi = (y - 1) % w.ny + 1
        xi = (x - 1) % w.nx + 1
        sub = a[np.ix_(zi, yi, xi)]
        sub[inside] = 1.0 / eps
        a[np.ix_(zi, yi, xi)] = sub
    _wrap_ghosts(a)
    return a


PATTERN_SEED_OFFSET = 1_000_003


def pattern_seed(w: Workload) -> int:
    return int(w.extra["seed"]) + PATTERN_SEED_OFFSET


def binary_pattern_material(w: Workload) -> np.ndarray:
    """Voxelwise Bernoulli(fill) eps in {1, 4} over the layer: voxel (z, y, x) of
    the layer, flat index i = ((z - hi) * ny + y - 1) * nx + x - 1, is eps 4
    when the i-th SplitMix64 draw of pattern_seed(w) is below fill."""
    ex = w.extra
    a = _base(w)
    u = splitmix_uniform(pattern_seed(w), np.arange(w.dh * w.ny * w.nx)).reshape(w.dh, w.ny, w.nx)
    a[1:-1, 1:-1, 1:-1] = np.where(u < ex["fill"], 1.0 / 4.0, 1.0)
    _wrap_ghosts(a)
    return a


def design_region_material(w: Workload, seed: int = 0) -> np.ndarray:
    """Continuous eps ~U[emin,emax] over the design region, 1 elsewhere: voxel
    (z, y, x) of the region, flat index i in its own (z, y, x) order, has
    eps = emin + (emax - emin) * the i-th SplitMix64 draw of seed."""
    ex = w.extra
    a = _base(w)
    shape = (w.dh, ex["y1"] - ex["y0"] + 1, ex["x1"] - ex["x0"] + 1)
    u = splitmix_uniform(seed, np.arange(int(np.prod(shape)))).reshape(shape)
    eps = ex["emin"] + (ex["emax"] - ex["emin"]) * u
    a[1:-1, ex["y0"]:ex["y1"] + 1, ex["x0"]:ex["x1"] + 1] = 1.0 / eps
    return a


def _wrap_ghosts(a: np.ndarray):
    a[1:-1, :, 0] = a[1:-1, :, -2]
    a[1:-1, :, -1] = a[1:-1, :, 1]
    a[1:-1, 0, :] = a[1:-1, -2, :]
    a[1:-1, -1, :] = a[1:-1, 1, :]


def material(w: Workload) -> np.ndarray:
    if w.structure == "spheres":
        return spheres_material(w)
    if w.structure == "pattern":
        return binary_pattern_material(w)
    if w.structure == "design":
        return design_region_material(w)
    return slit_material(w)


def make_run(w: Workload, directory: str, **kw) -> str:
    os.makedirs(directory, exist_ok=True)
    return write_input(os.path.join(directory, "inputFDTD.dat"), w, **kw)
