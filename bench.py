#!/usr/bin/env python3
"""Benchmark of the GB300 FDTD engine.

Workload: the 512x512x1024 Bloch cell (24-cell UPML in z, kx = 0.3*pi/dx, a
200-cell layer with 200 seeded dielectric spheres, TF/SF Gaussian pulse,
on-the-fly DFT at 300 frequencies on all six faces of the box, as the
reference accumulates them in 3D), FP32 fields with FP64 incident field and
FP64 DFT accumulation.  One bench step is one full time step of the hot path:
E update, UPML-E, Bloch, H update, UPML-H, Bloch, TF/SF, DFT sample, plus the
DFT accumulation.  The DFT buffer is empty when the clock starts and a flux
read ends the timed steps; on the FP32 tensor-core path that read adds the
samples still buffered on the fly and leaves them buffered, so the timed
time also carries their share of the commit they wait for (a full block's
commit is timed after the timed steps; its share is buffered / block).

Metric: Gcell/s = cells * steps / time.  `value` is device-timed (CUDA events
on the engine's stream) with the state resident in HBM; `e2e` goes through the
public API from host buffers (engine creation, material upload, the steps and
the flux read back).  `roofline` is for the dominant pass (the fused E+H pass
in FP32, the slower split pass otherwise): algorithmic bytes per pass over
its event-timed duration; `dft` reports the DFT's own work apart from it.
The default line also carries the batched form (256 uneven cells) as `batch`.

--impl reference times the CPU restatement of the reference (the oracle; the
Fortran reference has no compiler here) on the host cores, on a bounded
column of the same workload, and scales its per-cell and per-DFT-point costs
to the full workload (marked "extrapolated").
"""
import argparse
import glob
import importlib
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG = "irisfdtd-academic_gb300"
METRIC = "Gcell/s (E+H Yee step) & %HBM peak, FP32/batched vs FP64 plain, T/R err<=1e-4"


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Dist:
    """Host-side barrier and max-reduction across replicas (gloo; no data-path collective)."""

    def __init__(self, world):
        self.world = world
        self.dist = None
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, v):
        if not self.dist:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


# ---------------------------------------------------------------------------
# clocks during the timed region

CLK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def start_clocks(device):
    try:
        f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        pr = subprocess.Popen(["nvidia-smi", f"--query-gpu={CLK_FIELDS}", "--format=csv,noheader,nounits",
                               "-lms", "200", "-i", str(device)], stdout=f, stderr=subprocess.DEVNULL)
        return pr, f.name
    except Exception:
        return None, None


def stop_clocks(pr, path):
    if pr is None:
        return None
    pr.terminate()
    try:
        pr.wait(timeout=5)
    except Exception:
        pr.kill()
    sm, mx, reasons = [], None, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    try:
        for line in open(path):
            v = [x.strip() for x in line.split(",")]
            if len(v) < 9:
                continue
            try:
                sm.append(float(v[1]))
                mx = float(v[2])
            except ValueError:
                continue
            for n, x in zip(names, v[5:9]):
                if x.lower() in ("active", "1"):
                    reasons.add(n)
        os.unlink(path)
    except OSError:
        pass
    if not sm:
        return None
    return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------

def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kernel, workload):
    """DRAM bytes per pass (per launch for a one-launch pass) from a committed
    ncu summary, if one exists."""
    for f in glob.glob(os.path.join(ROOT, "profiles", "*.json")):
        try:
            d = json.load(open(f))
        except Exception:
            continue
        if d.get("kernel") != kernel or d.get("workload") != workload:
            continue
        for key in ("dram_bytes_per_pass", "dram_bytes_per_launch"):
            if key in d:
                return float(d[key]), os.path.relpath(f, ROOT)
    return None, None


def cfg_mod():
    return importlib.import_module(PKG + ".configs")


def setup_workload(n, rank=0, grid=None, nof=None):
    cfg = importlib.import_module(PKG + ".configs")
    w = cfg.workload(n)
    if grid:
        w = cfg.resized(w, *grid, nof=nof)
    # replicas sweep the Bloch phase (independent k-points)
    w.akx = w.akx + 0.01 * rank
    t = time.perf_counter()
    eps = cfg.material(w)
    t_mat = time.perf_counter() - t
    d = tempfile.mkdtemp(prefix="iris_bench_")
    path = cfg.write_input(os.path.join(d, "inputFDTD.dat"), w)
    return w, path, eps, t_mat


def algorithmic_bytes(w, p, sc, sm):
    """Per launch of the E and H updates: 9 complex values per cell (read own
    field, read the other field, write own field, 3 components), the real
    inverse permittivity per structure cell (E only), and the UPML auxiliary
    read+write per PML cell (3 complex each way)."""
    cells = w.nx * w.ny * w.nz
    npml = w.nx * w.ny * (p.pmlzi + (p.nz - p.pmlzf + 1))
    nstruct = w.nx * w.ny * (p.hf - p.hi + 1)
    e = cells * 9 * sc + nstruct * sm + npml * 6 * sc
    h = cells * 9 * sc + npml * 6 * sc
    return e, h


def dft_accounting(P, nof, kblock, sc, K, kms, kn, buffered, flux_points, commit_ms):
    """The DFT's own work over the K timed steps, apart from the stencil's.

    Every step gathers its P face samples into the ring (P x sc bytes
    written).  A commit accumulates the ring into the FP64 accumulators: it
    reads and writes all of them (2 x P x nof x 16 bytes) and reads the ring.
    The flux read that ends the timed steps reads the four flux components'
    accumulators (flux_points x nof x 16 bytes) and, on the tensor-core path,
    adds the `buffered` samples not yet committed on the fly.  The bytes
    below are those of the commits and flux reads that ran inside the timed
    region; `commit` is one full block's commit measured after it, whose
    share for the buffered samples (buffered / kblock of it) the timed
    region's value includes."""
    ncommit, nflux = kn["dft_block"], kn["flux"]
    acc_commit = ncommit * 2.0 * P * nof * 16
    ring_commit = (K - buffered) * P * sc  # every committed sample was gathered inside the window
    acc_flux = nflux * flux_points * nof * 16.0
    ring_flux = nflux * buffered * flux_points * sc
    out = {"points": P, "frequencies": nof, "block_samples": kblock, "timed_steps": K,
           "complex_macs_per_step": P * nof, "commits_in_window": ncommit, "flux_reads_in_window": nflux,
           "samples_left_buffered": buffered,
           "accumulator_bytes_per_step": int(round((acc_commit + acc_flux) / K)),
           "ring_bytes_per_step": P * sc,
           "block_ms_per_step": round(kms["dft_block"] / K, 4), "flux_ms_per_step": round(kms["flux"] / K, 4),
           "gather_ms_per_step": round(kms["dft_gather"] / K, 4)}
    if kms["dft_block"] > 0 and ncommit:
        out["block_gbs"] = round((acc_commit + ring_commit) / (kms["dft_block"] * 1e-3) / 1e9, 1)
    if kms["flux"] > 0 and nflux:
        out["flux_gbs"] = round((acc_flux + ring_flux) / (kms["flux"] * 1e-3) / 1e9, 1)
    if kms["dft_gather"] > 0:
        out["gather_gbs"] = round(2.0 * K * P * sc / (kms["dft_gather"] * 1e-3) / 1e9, 1)
    if commit_ms:
        full = 2.0 * P * nof * 16 + kblock * P * sc
        out["commit"] = {"block_samples": kblock, "ms": round(commit_ms, 3),
                         "gbs": round(full / (commit_ms * 1e-3) / 1e9, 1),
                         "share_ms_in_value": round(commit_ms * buffered / kblock, 4),
                         "what": ("one commit of a full block of samples, timed by CUDA events after the timed "
                                  "steps; the value's time includes its share for the samples the timed steps "
                                  "left buffered")}
    return out


def full_block_commit(eng, it, kb, buffered):
    """Steps on from it until the DFT buffer (buffered samples in it) is full and
    commits: the device time of that one commit of kb samples (ms)."""
    eng.timing_start(per_kernel=True)
    eng.step(it, kb - buffered)
    _, kc, nc = eng.timing_read()
    assert nc["dft_block"] == 1 and eng.info()["dft_buffered"] == 0, (nc, eng.info())
    return kc["dft_block"], it + kb - buffered


def flux_points(info):
    """Sample points one flux read touches: the four flux components of every
    face location of one box (P counts six components per location)."""
    return info["dft_points"] * 4 // 6 // max(1, info["boxes"])


def run_engine(args, rank, world, local):
    iris = importlib.import_module(PKG)
    D = Dist(world)
    w, path, eps, t_mat = setup_workload(args.workload, rank, args.grid, args.nof)
    p, fw, _ = iris.setparam(path)
    p.akx_re = w.akx
    p.device = local
    prec = iris.FP32 if args.precision == "fp32" else iris.FP64
    cells = w.nx * w.ny * w.nz
    K, W = args.steps, args.warmup
    if np.iscomplexobj(eps) and not np.any(eps.imag):
        eps = np.ascontiguousarray(eps.real)  # a lossless material crosses the API as a real array

    # the process's CUDA context and the kernels' modules come up once, on a
    # small engine of the same configuration, before the end-to-end clock;
    # 16 x 16 columns keep it above the persistent kernel's cell limit, so it
    # steps with the kernels the full grid uses
    warm_p = p.copy()
    warm_p.nx, warm_p.ny = min(p.nx, 16), min(p.ny, 16)
    for box in (warm_p.box1, warm_p.box2):  # x and y bounds of the DFT box inside the small grid
        box[0], box[1], box[2], box[3] = 1, warm_p.nx, 1, warm_p.ny
    warm_p.aix, warm_p.afx = 1, 0  # no slit
    wq = iris.Engine(warm_p, fw, precision=prec, dft_block=args.dft_block, device=local, stencil=args.stencil,
                     graph=args.graph, dft_kernel=args.dft_kernel)
    wq.step(1, 4)
    wq.flux(0)
    wq.close()

    # --- end to end through the public API, host buffers in and out
    D.barrier()
    t0 = time.perf_counter()
    eng = iris.Engine(p, fw, precision=prec, dft_block=args.dft_block, device=local, stencil=args.stencil,
                      graph=args.graph, dft_kernel=args.dft_kernel)
    if w.structure == "spheres":
        # the geometry crosses the API as the spheres' parameters; the engine voxelises them
        sph = cfg_mod().sphere_params(w)
        eng.material_spheres(sph)
        h2d = sph.nbytes + fw.size * 8
        mat_what = "iris_material_spheres (%d spheres, voxelised on the device)" % sph.shape[0]
    else:
        eng.set_material(eps)
        h2d = eps.size * eps.itemsize + fw.size * 8
        mat_what = "iris_set_material (host eps)"
    eng.step(1, K)
    J = eng.flux(0)
    t_e2e = time.perf_counter() - t0
    info = eng.info()
    buffered_e2e = info["dft_buffered"]
    d2h = J.size * 8

    # --- device-timed steady state: the DFT buffer is empty when the clock
    # starts; the flux read that ends the timed steps accumulates every timed
    # sample (on the tensor-core path it adds the samples still buffered on
    # the fly and leaves them buffered, so the share of their later commit is
    # measured below and added to the timed region)
    it = K + 1
    eng.step(it, W)
    it += W
    eng.dft_commit()
    eng.sync()
    D.barrier()
    pr, cpath = start_clocks(local)
    eng.timing_start(per_kernel=True)
    eng.step(it, K)
    eng.flux(0)
    win_ms, kms, kn = eng.timing_read()
    clocks = stop_clocks(pr, cpath)
    it += K
    buffered = eng.info()["dft_buffered"]
    commit_ms = 0.0
    if buffered or buffered_e2e:
        commit_ms, it = full_block_commit(eng, it, info["dft_block"], buffered)
    reg_ms = D.max(win_ms + commit_ms * buffered / info["dft_block"])
    t_e2e = D.max(t_e2e + commit_ms * 1e-3 * buffered_e2e / info["dft_block"])
    graph_line = None
    if args.graph:
        # the same steps replayed from captured graphs (per-kernel events off)
        eng.dft_commit()
        eng.timing_start(per_kernel=False)
        eng.step(it, K)
        reg_g, _, _ = eng.timing_read()
        it += K
        reg_g = D.max(reg_g)
        graph_line = {"value": round(world * cells * K / (reg_g * 1e-3) / 1e9, 3), "unit": "Gcell/s",
                      "ms_per_step": round(reg_g / K, 4),
                      "what": "device time of %d steps replayed as whole DFT blocks from one CUDA graph" % K}
    eng.close()

    sc, sm = (8, 4) if prec == iris.FP32 else (16, 8)
    eb, hb = algorithmic_bytes(w, p, sc, sm)
    hbm, src = peaks()
    fused = kn["fused_eh"] > 0
    persistent = kn["persistent"] > 0
    if persistent:
        # small grids: whole steps in one cooperative launch per span; its
        # time per step against both passes' algorithmic bytes (the fields
        # live in L2 there, so the fraction only says how far from a stream)
        t_p = kms["persistent"] / K * 1e-3
        dom, db, dt_ = "persistent", eb + hb, t_p
        t_e = t_h = t_p / 2
        min_bytes = db
    elif fused:
        # one fused pass per step (two concurrent launches: the planes outside the
        # UPML slabs and the slabs) does the whole E+H step: the algorithmic bytes of both passes
        t_f = kms["fused_eh"] / K * 1e-3
        dom, db, dt_ = "fused_eh", eb + hb, t_f
        t_e = t_h = t_f / 2
        # what one fused pass must move at least: read E,H and write E,H (12 complex per
        # cell), eps_inv in the structure, D read+write and B read+write in the PML
        npml = w.nx * w.ny * (p.pmlzi + (p.nz - p.pmlzf + 1))
        min_bytes = cells * 12 * sc + w.nx * w.ny * (p.hf - p.hi + 1) * sm + npml * 12 * sc
    else:
        t_e = kms["update_e"] / max(kn["update_e"], 1) * 1e-3
        t_h = kms["update_h"] / max(kn["update_h"], 1) * 1e-3
        dom, db, dt_ = ("update_h", hb, t_h) if t_h >= t_e else ("update_e", eb, t_e)
        min_bytes = db
    achieved = db / dt_ / 1e9
    wl_name = w.name
    traffic, tsrc = ncu_traffic(dom, w.name + "_" + args.precision)
    # one fused timer per step spans its launches: the planes outside the UPML
    # slabs and, concurrently, the slabs (one launch when no plane lies outside);
    # a commit is two launches (twiddles, block); a flux read on the tensor-core
    # path three (twiddles of the buffered samples, the tile partials, their sum)
    fused_launches = 2 if p.pmlzf - 2 >= p.pmlzi + 1 else 1
    dft_tc = prec == iris.FP32 and args.dft_kernel != iris.DFT_KERNEL_CUDA
    flux_launches = (3 if buffered else 2) if dft_tc else 1
    # a persistent span is one table launch (TF/SF variants) and one cooperative launch
    launches = kn["update_e"] + kn["update_h"] + kn["tfsf"] + kn["dft_gather"] + kn["flux"] * flux_launches + \
        kn["fused_eh"] * fused_launches + kn["dft_block"] * 2 + kn["persistent"] * 2
    value = world * cells * K / (reg_ms * 1e-3) / 1e9
    out = {
        "metric": METRIC,
        "value": round(value, 3),
        "unit": "Gcell/s",
        "n_gpus": world,
        "steps": K,
        "warmup": W,
        "ms_per_step": round(reg_ms / K, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("c64 fields (fp32), fp64 incident field, compensated fp32 (double-float) DFT accumulation"
                  if prec == iris.FP32 else "c128 (fp64)"),
        "data": ("synthetic (seeded spheres, numpy PCG64 seed 0)" if w.structure == "spheres"
                 else f"synthetic ({w.structure} geometry)"),
        "config": {
            "workload": wl_name,
            "grid": [w.nx, w.ny, w.nz], "upml": p.pmlzi, "nof": w.nof, "dft_points": info["dft_points"],
            "dft_block": info["dft_block"], "precision": args.precision,
            "dft_kernel": ["engine default", "cuda cores", "tensor cores (tcgen05 tf32x3)"][args.dft_kernel],
            "l2": l2_note(2 * 3 * info["comp_elems"] * info["bytes_per_complex"], info["dft_points"] * w.nof * 16),
            "parallelism": f"replicas x{world} (independent Bloch cells, one per GPU)",
        },
        "e2e": {"value": round(world * cells * K / t_e2e / 1e9, 3), "unit": "Gcell/s",
                "h2d_bytes_per_step": round(h2d / K, 1), "d2h_bytes_per_step": round(d2h / K, 1),
                "what": ("iris_create + %s + %d steps + iris_flux to host, in a process whose CUDA context was "
                         "started by a small engine before the clock; the DFT accumulators are first written "
                         "by the run's first commit (no zeroing pass), and a flux read before that commit "
                         "reads only the buffered samples" % (mat_what, K))},
        "gpu_launches": int(launches),
        "kernels_ms_per_step": {k: round(v / K, 4) for k, v in kms.items()},
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "peak_source": src,
                     "traffic": traffic, "traffic_source": tsrc,
                     "algorithmic_bytes_per_pass": db,
                     "min_bytes_per_pass": min_bytes,
                     "frac_of_min_bytes": round(min_bytes / dt_ / 1e9 / hbm, 4)},
        "window_ms_per_step": round(win_ms / K, 4),
        "stencil_gcells": round(cells / ((t_e + t_h)) / 1e9, 3),
        "dft": dft_accounting(info["dft_points"], w.nof, info["dft_block"], sc, K, kms, kn, buffered,
                              flux_points(info), commit_ms),
        "clocks": clocks,
        "material_setup_s": round(t_mat, 2),
    }
    if graph_line:
        out["graph"] = graph_line
    if rank == 0 and world == 1 and args.workload == 2 and not args.grid:
        out["tr_error"] = tr_error(iris, p, fw, eps, local)
    if rank == 0 and world == 1 and not args.no_fp64_compare and prec == iris.FP32:
        out["fp64_plain"] = fp64_compare(iris, p, fw, eps, cells, local)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(w, info["dft_points"], args.cpu_sample_steps)
    if args.workload == 3 and not args.grid and not args.no_batch and prec == iris.FP32:
        # the batched form (256 uneven cells) on the same GPU(s), same steps and warm-up
        bt = guarded(measure_batch, iris, args, rank, world, local, K, W, D)
        keys = ("value", "unit", "ms_per_step", "steps", "config", "e2e", "gpu_launches", "kernels_ms_per_step",
                "window_ms_per_step", "dft_commit", "roofline", "stencil_gcells", "clocks", "error")
        out["batch"] = {k: bt[k] for k in keys if k in bt}
    if args.workload == 3 and not args.grid and not args.no_configs and world == 1:
        # the other named workloads, each through the public API on this GPU
        out["slab_4x4x512_fp64"] = guarded(measure_tiny, iris, local)
        out["slit_256x4x768"] = guarded(measure_slit, iris, local)
        out["adjoint_160x160x512"] = guarded(measure_adjoint, iris, local, args.adjoint_fd_voxels)
    D.close()
    return out


def run_batch(args, rank, world, local):
    """The batched workload as its own bench line (--workload 4)."""
    iris = importlib.import_module(PKG)
    D = Dist(world)
    out = measure_batch(iris, args, rank, world, local, args.steps, args.warmup, D,
                        loop_sample=args.loop_sample if rank == 0 and world == 1 else 0)
    D.close()
    return out


def measure_batch(iris, args, rank, world, local, K, W, D, loop_sample=0):
    """The batched workload: 256 independent Bloch cells of uneven size (seed+i per cell),
    FP32 fields, FP64 DFT at 128 frequencies on the reflection and transmission
    planes, all cells stepped by one launch per operator.  Timing as for the
    single engine: the DFT buffer empty when the clock starts, K steps and a
    flux read, plus the share of the buffered samples' later commit (one full
    block's commit, measured after the timed steps)."""
    cfg = importlib.import_module(PKG + ".configs")
    ncells = args.cells
    ws = cfg.batch_cells(ncells, seed=1000 * rank, nof=128)
    d = tempfile.mkdtemp(prefix="iris_batch_")
    params = []
    for i, w in enumerate(ws):
        p, fw, _ = iris.setparam(cfg.write_input(os.path.join(d, f"c{i}.dat"), w))
        p.device = local
        params.append(p)
    cells = sum(w.cells for w in ws)
    D.barrier()
    t0 = time.perf_counter()
    b = iris.Batch(params, fw, precision=iris.FP32, dft_faces=iris.DFT_Z, device=local)
    for i, w in enumerate(ws):
        # each cell's binary pattern generated on the device from its seed and fill
        b.material_pattern(i, cfg.pattern_seed(w), w.extra["fill"], 4.0, 1.0)
    if args.tile is not None:
        b.set_tile(args.tile)
        tile, tune_ms = iris.TILES[args.tile], {}
    else:
        tile, tune_ms = b.tune(reps=2)
    b.step(1, K)
    J = [b.flux(i) for i in range(ncells)]
    t_e2e = time.perf_counter() - t0
    info = b.info()
    buffered_e2e = info["dft_buffered"]
    kb = info["dft_block"]
    it = K + 1
    b.step(it, W)
    it += W
    b.dft_commit()
    D.barrier()
    pr, cpath = start_clocks(local)
    b.timing_start(per_kernel=True)
    b.step(it, K)
    b.flux(0)
    win_ms, kms, kn = b.timing_read()
    clocks = stop_clocks(pr, cpath)
    it += K
    buffered = b.info()["dft_buffered"]
    commit_ms = 0.0
    if buffered or buffered_e2e:
        b.timing_start(per_kernel=True)
        b.step(it, kb - buffered)
        _, kc, nc = b.timing_read()
        assert nc["dft_block"] == 1 and b.info()["dft_buffered"] == 0, nc
        commit_ms = kc["dft_block"]
    reg_ms = D.max(win_ms + commit_ms * buffered / kb)
    t_e2e = D.max(t_e2e + commit_ms * 1e-3 * buffered_e2e / kb)
    b.close()
    hbm, src = peaks()
    # algorithmic bytes of one E and one H pass over every cell (as for one engine)
    eb = hb = 0
    for w, p in zip(ws, params):
        e, h = algorithmic_bytes(w, p, 8, 4)
        eb += e
        hb += h
    if kn["fused_eh"] > 0:
        # the fused work list: one pass per step (its launches each timed) moves both passes' bytes
        t_f = kms["fused_eh"] / K * 1e-3
        dom, db, dt_ = "fused_eh", eb + hb, t_f
        t_e = t_h = t_f / 2
    else:
        t_e = kms["update_e"] / kn["update_e"] * 1e-3
        t_h = kms["update_h"] / kn["update_h"] * 1e-3
        dom, db, dt_ = ("update_h", hb, t_h) if t_h >= t_e else ("update_e", eb, t_e)
    achieved = db / dt_ / 1e9
    flux_launches = 3 if buffered else 2
    launches = info["launches_per_pass"] * (kn["update_e"] + kn["update_h"]) + kn["fused_eh"] + \
        kn["tfsf"] + kn["dft_gather"] + kn["flux"] * flux_launches + 2 * kn["dft_block"]
    value = world * cells * K / (reg_ms * 1e-3) / 1e9
    h2d = 0  # the patterns are generated on the device
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": "Gcell/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": round(reg_ms / K, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 fields (fp32), fp64 incident field, compensated fp32 (double-float) DFT accumulation",
        "data": "synthetic (seeded binary eps patterns, numpy PCG64 seed+i per cell)",
        "config": {"workload": f"batch of {ncells} uneven Bloch cells", "grid_cells": cells,
                   "nof": 128, "dft_points": info["dft_points"], "dft_block": kb,
                   "dft_faces": "z planes (reflection, transmission)", "tile": list(tile),
                   "tune_ms_per_eh_pass": {"_".join(map(str, k)) if isinstance(k[0], str) else "x".join(map(str, k)):
                                           round(v, 3) for k, v in tune_ms.items()},
                   "l2": "working set >> 129 MB L2; no flush needed",
                   "parallelism": f"replicas x{world} (independent batches, one per GPU)"},
        "e2e": {"value": round(world * cells * K / t_e2e / 1e9, 3), "unit": "Gcell/s",
                "h2d_bytes_per_step": round(h2d / K, 1), "d2h_bytes_per_step": round(sum(j.size for j in J) * 8 / K, 1),
                "what": ("iris_batch_create + iris_batch_material_pattern x%d (generated on the device) + tune + "
                         "%d steps + flux of every cell" % (ncells, K))},
        "gpu_launches": int(launches),
        "kernels_ms_per_step": {k: round(v / K, 4) for k, v in kms.items()},
        "window_ms_per_step": round(win_ms / K, 4),
        "dft_commit": {"block_samples": kb, "ms": round(commit_ms, 3), "samples_left_buffered": buffered,
                       "share_ms_in_value": round(commit_ms * buffered / kb, 4)},
        "roofline": {"kernel": "batch_" + dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": hbm,
                     "unit": "GB/s", "frac": round(achieved / hbm, 4), "peak_source": src, "traffic": None,
                     "algorithmic_bytes_per_pass": db},
        "stencil_gcells": round(cells / (t_e + t_h) / 1e9, 3),
        "clocks": clocks,
    }
    if loop_sample:
        out["loop_plain"] = loop_plain(iris, ws, params, fw, local, loop_sample, steps=16)
    return out


def run_adjoint(args, rank, world, local):
    """The gradient workload: dL/d eps over a 128x128x32 design region (eps ~U[1,12],
    seed 0) of a 160x160x512 cell, L = sum over 64 frequencies of J6, FP32
    forward and adjoint, checkpoints every 256 steps.  Reports the gradient
    throughput, its cost against the forward solve, and its error against
    the FP64 adjoint and against central differences of the FP64 forward."""
    iris = importlib.import_module(PKG)
    cfg = importlib.import_module(PKG + ".configs")
    D = Dist(world)
    w = cfg.workload(5)
    ex = w.extra
    design = (ex["x0"], ex["x1"], ex["y0"], ex["y1"], w.hi, w.hi + w.dh - 1)
    t = time.perf_counter()
    eps_inv = cfg.design_region_material(w, seed=rank).real
    t_mat = time.perf_counter() - t
    path = cfg.write_input(os.path.join(tempfile.mkdtemp(prefix="iris_adj_"), "inputFDTD.dat"), w)
    p, fw, _ = iris.setparam(path)
    p.device = local
    N = args.adjoint_steps or w.nsteps
    cells = w.nx * w.ny * w.nz
    eta = eps_inv[1:-1, design[2]:design[3] + 1, design[0]:design[1] + 1].copy()

    def solve(precision, warm, checkpoint_every=256):
        adj = iris.Adjoint(p, fw, design, checkpoint_every=checkpoint_every, precision=precision, device=local)
        adj.set_material(eps_inv)
        if warm:
            adj.forward(8)
            adj.backward()
        t0 = time.perf_counter()
        L, _ = adj.forward(N)
        g = adj.backward()
        wall = time.perf_counter() - t0
        return adj, L, g, adj.timing(), wall

    D.barrier()
    pr, cpath = start_clocks(local)
    adj32, L32, g32, tm32, wall32 = solve(iris.FP32, True)
    clocks = stop_clocks(pr, cpath)
    fwd_ms = D.max(tm32["forward_ms"])
    bwd_ms = D.max(tm32["recompute_ms"] + tm32["adjoint_ms"])
    out = {
        "metric": METRIC, "value": round(world * cells * N / ((fwd_ms + bwd_ms) * 1e-3) / 1e9, 3),
        "unit": "Gcell/s", "n_gpus": world, "steps": N, "warmup": 8,
        "ms_per_step": round((fwd_ms + bwd_ms) / N, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64 fields and adjoint (fp32), fp64 DFT and gradient accumulation",
        "data": "synthetic (design eps ~U[1,12], numpy PCG64 seed = rank)",
        "config": {"workload": f"{w.name} gradient", "grid": [w.nx, w.ny, w.nz],
                   "design_region": list(design), "nof": w.nof, "checkpoint_every": 256,
                   "objective": "sum_w J6(w)",
                   "l2": "fields 2 x %.2f GB >> 129 MB L2" % (cells * 24 / 1e9),
                   "parallelism": f"replicas x{world} (independent designs, one per GPU)"},
        "value_is": "grid cell-updates of the forward solve / device time of forward + backward",
        "forward_gcells": round(cells * N / (fwd_ms * 1e-3) / 1e9, 3),
        "forward_ms": round(fwd_ms, 1), "recompute_ms": round(tm32["recompute_ms"], 1),
        "adjoint_ms": round(tm32["adjoint_ms"], 1),
        "gradient_cost_vs_forward": round(bwd_ms / fwd_ms, 3),
        "e2e": {"value": round(world * cells * N / wall32 / 1e9, 3), "unit": "Gcell/s",
                "h2d_bytes_per_step": round(eps_inv.size * 16 / N, 1),
                "d2h_bytes_per_step": round(g32.size * 8 / N, 1),
                "what": "forward (%d steps, checkpoints) + backward through the C ABI, gradient to host" % N},
        "clocks": clocks, "material_setup_s": round(t_mat, 2),
    }
    if rank == 0 and world == 1:
        # the same gradient with every step's design-region curls kept in HBM
        # (one segment: no checkpoints to restore, no recompute sweep)
        adj32.close()
        adjR, _, gR, tmR, _ = solve(iris.FP32, False, checkpoint_every=N)
        adjR.close()
        out["no_recompute"] = {
            "checkpoint_every": N, "recorded_bytes": int(N * 3 * eta.size * 8),
            "forward_ms": round(tmR["forward_ms"], 1), "backward_ms": round(tmR["recompute_ms"] + tmR["adjoint_ms"], 1),
            "gradient_cost_vs_forward": round((tmR["recompute_ms"] + tmR["adjoint_ms"]) / tmR["forward_ms"], 3),
            "value": round(cells * N / ((tmR["forward_ms"] + tmR["recompute_ms"] + tmR["adjoint_ms"]) * 1e-3) / 1e9, 3),
            "gradient_bitwise_equal": bool(np.array_equal(gR, g32))}
    hbm, src = peaks()
    eb, hb = algorithmic_bytes(w, p, 8, 4)
    fwd_bw = (eb + hb) * N / (fwd_ms * 1e-3) / 1e9
    out["roofline"] = {"kernel": "forward step (update_e + update_h + tfsf + dft)", "bound": "hbm",
                       "achieved": round(fwd_bw, 1), "peak": hbm, "unit": "GB/s", "frac": round(fwd_bw / hbm, 4),
                       "peak_source": src, "traffic": None}
    if rank == 0 and world == 1 and not args.no_fp64_compare:
        adj64, L64, g64, tm64, _ = solve(iris.FP64, False)
        g32e, g64e = -g32 * eta ** 2, -g64 * eta ** 2
        check = {"L_rel_err_fp32": abs(L32 - L64) / abs(L64),
                 "grad_rel_err_fp32_vs_fp64": float(np.max(np.abs(g32e - g64e)) / np.max(np.abs(g64e))),
                 "fp64_forward_ms": round(tm64["forward_ms"], 1),
                 "fp64_backward_ms": round(tm64["recompute_ms"] + tm64["adjoint_ms"], 1)}
        if args.fd_voxels:
            r = np.random.default_rng(0)
            eps = 1.0 / eta
            fd, ad32, ad64 = [], [], []
            h = 1e-3
            for q in r.choice(eta.size, args.fd_voxels, replace=False):
                idx = np.unravel_index(q, eta.shape)
                v = []
                for sgn in (1, -1):
                    e2 = eps.copy()
                    e2[idx] += sgn * h
                    adj64.set_design(1.0 / e2)
                    v.append(adj64.forward(N)[0])
                fd.append((v[0] - v[1]) / (2 * h))
                ad32.append(g32e[idx])
                ad64.append(g64e[idx])
            fd, ad32, ad64 = map(np.asarray, (fd, ad32, ad64))
            check["fd_voxels"] = int(args.fd_voxels)
            check["fd_h"] = h
            check["grad_rel_err_fp32_vs_fd"] = float(np.max(np.abs(ad32 - fd)) / np.max(np.abs(fd)))
            check["grad_rel_err_fp64_vs_fd"] = float(np.max(np.abs(ad64 - fd)) / np.max(np.abs(fd)))
        out["gradient_check"] = check
        adj64.close()
    adj32.close()
    D.close()
    return out


def loop_plain(iris, ws, params, fw, local, nsample, steps):
    """The same cells stepped one after another, each on its own engine (the plain
    solver in a loop), on a sample of the batch: aggregate Gcell/s."""
    tot_cells, tot_ms = 0, 0.0
    idx = list(range(0, len(ws), max(1, len(ws) // nsample)))[:nsample]
    for i in idx:
        q = params[i].copy()
        q.dft_faces = iris.DFT_Z
        e = iris.Engine(q, fw, precision=iris.FP32, device=local)
        e.material_pattern(cfg_mod().pattern_seed(ws[i]), ws[i].extra["fill"], 4.0, 1.0)
        e.step(1, 3)
        e.sync()
        e.timing_start(per_kernel=False)
        e.step(4, steps)
        reg, _, _ = e.timing_read()
        e.close()
        tot_cells += ws[i].cells * steps
        tot_ms += reg
    return {"value": round(tot_cells / (tot_ms * 1e-3) / 1e9, 3), "unit": "Gcell/s", "cells_sampled": len(idx),
            "steps": steps, "note": "each sampled cell on its own engine, device time summed"}


def tr_error(iris, p, fw, eps, local):
    """FP32 against FP64 over the whole run (texit steps): R = J5/(J5+J6) and
    T = J6/(J5+J6) of box 1 per wavelength, their largest absolute
    differences, and each precision's device time.  The FP64 engine stands
    for the FP64 oracle (tests/test_gpu_slit.py holds it within 1e-12 of the
    oracle on this grid); z-plane DFTs only (all T/R needs)."""
    out, cells = {}, p.nx * p.ny * p.nz
    for prec in (iris.FP64, iris.FP32):
        q = p.copy()
        q.dft_faces = iris.DFT_Z
        e = iris.Engine(q, fw, precision=prec, device=local)
        e.set_material(eps)
        t0 = time.perf_counter()
        e.timing_start(per_kernel=False)
        e.step(1, p.texit)
        J = e.flux(0)
        ms, _, _ = e.timing_read()
        out[prec] = (iris.tr_normalise(J[4], J[5]), time.perf_counter() - t0, ms)
        e.close()
    (r64, t64), s64, ms64 = out[iris.FP64]
    (r32, t32), s32, ms32 = out[iris.FP32]
    return {"grid": [p.nx, p.ny, p.nz], "steps": p.texit, "nof": p.nof,
            "R_max_abs_err": float(np.max(np.abs(r32 - r64))),
            "T_max_abs_err": float(np.max(np.abs(t32 - t64))),
            "R_rel_err": float(np.max(np.abs(r32 - r64)) / np.max(np.abs(r64))),
            "T_rel_err": float(np.max(np.abs(t32 - t64)) / np.max(np.abs(t64))),
            "fp64_gcells": round(cells * p.texit / (ms64 * 1e-3) / 1e9, 3),
            "fp32_gcells": round(cells * p.texit / (ms32 * 1e-3) / 1e9, 3),
            "device_ms": {"fp64": round(ms64, 1), "fp32": round(ms32, 1)},
            "wall_s": {"fp64": round(s64, 2), "fp32": round(s32, 2)},
            "note": ("FP32 (tensor-core DFT) against FP64 over the full run, per spectrum, both on the default "
                     "stencil (the persistent whole-step kernel on a grid this size; spectra bitwise those of the "
                     "split passes); its state (75 MB) lives in the 129 MB L2, so no HBM roofline applies")}


def guarded(fn, *a, **k):
    """A sub-measurement of the default line: its result, or its error (the
    main line stands either way)."""
    try:
        return fn(*a, **k)
    except Exception as e:  # noqa: BLE001
        return {"error": f"{type(e).__name__}: {e}"}


def measure_slit(iris, local):
    """The 256x4x768 slit array, FP32 against FP64 over its 8000 steps."""
    cfg = importlib.import_module(PKG + ".configs")
    w = cfg.workload(2)
    path = cfg.write_input(os.path.join(tempfile.mkdtemp(prefix="iris_slit_"), "inputFDTD.dat"), w)
    p, fw, _ = iris.setparam(path)
    p.device = local
    return tr_error(iris, p, fw, cfg.slit_material(w), local)


def measure_tiny(iris, local):
    """The 4x4x512 FP64 slab, DFT of the z = 30 and z = 480 planes at
    200 frequencies, 4000 steps, stepped by the persistent kernel (one
    cooperative launch per span of steps); the same run through the split
    passes replayed from CUDA graphs, which must give the same spectra bit
    for bit; and the reference's 3D DFT over every face pair for scale."""
    cfg = importlib.import_module(PKG + ".configs")
    w = cfg.workload(1)
    path = cfg.write_input(os.path.join(tempfile.mkdtemp(prefix="iris_tiny_"), "inputFDTD.dat"), w)
    p, fw, _ = iris.setparam(path)
    p.device = local
    cells, N = w.cells, p.texit
    res = {}
    for name, stencil, graph, faces in (("persistent", iris.STENCIL_PERSISTENT, False, iris.DFT_Z),
                                        ("split_graphs", iris.STENCIL_SPLIT, True, iris.DFT_Z),
                                        ("persistent_all_faces", iris.STENCIL_PERSISTENT, False, iris.DFT_ALL)):
        q = p.copy()
        q.dft_faces = faces
        e = iris.Engine(q, fw, precision=iris.FP64, device=local, stencil=stencil, graph=graph)
        e.step(1, 8)  # modules loaded, graphs captured before the clock
        e.flux(0)
        e.close()
        t0 = time.perf_counter()
        e = iris.Engine(q, fw, precision=iris.FP64, device=local, stencil=stencil, graph=graph)
        e.timing_start(per_kernel=False)
        e.step(1, N)
        J = e.flux(0)
        ms, _, _ = e.timing_read()
        wall = time.perf_counter() - t0
        e.close()
        res[name] = (J, ms, wall)
    J0, ms0, wall0 = res["persistent"]
    Jg, msg, _ = res["split_graphs"]
    Ja, msa, _ = res["persistent_all_faces"]
    R, T = iris.tr_normalise(J0[4], J0[5])
    return {"workload": "slab_4x4x512_fp64", "grid": [w.nx, w.ny, w.nz], "steps": N, "nof": p.nof,
            "dft_faces": "z planes 30 and 480", "value": round(cells * N / (ms0 * 1e-3) / 1e9, 4),
            "unit": "Gcell/s", "ms_per_step": round(ms0 / N, 5), "dtype": "c128 (fp64)",
            "e2e": {"value": round(cells * N / wall0 / 1e9, 4), "unit": "Gcell/s",
                    "what": "iris_create + %d steps + iris_flux to host" % N},
            "split_graphs_ms_per_step": round(msg / N, 5),
            "speedup_vs_split_graphs": round(msg / ms0, 2),
            "spectra_bitwise_equal_to_split": bool(np.array_equal(J0, Jg)),
            "all_faces_ms_per_step": round(msa / N, 5),
            "T_at_first_and_last_frequency": [float(T[0]), float(T[-1])],
            "note": ("launch-bound: 8192 cells a step; the reference's 3D DFT over every face pair "
                     "(43488 points x 200 frequencies) is FP64-ALU-bound instead")}


def measure_adjoint(iris, local, fd_voxels=64):
    """dL/d eps over the 128x128x32 design region of the 160x160x512
    cell, FP32 forward and adjoint over 6000 steps with checkpoints every 256;
    the gradient against the FP64 adjoint, and against central differences
    (h = 1e-3) of the FP64 forward along a seeded +-1 direction over
    fd_voxels seeded voxels (one directional derivative: two FP64 solves)."""
    cfg = importlib.import_module(PKG + ".configs")
    w = cfg.workload(5)
    ex = w.extra
    design = (ex["x0"], ex["x1"], ex["y0"], ex["y1"], w.hi, w.hi + w.dh - 1)
    eps_inv = cfg.design_region_material(w, seed=0).real
    path = cfg.write_input(os.path.join(tempfile.mkdtemp(prefix="iris_adj_"), "inputFDTD.dat"), w)
    p, fw, _ = iris.setparam(path)
    p.device = local
    N, cells = w.nsteps, w.cells
    eta = eps_inv[1:-1, design[2]:design[3] + 1, design[0]:design[1] + 1].copy()

    def solve(precision):
        adj = iris.Adjoint(p, fw, design, checkpoint_every=256, precision=precision, device=local)
        adj.set_material(eps_inv)
        t0 = time.perf_counter()
        L, _ = adj.forward(N)
        g = adj.backward()
        return adj, L, -g * eta ** 2, adj.timing(), time.perf_counter() - t0

    a32, L32, g32, tm32, wall32 = solve(iris.FP32)
    a32.close()
    a64, L64, g64, tm64, _ = solve(iris.FP64)
    fwd, bwd = tm32["forward_ms"], tm32["recompute_ms"] + tm32["adjoint_ms"]
    r = np.random.default_rng(0)
    idx = r.choice(eta.size, fd_voxels, replace=False)
    v = np.zeros(eta.size)
    v[idx] = r.choice([-1.0, 1.0], fd_voxels)
    v = v.reshape(eta.shape)
    h = 1e-3
    Ls = []
    for sgn in (1, -1):
        a64.set_design(1.0 / (1.0 / eta + sgn * h * v))
        Ls.append(a64.forward(N)[0])
    a64.close()
    fd = (Ls[0] - Ls[1]) / (2 * h)
    d32, d64 = float(np.sum(g32 * v)), float(np.sum(g64 * v))
    return {"workload": f"{w.name} gradient", "grid": [w.nx, w.ny, w.nz], "design_region": list(design),
            "steps": N, "nof": w.nof, "checkpoint_every": 256,
            "value": round(cells * N / ((fwd + bwd) * 1e-3) / 1e9, 3), "unit": "Gcell/s",
            "value_is": "grid cell-updates of the forward solve / device time of forward + backward (FP32)",
            "forward_gcells": round(cells * N / (fwd * 1e-3) / 1e9, 3),
            "forward_ms": round(fwd, 1), "backward_ms": round(bwd, 1),
            "gradient_cost_vs_forward": round(bwd / fwd, 3),
            "e2e_wall_s": round(wall32, 2),
            "grad_rel_err_fp32_vs_fp64": float(np.max(np.abs(g32 - g64)) / np.max(np.abs(g64))),
            "L_rel_err_fp32_vs_fp64": abs(L32 - L64) / abs(L64),
            "fd_check": {"voxels": fd_voxels, "h": h, "direction": "seeded +-1 on the voxels, 0 elsewhere",
                         "fd_fp64": fd, "adjoint_fp64": d64, "adjoint_fp32": d32,
                         "rel_err_fp64": abs(d64 - fd) / abs(fd), "rel_err_fp32": abs(d32 - fd) / abs(fd)},
            "fp64_forward_ms": round(tm64["forward_ms"], 1),
            "fp64_backward_ms": round(tm64["recompute_ms"] + tm64["adjoint_ms"], 1)}


def fp64_compare(iris, p, fw, eps, cells, local, K=32, W=3):
    """The same workload in FP64 (parity mode) over K steps: one whole FP64 DFT
    block (K = 32 samples), so its accumulation is inside the timed steps."""
    eng = iris.Engine(p, fw, precision=iris.FP64, device=local)
    eng.set_material(eps)
    eng.step(1, W)
    eng.sync()
    eng.timing_start(per_kernel=True)
    eng.step(W + 1, K)
    reg_ms, kms, kn = eng.timing_read()
    eng.close()
    st = (kms["update_e"] + kms["update_h"]) / K * 1e-3
    return {"value": round(cells * K / (reg_ms * 1e-3) / 1e9, 3), "unit": "Gcell/s", "steps": K,
            "stencil_gcells": round(cells / st / 1e9, 3),
            "kernels_ms_per_step": {k: round(v / K, 3) for k, v in kms.items()},
            "note": "same workload, FP64 fields and DFT (parity mode), per step incl. one DFT block of 32"}


def column(w, side):
    """A side x side column of workload w: all of z (the same UPML, source,
    structure layer, DFT planes and frequencies), the DFT box across the
    column, the Bloch phase per period scaled to the column's width.  w
    itself when it is no wider."""
    cfg = importlib.import_module(PKG + ".configs")
    nx, ny = min(side, w.nx), min(side, w.ny)
    if (nx, ny) == (w.nx, w.ny):
        return w
    extra = dict(w.extra)
    structure = w.structure
    if structure == "spheres":
        extra["nspheres"] = 4
    elif structure == "design":
        structure = "slab"
    dx = int(round(w.dx * nx / w.nx)) if w.dx else 0
    return cfg.Workload(f"{w.name}_column_{nx}x{ny}", nx, ny, w.nz, w.pmlzi, w.pmlzf, w.hi, w.dh, w.eps_bbox, dx,
                        w.tfsf_zi, (1, nx, 1, ny, w.box[4], w.box[5]), w.nof, w.nsteps, w.eps1, w.eps3,
                        w.akx * nx / w.nx, w.aky * ny / w.ny, structure, extra)


def cpu_sample(w, side, threads, steps, warm=1):
    """Oracle on a side x side column of workload w (see column()): seconds per
    cell-step (everything but the DFT) and per DFT point-frequency-step."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import iris_oracle as O
    cfg = importlib.import_module(PKG + ".configs")
    ws = column(w, side)
    d = tempfile.mkdtemp(prefix="iris_cpu_")
    path = cfg.write_input(os.path.join(d, "inputFDTD.dat"), ws)
    op = O.setparam(path)
    o = O.Oracle(op, ak=(complex(ws.akx), complex(ws.aky), 0j), threads=threads)
    o.set_eps_inv(cfg.material(ws))
    if warm:
        o.run_timed(1, warm)
    td, tr = o.run_timed(1 + warm, steps)
    npts = o.total_points()
    o.close()
    return tr / (ws.cells * steps), td / (npts * op.nof * steps), ws


def host_cpu():
    """The host CPU as /proc/cpuinfo names it (x86: model name; Arm: implementer and part)."""
    import platform
    name, arm = None, {}
    try:
        for line in open("/proc/cpuinfo"):
            k, _, v = line.partition(":")
            k, v = k.strip(), v.strip()
            if k == "model name" and name is None:
                name = v
            elif k in ("CPU implementer", "CPU part") and k not in arm:
                arm[k] = v
    except OSError:
        pass
    if name is None and arm:
        name = "Arm implementer %s part %s" % (arm.get("CPU implementer", "?"), arm.get("CPU part", "?"))
    return {"cpu": name or platform.processor() or "unknown", "machine": platform.machine(),
            "nproc": os.cpu_count() or 1}


def cpu_baseline(w, full_points, steps=192, side=32, single_steps=8, single_side=16):
    """The oracle on all host cores (the reported value) and, like the
    reference (which has no threading), on one core over a smaller sample."""
    threads = os.cpu_count() or 1
    cells = w.nx * w.ny * w.nz

    def sample(thr, sd, st):
        t0 = time.perf_counter()
        t_cell, t_pf, _ = cpu_sample(w, sd, thr, st)
        wall = time.perf_counter() - t0
        return t_cell, t_pf, cells / (t_cell * cells + t_pf * full_points * w.nof) / 1e9, wall

    t_cell, t_pf, v, wall = sample(threads, side, steps)
    t_cell1, t_pf1, v1, wall1 = sample(1, single_side, single_steps)
    return {"value": round(v, 6), "unit": "Gcell/s", "cores": threads, "kind": "port",
            "sample": (f"oracle (C++ FP64 restatement, OpenMP {threads} threads) on a {side}x{side}x{w.nz} column of "
                       f"the workload for {steps} steps ({wall:.1f} s); per-cell ({t_cell * 1e9:.2f} ns) and per-DFT-"
                       f"point-frequency ({t_pf * 1e9:.3f} ns) costs scaled to the full grid and its {full_points} "
                       f"DFT points x {w.nof} frequencies"),
            "single_thread": {"value": round(v1, 6), "unit": "Gcell/s", "cores": 1,
                              "sample": (f"the same on one thread, a {single_side}x{single_side}x{w.nz} column for "
                                         f"{single_steps} steps ({wall1:.1f} s); per-cell {t_cell1 * 1e9:.2f} ns, "
                                         f"per-DFT-point-frequency {t_pf1 * 1e9:.3f} ns")},
            "host": host_cpu()}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    cfg = importlib.import_module(PKG + ".configs")
    if args.workload == 4:
        # the batch: the oracle's per-cell and per-point costs on a column of
        # its first cell, scaled to the whole batch (z-plane DFT at 128 freq.)
        ws = cfg.batch_cells(args.cells, nof=128)
        w = ws[0]
        cells_all = sum(x.cells for x in ws)
        pts_all = sum(12 * x.nx * x.ny for x in ws)
    else:
        w = cfg.workload(args.workload)
        cells_all = pts_all = None
    threads = os.cpu_count() or 1
    # total DFT points of the full workload (x, y and z face pairs of the box)
    b = w.box
    nbx, nby, nbz = b[1] - b[0] + 1, b[3] - b[2] + 1, b[5] - b[4] + 1
    full_points = 12 * (nby * nbz + nbx * nbz + nbx * nby) if pts_all is None else pts_all
    cells = w.nx * w.ny * w.nz if cells_all is None else cells_all
    # a column sized so that warmup + steps finish in about a minute
    side = 16 if args.steps + args.warmup > 40 else 24
    t_cell_w, t_pf_w, _ = cpu_sample(w, side, threads, max(1, args.warmup), warm=0)
    t0 = time.perf_counter()
    t_cell, t_pf, ws = cpu_sample(w, side, threads, args.steps, warm=0)
    wall = time.perf_counter() - t0
    t_step = t_cell * cells + t_pf * full_points * w.nof
    v = cells / t_step / 1e9
    extrapolated = ws is not w or cells_all is not None
    if extrapolated:
        sample = (f"oracle (C++ FP64 restatement of the Fortran path, OpenMP {threads} threads) run on a "
                  f"{ws.nx}x{ws.ny}x{ws.nz} column of {w.name} for {args.steps} steps ({wall:.1f} s); its measured "
                  f"cost per cell-step and per DFT point-frequency-step scaled to the {cells} cells and "
                  f"{full_points} DFT points x {w.nof} frequencies of the workload (a model, not a run of it)")
    else:
        sample = (f"oracle (C++ FP64 restatement of the Fortran path, OpenMP {threads} threads) run on the whole "
                  f"{w.nx}x{w.ny}x{w.nz} workload for {args.steps} steps ({wall:.1f} s)")
    return {
        "metric": METRIC, "impl": "reference", "value": round(v, 6), "unit": "Gcell/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_step * 1e3, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128 (fp64)",
        "data": "synthetic (seeded inputs of the workload's shape)",
        "config": {"workload": (f"batch of {args.cells} cells, per-cell costs of {w.name}"
                                if args.workload == 4 else w.name),
                   "grid": [w.nx, w.ny, w.nz], "grid_cells": cells, "nof": w.nof},
        "cpu_baseline": {"value": round(v, 6), "unit": "Gcell/s", "cores": threads, "kind": "port",
                         "sample": sample, "extrapolated": extrapolated,
                         "column": [ws.nx, ws.ny, ws.nz],
                         "seconds_per_cell_step": t_cell, "seconds_per_point_frequency_step": t_pf,
                         "timed_seconds": round(wall, 3)},
        "extrapolated": extrapolated,
        "e2e": {"value": round(v, 6), "unit": "Gcell/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def l2_note(field_bytes, acc_bytes):
    """The config's statement about the 129 MB L2 between timed steps."""
    ws = field_bytes + acc_bytes
    if ws > 4 * 129e6:
        return "working set (fields %.2f GB, DFT accumulators %.2f GB) >> 129 MB L2; no flush needed" % (
            field_bytes / 1e9, acc_bytes / 1e9)
    return ("working set (fields %.1f MB, DFT accumulators %.1f MB) within reach of the 129 MB L2 and not "
            "flushed between steps: a grid this small lives in L2 in any real run" % (field_bytes / 1e6, acc_bytes / 1e6))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=512)
    ap.add_argument("--warmup", type=int, default=64)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", type=int, default=3)
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="default workload: skip the batched-form sub-measurement")
    ap.add_argument("--no-configs", action="store_true",
                    help="default workload: skip the 4x4x512 slab, slit-array and adjoint sub-measurements")
    ap.add_argument("--adjoint-fd-voxels", type=int, default=64,
                    help="default line: voxels of the adjoint's directional finite-difference check")
    ap.add_argument("--cpu-sample-steps", type=int, default=192)
    ap.add_argument("--grid", type=int, nargs=3, default=None, metavar=("NX", "NY", "NZ"),
                    help="run the workload resized to this grid (profiling cases)")
    ap.add_argument("--nof", type=int, default=None, help="number of DFT frequencies with --grid")
    ap.add_argument("--dft-block", type=int, default=0, help="DFT samples per accumulation block (0: engine default)")
    ap.add_argument("--stencil", type=int, default=0, choices=[0, 1, 2, 3],
                    help="0: engine default, 1: split E and H passes, 2: fused E+H pass (fp32), 3: streamed split passes (fp32)")
    ap.add_argument("--dft-kernel", type=int, default=0, choices=[0, 1, 2],
                    help="FP32 DFT block: 0 engine default, 1 CUDA cores, 2 tensor cores (tcgen05)")
    ap.add_argument("--graph", action="store_true",
                    help="step whole DFT blocks from a captured CUDA graph (e2e run and an extra timed run)")
    ap.add_argument("--cells", type=int, default=256, help="cells in the batch (workload 4)")
    ap.add_argument("--tile", type=int, default=None, help="workload 4: this work-list tile instead of the autotuner's")
    ap.add_argument("--adjoint-steps", type=int, default=0, help="workload 5: forward steps (0: the workload's 6000)")
    ap.add_argument("--fd-voxels", type=int, default=4,
                    help="workload 5: voxels checked against central differences of the FP64 forward")
    ap.add_argument("--loop-sample", type=int, default=16,
                    help="workload 4: cells of the batch also stepped one by one on plain engines (0: skip)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    rank, world, local = env_rank()
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    elif args.workload == 4:
        out = run_batch(args, rank, world, local)
    elif args.workload == 5:
        out = run_adjoint(args, rank, world, local)
    else:
        out = run_engine(args, rank, world, local)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
