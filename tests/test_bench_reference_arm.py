"""bench.py's reference arm on the CPU: it times the oracle (the restated
reference path) on a bounded sample of the default workload and prints one
JSON line with the contract's keys; under a multi-rank launch the ranks
other than 0 exit 0 without output."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def run_bench(*args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, env=e,
                          capture_output=True, text=True, timeout=600)


def test_reference_arm_line():
    r = run_bench("--impl", "reference", "--steps", "1", "--warmup", "3")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "Gcell/s" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1 and d["vs_baseline"] is None
    assert d["value"] > 0 and d["config"]["workload"] == "spheres_512x512x1024"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "Gcell/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    r = run_bench("--impl", "reference", "--steps", "1", "--warmup", "3",
                  env={"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2", "MASTER_ADDR": "127.0.0.1",
                       "MASTER_PORT": "29571"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


def test_warmup_below_three_is_refused():
    r = run_bench("--impl", "reference", "--steps", "1", "--warmup", "1")
    assert r.returncode != 0 and "warmup" in r.stderr


def bench_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_dft_accounting():
    """The accumulator bytes charged are those of the commits and flux reads that
    ran inside the timed steps, not a per-block average."""
    b = bench_module()
    P, nof, kb, sc = 1200, 300, 512, 8
    fp = P * 4 // 6
    kn = {"dft_block": 0, "flux": 1, "dft_gather": 20}
    kms = {"dft_block": 0.0, "flux": 2.0, "dft_gather": 0.5}
    # 20 steps, no commit inside the window, one flux read over 20 buffered samples
    d = b.dft_accounting(P, nof, kb, sc, 20, kms, kn, 20, fp, 40.0)
    assert d["complex_macs_per_step"] == P * nof and d["ring_bytes_per_step"] == P * sc
    assert d["commits_in_window"] == 0 and d["samples_left_buffered"] == 20
    assert d["accumulator_bytes_per_step"] == round(fp * nof * 16 / 20)
    assert "block_gbs" not in d
    assert abs(d["flux_gbs"] - (fp * nof * 16 + 20 * fp * sc) / 2.0e-3 / 1e9) < 0.1
    assert abs(d["gather_gbs"] - 2 * 20 * P * sc / 0.5e-3 / 1e9) < 0.1
    assert d["commit"]["share_ms_in_value"] == round(40.0 * 20 / kb, 4)
    # 512 steps: one commit of the whole block inside the window, nothing left buffered
    kn = {"dft_block": 1, "flux": 1, "dft_gather": 512}
    kms = {"dft_block": 30.0, "flux": 2.0, "dft_gather": 10.0}
    d = b.dft_accounting(P, nof, kb, sc, 512, kms, kn, 0, fp, 0.0)
    assert d["accumulator_bytes_per_step"] == round((2 * P * nof * 16 + fp * nof * 16) / 512)
    assert abs(d["block_gbs"] - (2 * P * nof * 16 + 512 * P * sc) / 30.0e-3 / 1e9) < 0.1
    assert "commit" not in d


def test_cpu_baseline_keys():
    b = bench_module()
    cfg = __import__("importlib").import_module("irisfdtd-academic_gb300.configs")
    w = cfg.workload(3)
    d = b.cpu_baseline(w, 14856192, steps=1, side=8, single_steps=1, single_side=8)
    assert d["kind"] == "port" and d["unit"] == "Gcell/s" and d["value"] > 0 and d["cores"] >= 1
    assert d["single_thread"]["cores"] == 1 and d["single_thread"]["value"] > 0
    assert d["host"]["nproc"] >= 1 and d["host"]["cpu"]
