"""CPU test of bench.py's reference arm: it runs without a GPU (the CPU
restatement on the host cores) and prints one JSON line with the keys the
benchmark contract asks for."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--nt", "40",
                          "--shots", "2", "--steps", "1", "--warmup", "0"], capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "shot-gradients/s"
    for k in ("metric", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling", "dtype", "data",
              "config"):
        assert k in d, k
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["cpu_baseline_with_strip_io"]["value"] > 0
    # every step is the whole workload, named with the same keys as the GPU arm's config
    assert d["config"]["shots_per_gpu"] == 2 and d["config"]["nt"] == 40
    assert "all 2 shots" in d["cpu_baseline"]["sample"]


def test_work_units_give_the_published_per_shot_figures():
    """U and B per shot-gradient of the benchmark configurations, as the
    measured tables quote them (481x141: 1.263 GPt and 47.10 GB; 201x101:
    0.244 GPt and 8.82 GB; 2001x601: 25.56 GPt and 992.3 GB)."""
    sys.path.insert(0, ROOT)
    try:
        import bench
    finally:
        sys.path.remove(ROOT)
    for (nx, nz, npml, nt, u, b) in ((481, 141, 40, 4000, 1.263e9, 47.10e9), (201, 101, 40, 2000, 0.244e9, 8.82e9),
                                     (2001, 601, 60, 6000, 25.56e9, 992.3e9)):
        U, B = bench.work_units(nx, nz, npml, nt, nx)
        assert abs(U / u - 1) < 2e-3 and abs(B / b - 1) < 2e-3, (nx, U, B)
    # the per-step bytes: 64 per PML-grid point, 56 per interior point, 8 per strip value
    U1, B1 = bench.work_units(10, 8, 2, 2, 3)
    assert U1 == 2 * 14 * 12 + 80 and B1 == 64 * 14 * 12 + 56 * 80 + 8 * (90 + 48) + 8 * 2 * 3
