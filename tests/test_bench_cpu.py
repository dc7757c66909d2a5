"""The reference arm of bench.py on CPU: one JSON line with the contract's keys, the
oracle port timed on the host cores, and silence on ranks other than 0."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(env_extra, *args):
    env = dict(os.environ, **env_extra)
    r = subprocess.run([sys.executable, "bench.py", *args], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return [json.loads(line) for line in r.stdout.splitlines() if line.startswith("{")]


def test_reference_arm_line():
    import bench

    lines = run_bench({}, "--impl", "reference", "--m", "100", "--steps", "1", "--warmup", "3", "--ref-iters", "5",
                      "--fp64-iters", "50")
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["config"] == bench.bench_config(100, 1)  # the same dict as the GPU arm's
    # what was measured and what was extrapolated: the assembly whole, the iteration count x10
    assert cb["extrapolated"] == {"assembly_x": 1, "iters_x": 10.0}
    assert abs(d["value"] - 1.0 / (cb["t_assembly_s"] + 50 * cb["t_iter_s"])) < 1e-9 * d["value"]
    assert abs(d["ms_per_step"] - 5e3 * cb["t_iter_s"]) < 1e-6 * d["ms_per_step"]


def test_reference_arm_other_ranks_print_nothing():
    assert run_bench({"RANK": "1", "WORLD_SIZE": "2"}, "--impl", "reference", "--m", "100", "--steps", "1") == []


def test_clock_sampler_summary():
    """The clocks object from nvidia-smi rows: median SM clock, max clock, active reasons."""
    import bench

    cs = bench.ClockSampler(0)
    cs.rows = [["0", "2070", "2070", "900.1", "0x0", "Not Active", "Not Active", "Not Active", "Not Active"],
               ["0", "1980", "2070", "1390.5", "0x4", "Not Active", "Not Active", "Not Active", "Active"],
               ["0", "2070", "2070", "1100.0", "0x0", "Not Active", "Not Active", "Not Active", "Not Active"],
               ["garbage"]]
    c = cs.stop()
    assert c == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    assert bench.ClockSampler(0).stop() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_roofline_inputs():
    """The banded iteration's algorithmic byte model at the 4M-DOF layout the bench reports,
    and the DRAM traffic read back from the committed data file of the ncu capture."""
    import bench

    layout = {"rows": 4004001, "stored": 28020160, "uniform_entries": 27558016, "slices": 125126}
    assert bench.zcg_bytes(layout) == 38 * 4004001 + 4 * 28020160 + 2 * 462144 + 8 * 125126 == 266157974
    t = bench.profiled_traffic("k_zcg_iter", 2000)
    assert t is not None and 0.5 * 266157974 < t < 1.2 * 266157974
    assert bench.profiled_traffic("k_zcg_iter", 1000) is None  # recorded for the 2000x2000 workload only
    assert bench.profiled_traffic("no_such_kernel", 2000) is None
    # the FP64 assembly kernels of the same workload: the element pass reads kappa and f
    # (384 MB, no geometry) and writes sigma and the load terms (256 MB, part of it still
    # in L2 at the end); the row pass writes at least the operator values of the
    # 28M-entry pattern
    ep = bench.profiled_traffic("k_element_prepass", 2000)
    rows = bench.profiled_traffic("k_poisson_system", 2000)
    assert ep is not None and 384e6 + 128e6 <= ep <= 384e6 + 256e6
    assert rows is not None and rows > 8 * 28012001


def test_shared_config_and_parity_helpers(oracle):
    """Both arms print bench_config's dict; the parity helpers measure what they say."""
    import numpy as np
    import scipy.sparse as sp

    import bench

    c = bench.bench_config(2000, 1)
    assert c["dof"] == 4004001 and c["nnz"] == 28012001 and c["workload"].startswith("poisson-2000x2000")
    K = sp.csc_matrix(np.array([[4.0, -1.0, -1e-14], [-1.0, 4.0, -1.0], [-1e-14, -1.0, 4.0]]))
    K2 = K.copy()
    K2.data = K2.data * (1 + 1e-13)
    p = bench.matrix_parity(K2, K)
    assert p["pattern_equal"] and abs(p["max_err_row_scaled"] - 1e-13) < 1e-15
    assert p["entries_compared_elementwise"] == 7 and abs(p["max_err_elementwise"] - 1e-13) < 1e-15
    K3 = sp.csc_matrix(np.diag([1.0, 2.0, 3.0]))
    assert bench.matrix_parity(K3, K) == {"pattern_equal": False}
    x = np.array([1.0, 2.0, 3.0])
    r, rep = bench.residual_report(K, x, K @ x + np.array([0.0, 1e-12, 0.0]), oracle)
    assert abs(rep["relres"] - 1e-12 / np.linalg.norm(K @ x)) < 1e-15
