"""bench.py --impl reference: the line the reference arm prints (CPU).

The reference arm times the CPU restatement of the reference's loop on the
host cores and prints one JSON line with the same metric, unit and config
as the GPU arm plus "impl": "reference", a cpu_baseline block and an e2e
block with no host-device traffic.  Run here on a small mesh (the full
1M-cell mesh is swapped for a 2k-cell one) so it finishes in seconds.
"""
import argparse
import io
import json
import os
import sys
from contextlib import redirect_stdout

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    from finitevolume_gb300 import meshgen

    monkeypatch.setattr(bench, "load_mesh", lambda: meshgen.naca_mixed(32, 16, seed=0))
    monkeypatch.setenv("FV_REF_SECONDS", "2")
    args = argparse.Namespace(gpus=1, steps=3, warmup=1)
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(args, 0)
    lines = [ln for ln in buf.getvalue().splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == "Mcell-iters/s"
    assert d["higher_is_better"] is True and d["n_gpus"] == 1
    assert d["value"] > 0 and 1 <= d["steps"] <= 3 and d["warmup"] == 3
    # the same config block as the GPU arm prints
    assert d["config"] == bench.headline_config(d["config"]["cells"], d["config"]["faces"], 1)
    assert d["config"]["workload"] == "naca0012_mixed_1M_o2_hllc_lsq_venkat_rk3"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "Mcell-iters/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_print_nothing():
    sys.path.insert(0, ROOT)
    import bench
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(argparse.Namespace(gpus=2, steps=3, warmup=1), 1)
    assert buf.getvalue() == ""


def test_cpu_baseline_block_has_all_threads_and_single_thread_samples():
    sys.path.insert(0, ROOT)
    import bench
    from finitevolume_gb300 import meshgen
    from oracle import port

    poly = meshgen.naca_mixed(32, 16, seed=0)
    before = port.num_threads()
    keep = {}
    cb = bench.cpu_baseline_block(poly, 0.5, 0.5, keep=keep)
    assert cb["kind"] == "port" and cb["unit"] == "Mcell-iters/s" and cb["value"] > 0
    # the port's field is kept for the headline parity check
    assert keep["field"].shape == (poly.n_cells, 4) and keep["iterations"] >= 2
    assert cb["cores"] == before
    st = cb["single_thread"]
    assert st["cores"] == 1 and st["value"] > 0 and st["unit"] == "Mcell-iters/s"
    assert port.num_threads() == before  # thread count restored


def test_config1_cpu_baseline():
    sys.path.insert(0, ROOT)
    import bench
    cb = bench.config1_cpu_rate(steps=50, seconds=0.2)
    assert cb["kind"] == "port" and cb["value"] > 0 and cb["cores"] >= 1
    assert cb["unit"] == "Mcell-iters/s" and "of the 50 iterations" in cb["sample"]
