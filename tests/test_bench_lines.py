"""bench.py on the host: the reference arm's JSON line (the C restatement timed on the host
cores) and the clock summary that decides whether a timed run saw throttling."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["unit"] == "E-points/s" and line["higher_is_better"] is True
    assert (line["steps"], line["warmup"], line["n_gpus"]) == (1, 3, 1)
    assert abs(line["ms_per_step"] - 1e3 * line["config"]["points_per_step"] / line["value"]) \
        <= 1e-6 * line["ms_per_step"]
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "E-points/s",
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert line["config"]["slabs"] == 100 and line["config"]["orbitals_per_slab"] == 128


def test_clock_summary_reports_throttle_reasons():
    import bench
    c = bench.Clocks(0)
    idle = ["Not Active"] * 4
    c.rows = [["0", "2070", "2070", "900.5", "0x0"] + idle,
              ["0", "1980", "2070", "1395.0", "0x4"] + idle[:3] + ["Active"],
              ["0", "2070", "2070", "1200.0", "0x0"] + idle,
              ["0", "[N/A]"]]  # a torn sample is skipped
    s = c.stop()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"] and s["samples"] == 4
    c.rows = [["0", "1500", "2070", "700.0", "0x40", "Not Active", "Active", "Not Active",
               "Not Active"]]
    assert c.stop()["reasons"] == ["hw_thermal_slowdown"]
