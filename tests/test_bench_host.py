"""Host side of bench.py on CPU: the reference arm's JSON line (the oracle on
the host cores, whole transforms each timed), the coefficient NMSE and the
parsing of the clock record."""
import json
import subprocess
import sys
import tempfile

import numpy as np

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.strip().splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"]["workload"] == "q4_n20_b7_C3_nso_R2_S1000_10dB"
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    # every claimed step was timed: one whole transform per step, the time a real one
    assert d["steps"] == 1 and len(cb["step_s"]) == 1
    assert np.isclose(d["ms_per_step"], 1e3 * cb["step_s"][0]) and np.isclose(d["value"], 1.0 / cb["step_s"][0])
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


class _Req:
    def __init__(self, locq, strengths):
        self.locq, self.strengths = np.asarray(locq), np.asarray(strengths)


def test_coefficient_nmse():
    req = _Req([[0, 1], [1, 0]], [3 + 4j, 1.0])                      # support (0,1) and (1,0); |a|^2 = 25 + 1
    assert bench.coef_nmse(np.array([[0, 1], [1, 0]]), np.array([3 + 4j, 1.0]), req) == 0.0
    # a missed coefficient counts its whole energy, a spurious one its own
    assert np.isclose(bench.coef_nmse(np.array([[0, 1]]), np.array([3 + 4j]), req), 1 / 26)
    got = bench.coef_nmse(np.array([[0, 1], [1, 0], [1, 1]]), np.array([3 + 4j, 1.0, 0.5]), req)
    assert np.isclose(got, 0.25 / 26)


class _Proc:
    def terminate(self):
        pass

    def wait(self):
        pass


def _clocks_from(rows):
    c = bench.Clocks.__new__(bench.Clocks)
    c.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
    c.f.write("\n".join(rows) + "\n")
    c.p = _Proc()
    return c.stop()


def test_clock_record_parsing():
    na, act = "Not Active", "Active"
    row = "0, {} MHz, 2070 MHz, 900.00 W, 0x0, {}, {}, {}, {}"
    got = _clocks_from([row.format(2070, na, na, na, na), row.format(2040, na, na, na, act),
                        row.format(2070, na, na, na, na)])
    assert got["sm_mhz"] == 2070.0 and got["sm_max_mhz"] == 2070.0 and got["samples"] == 3
    assert got["reasons"] == ["sw_power_cap"]
    got = _clocks_from([row.format(1500, act, na, act, na), "garbage line"])
    assert got["samples"] == 1 and got["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]
