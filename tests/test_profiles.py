"""The measured figures the bench line reads from profiles/ (CPU).

bench.py takes `roofline.traffic` from profiles/traffic_<workload>.json and
`roofline.dominant` from profiles/launches_<workload>.json.  These checks keep
those summaries self-consistent: DRAM traffic with writes counted can not be
below the step's algorithmic bytes (every field the step reads and writes once),
and the launch-list shares are fractions of one total.
"""
import json
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROF = os.path.join(ROOT, "profiles")

# algorithmic bytes per grid point and step (bench.py ALG_BYTES_STEP): every state
# field read and written once, every model field read once -- acoustic 7 state
# x 8 B + 4 model x 4 B, constant-Q 8 state x 8 B + 8 model x 4 B
ALG = {"artm3": 72.0, "qrtm4": 96.0}


@pytest.mark.parametrize("workload", sorted(ALG))
def test_traffic_is_not_below_the_algorithmic_bytes(workload):
    p = os.path.join(PROF, f"traffic_{workload}.json")
    if not os.path.exists(p):
        pytest.skip("no traffic summary")
    t = json.load(open(p))
    assert t["bytes_per_point"] >= ALG[workload], t
    assert t["dram_bytes_per_step"] > 0


def test_launch_list_shares():
    p = os.path.join(PROF, "launches_qrtm4.json")
    if not os.path.exists(p):
        pytest.skip("no launch list")
    L = json.load(open(p))
    ks = L["kernels"]
    assert sum(k["launches"] for k in ks) == L["launches"]
    assert abs(sum(k["total_ms"] for k in ks) - L["total_ms"]) < 1e-3 * L["total_ms"]
    assert abs(sum(k["share"] for k in ks) - 1.0) < 1e-3
    shares = [k["share"] for k in ks]
    assert shares == sorted(shares, reverse=True)
