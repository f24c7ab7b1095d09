"""The bench's one-line record (no GPU): it carries the contract's keys and a
summary of every leg, and stays short enough that a 1 500-character tail of
the run's output holds all of it."""
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _bench():
    sys.path.insert(0, str(ROOT))
    import bench

    return bench


def _full_result(bench):
    big = 1234567890.123456
    return {
        "metric": "cell-updates/s", "value": big, "unit": "cell-updates/s", "n_gpus": 1,
        "steps": 20, "warmup": 3, "ms_per_step": 2.6833333, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "gpu_launches": 40, "config": bench.config(),
        "e2e": {"value": big, "unit": "cell-updates/s", "h2d_bytes_per_step": 127401984,
                "d2h_bytes_per_step": 127402000},
        "cpu_baseline": {"value": 54712345.6789, "unit": "cell-updates/s", "cores": 16,
                         "kind": "port", "sample": "8 patch rows (512 patches) per step, 1253 steps"},
        "roofline": {"bound": "hbm", "achieved": 87.7912345, "peak": 6686.1, "unit": "GB/s",
                     "frac": 0.013123456, "traffic": 233024256.0, "kernel_ms": 2.6},
        "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"],
                   "samples": 40},
        "fp64": {"frac_of_measured_dfma": 0.84912345, "achieved_gops": 446.78,
                 "peak_dfma_gops": 526.355},
        "plain_per_patch": {"value": 126651401.69, "lone_patch_us": 121.52},
        "served": {"value": 3061234567.8, "scenarios": 64,
                   "workload": "64 flood scenarios, cells log-uniform [1e4, 4e6], mx in {8,16,32}, "
                               "dx 5 m, horizons 1-6 h x1",
                   "p50_latency_s": 20.81234, "p99_latency_s": 96.1234,
                   "slowdown_vs_isolated": {"p50": 3.061234, "p99": 5.861234},
                   "wet_fraction": 0.0504524, "vs_plain_per_patch": 95.31234,
                   "alone_equals_mix": True},
        "batched": {"value": 394999999.9, "speedup_vs_one_by_one": 1.131234,
                    "batch_equals_one_by_one": True},
        "forest": {"value": 42171234.5, "regrid_parity": {"mismatching_regrids": 0},
                   "to_60s": {"subcycled_batch": {"speedup_vs_one_by_one": 3.881234}}},
        "served_amr": {"value": 343612345.6, "p99_latency_s": 0.635123,
                       "slowdown_vs_isolated": {"p99": 7.181234}},
        "large": {"value": 547412345.6},
        "dem": {"value": 1461234567.8},
    }


def test_compact_line_keeps_the_contract_keys_and_fits_the_tail():
    bench = _bench()
    line = json.dumps(bench.compact(_full_result(bench)), separators=(",", ":"))
    assert len(line) <= 1450, len(line)
    d = json.loads(line)
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "e2e", "gpu_launches", "roofline", "cpu_baseline", "clocks"):
        assert k in d, k
    assert set(d["roofline"]) >= {"bound", "achieved", "peak", "unit", "frac", "traffic"}
    assert set(d["clocks"]) == {"sm_mhz", "sm_max_mhz", "reasons"}
    for leg in ("served", "batched", "forest", "served_amr", "fp64", "plain_per_patch"):
        assert leg in d, leg
    assert {"p50_s", "p99_s", "slowdown_p99", "vs_plain_per_patch"} <= set(d["served"])


def test_both_arms_share_the_config():
    bench = _bench()
    assert bench.config() == bench.config()
    assert "sample" not in bench.config()
