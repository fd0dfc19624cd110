"""The JSON line bench.py prints for the reference arm, on the CPU: one
rank, a one-grid workload, every key the driver reads, and the form
selector the GPU arm's legs use."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    sys.path.insert(0, ROOT)
    import bench
    return bench


def test_reference_arm_line(capsys):
    bench = _bench()

    class A:
        tiles, n, steps, warmup, gpus = (1, 1, 1), 8, 1, 1, 1
    assert bench.run_reference(A(), rank=0) == 0
    out = [ln for ln in capsys.readouterr().out.splitlines() if ln.startswith("{")]
    assert len(out) == 1
    d = json.loads(out[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["higher_is_better"] is True and d["value"] > 0
    assert d["config"]["same_config"] is True and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_flow_params_forms():
    bench = _bench()
    from mglet_gb300 import abi
    assert bench.flow_params("mixed").form == abi.FORM_MIXED
    assert bench.flow_params("plain").form == abi.FORM_PLAIN
    assert bench.flow_params("plain_fma").form == abi.FORM_PLAIN_FMA
    p = bench.flow_params("mixed")
    assert (p.ninner, p.nouter, p.epcorr) == (5, 9, 1e-10)
