"""CPU checks of bench.py's command line (the GPU workloads stubbed): one
JSON line on stdout, the CPU baseline attached to the headline line of a
one-GPU run only, the per-workload default step counts."""
import json
import sys

import pytest

sys.path.insert(0, __import__("os").path.dirname(__import__("os").path.dirname(__file__)))
import bench  # noqa: E402


def run_main(monkeypatch, capsys, argv):
    seen = {}

    def fake(name):
        def run(args, rank, world, local):
            seen["args"] = args
            return {"metric": "tours/s", "value": 1.0, "workload": name}
        return run

    for name in ("run_ours", "run_batch", "run_learned", "run_large", "run_parity"):
        monkeypatch.setattr(bench, name, fake(name))
    monkeypatch.setattr(bench, "cpu_baseline", lambda: {"value": 2.0, "kind": "port"})
    monkeypatch.setattr(bench, "parity_cpu_baseline", lambda: {"value": 3.0, "kind": "port"})
    monkeypatch.setattr(bench, "batch_cpu_sample", lambda **kw: (4.0, 2, "sample"))
    monkeypatch.setattr(sys, "argv", ["bench.py"] + argv)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    bench.main()
    lines = [l for l in capsys.readouterr().out.splitlines() if l.strip()]
    assert len(lines) == 1
    return json.loads(lines[0]), seen["args"]


def test_headline_line_carries_the_cpu_baseline(monkeypatch, capsys):
    out, args = run_main(monkeypatch, capsys, [])
    assert out["workload"] == "run_parity" and out["cpu_baseline"]["value"] == 3.0
    assert args.steps == bench.DEFAULT_STEPS["parity_batch8"] and args.warmup >= 3


def test_single_colony_line_carries_its_cpu_baseline(monkeypatch, capsys):
    out, args = run_main(monkeypatch, capsys, ["--workload", "rbas_aging_n1000"])
    assert out["workload"] == "run_ours" and out["cpu_baseline"]["value"] == 2.0
    assert args.steps == bench.DEFAULT_STEPS["rbas_aging_n1000"]


def test_both_arms_share_the_parity_config():
    """The reference arm and the GPU arm print the same config dict."""
    import inspect
    src_ref = inspect.getsource(bench.run_reference_parity)
    src_gpu = inspect.getsource(bench.run_parity)
    for src in (src_ref, src_gpu):
        assert "dict(parity_config()" in src
    p = bench.parity_params()
    from acogpu_gb300 import _abi
    assert p.cand_k == 0 and p.nn_order == _abi.ACO_NN_REFERENCE_QSORT
    assert p.heuristic == _abi.ACO_HEURISTIC_LIBM and p.fallback == _abi.ACO_FALLBACK_REFERENCE
    assert p.tau0_mode == _abi.ACO_TAU0_REFERENCE and p.aging == 1


def test_no_cpu_baseline_flag(monkeypatch, capsys):
    out, _ = run_main(monkeypatch, capsys, ["--no-cpu-baseline", "--steps", "7"])
    assert "cpu_baseline" not in out


@pytest.mark.parametrize("workload,fn", [("large4096", "run_large"), ("learned", "run_learned")])
def test_other_workloads(monkeypatch, capsys, workload, fn):
    out, args = run_main(monkeypatch, capsys, ["--workload", workload])
    assert out["workload"] == fn and "cpu_baseline" not in out
    assert args.steps == bench.DEFAULT_STEPS[workload]


def test_batch_line_carries_the_sampled_cpu_baseline(monkeypatch, capsys):
    out, args = run_main(monkeypatch, capsys, ["--workload", "batch512"])
    assert out["workload"] == "run_batch" and out["cpu_baseline"]["value"] == 4.0
    assert args.steps == bench.DEFAULT_STEPS["batch512"]
