"""Host logic of bench.py that needs no GPU: the short batch / adjoint legs
carried on the main line report a failing leg as an error entry instead of
losing the line, and run with their own small step counts."""
import argparse
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_other_configs_reports_a_failing_leg(monkeypatch):
    seen = {}

    def ok(a, ws, local):
        seen["batch"] = (a.steps, a.warmup, a.fp64_sample, ws)
        return {"value": 1.0}

    def bad(a, ws, local):
        seen["adjoint"] = (a.steps, a.warmup, ws)
        raise RuntimeError("no device")

    monkeypatch.setattr(bench, "batch_result", ok)
    monkeypatch.setattr(bench, "adjoint_result", bad)
    args = argparse.Namespace(steps=10, warmup=3, fp64_sample=16)
    out = bench.other_configs(args, 0)
    assert out["batch"]["value"] == 1.0 and "wall_s" in out["batch"]
    assert out["adjoint"]["error"] == "RuntimeError: no device" and "wall_s" in out["adjoint"]
    assert seen["batch"] == (2, 1, 8, 1) and seen["adjoint"] == (5, 1, 1)
    assert args.steps == 10 and args.warmup == 3  # the main run's arguments are untouched


def test_workload_names():
    assert bench.workload_info("rmat22")[1] == "rmat15_32_64"
    desc, sample = bench.workload_info("rmat23_32_64")
    assert "RMAT scale 23" in desc and sample == "rmat14_32_64"
