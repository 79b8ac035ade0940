#!/usr/bin/env python3
"""Benchmark of the ApplicationClassification match on GB300.

One step = one whole match (cdist, initial normalisers and edge maxima, every
BP iteration, output in [Dn][Pn]) of the named synthetic workload, with the
data graph's CSR orderings built beforehand (they are per data graph, shared by
every pattern).  Prints one JSON line:

  value       match ms, job level: (max-over-ranks time of the K timed
              steps) / (K * ranks); inputs resident in HBM, larger than L2
  e2e         the same metric through the one-shot C-ABI call from pinned
              host buffers (acg_match_graphs_host): every step copies both
              graphs host->device, builds the CSRs, matches and copies mu back
              to the host
  roofline    the dominant kernel (the edge phase of a BP iteration) against
              the measured HBM copy bandwidth; the vertex phase beside it
  plain_fp64  the same match computed entirely in FP64, with the error of
              the mixed result against it
  cpu_baseline  the CPU oracle (a pass-by-pass restatement of the reference)
              on a bounded sample of the workload, scaled to a whole match,
              on all host threads and on one
  configs     short runs of the many-pattern batch and of the adjoint (the
              lines of --batch and --adjoint, with fewer steps)

``--impl reference`` times the CPU oracle instead (the reference program's
own CPU build needs its sources, which only the development machine has).
Multi-GPU runs are independent replicas (one match per rank, no collective in
the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    # name: (description, sample workload for the CPU baseline)
    "rmat22": ("RMAT scale 22 (4,194,304 vertices, edge factor 16, a=.57 b=c=.19, dedup, "
               "no self-loops), planted pattern 32 vertices / 64 edges, 13/17-dim N(0,1) features, "
               "seed 2", "rmat15_32_64"),
    "rmat18": ("RMAT scale 18 (262,144 vertices, edge factor 16), planted pattern 16 / 32, "
               "13/17-dim N(0,1) features, seed 1", "rmat14_16_32"),
    "rmat20": ("RMAT scale 20, planted pattern 16 / 32, seed 3", "rmat14_16_32"),
    "rmat16": ("RMAT scale 16 (65,536 vertices, edge factor 16), planted pattern 12 / 24, "
               "13/17-dim N(0,1) features, seed 4", "rmat14_12_24"),
    "rmat12": ("RMAT scale 12 (4,096 vertices, edge factor 16), planted pattern 12 / 24, "
               "13/17-dim N(0,1) features, seed 4", "rmat12_12_24"),
    "er1k": ("Erdos-Renyi 1,000 vertices / 20,000 edges, planted pattern 10 / 20, seed 0",
             "er1k"),
}


def workload_info(name: str):
    """(description, CPU-baseline sample) of a named workload."""
    if name in WORKLOADS:
        return WORKLOADS[name]
    parts = name[4:].split("_") if name.startswith("rmat") else []
    if len(parts) != 3 or not all(x.isdigit() for x in parts):
        raise SystemExit(f"unknown workload {name!r}")
    sc, pn, pe = (int(x) for x in parts)
    return (f"RMAT scale {sc} (edge factor 16, a=.57 b=c=.19, dedup, no self-loops), planted "
            f"pattern {pn} / {pe}, 13/17-dim N(0,1) features, seed {sc}",
            f"rmat{min(sc, 14)}_{pn}_{pe}")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="rmat22",
                    help="one of %s, or rmatS_P_E (RMAT scale S, pattern P/E)" % sorted(WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--edge-kernel", default="auto", choices=["auto", "stored", "fused"],
                    help="the mixed path's edge phase: read the stored edge cost matrix, or "
                         "recompute the costs on the tensor cores (acg_options.edge_kernel)")
    ap.add_argument("--cdist-kernel", default="auto", choices=["auto", "simt", "tensor"],
                    help="mixed path: cost matrices on the tensor cores where the shape allows "
                         "(auto), always on the CUDA cores (simt), or tensor cores only "
                         "(acg_options.cdist_kernel)")
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--e2e-warmup", type=int, default=2)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the short batch and adjoint runs carried on the main line")
    ap.add_argument("--batch", action="store_true",
                    help="the many-pattern workload instead: R-MAT 20 with 64 planted patterns "
                         "(Pn 4..48, Pe 2..4 Pn), batched against sequential single matches")
    ap.add_argument("--adjoint", action="store_true",
                    help="time the backward (acg_backward) against the forward of one match "
                         "(RMAT-16 with a 12/24 pattern by default)")
    ap.add_argument("--adjoint-workload", default="rmat16")
    ap.add_argument("--checkpoint-every", type=int, default=4)
    ap.add_argument("--batch-scale", type=int, default=20)
    ap.add_argument("--no-autotune", action="store_true",
                    help="batch mode: greedy grouping with the default launch shapes")
    ap.add_argument("--batch-patterns", type=int, default=64)
    ap.add_argument("--fp64-sample", type=int, default=16,
                    help="patterns timed in sequential FP64 (scaled to all of them)")
    return ap.parse_args()


def dist_setup(backend):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend)
    return ws, rank, local


def max_over_ranks(x: float, ws: int, device=None) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


# ----------------------------------------------------------------- clocks
class Clocks:
    """nvidia-smi samples every 200 ms while running (clock and throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)], stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        time.sleep(0.25)
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {}


def ncu_traffic(workload: str, precision: str):
    """Per-launch DRAM bytes of the iteration kernel from a committed ncu summary."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    return d.get(f"{workload}/{precision}")


# ----------------------------------------------------------- CPU baseline
def cpu_sample(workload: str, threads: int | None = None):
    """Time the CPU oracle on the bounded sample; returns (ms per full match, info).

    The sample graph comes from the oracle's own generator (the same bytes as
    the product's), so this leg never loads the product library."""
    from oracle import oracle

    full = _work_units(workload)
    sample = workload_info(workload)[1]
    d, p, _ = oracle.workload(sample)
    nt = threads or os.cpu_count() or 1
    _, el_us = oracle.match(d, p, threads=nt, return_elapsed=True)
    units = _units(d.num_nodes, d.num_edges, p.num_nodes, p.num_edges)
    ms = el_us / 1e3 * full / units
    info = {"sample": f"{sample}: {d.num_nodes} vertices / {d.num_edges} edges, pattern "
                      f"{p.num_nodes}/{p.num_edges}; {el_us/1e6:.2f} s measured, scaled by "
                      f"(De+Dn)*Pe*(Pn+1) to the full workload (x{full/units:.1f})",
            "cores": nt, "sample_s": el_us / 1e6, "sample_ms_per_unit": el_us / 1e3 / units}
    return ms, info


def cpu_validation(ms_per_unit: float, threads: int, name: str = "rmat18"):
    """One measured oracle match of a larger workload (R-MAT 18, 16/32 pattern:
    the reference's GPU configuration) beside the sample model's prediction for
    it, so the extrapolation from the sample is checked, not assumed."""
    from oracle import oracle

    d, p, _ = oracle.workload(name)
    _, el_us = oracle.match(d, p, threads=threads, return_elapsed=True)
    pred = ms_per_unit * _units(d.num_nodes, d.num_edges, p.num_nodes, p.num_edges)
    meas = el_us / 1e3
    return {"workload": f"{name}: {d.num_nodes} vertices / {d.num_edges} edges, pattern "
                        f"{p.num_nodes}/{p.num_edges}",
            "measured_ms": round(meas, 1), "predicted_ms": round(pred, 1),
            "model_error": round(pred / meas - 1.0, 3)}


def cpu_model() -> str:
    """The host CPU's model name as lscpu reports it (best effort)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
    except (OSError, subprocess.SubprocessError):
        return "unknown"
    for line in out.splitlines():
        if line.lower().startswith("model name:"):
            return line.split(":", 1)[1].strip()
    return "unknown"


def _units(dn, de, pn, pe):
    return (de + dn) * max(pe, 1) * (pn + 1)


_SHAPES = {"rmat22": (4194304, 65242331, 32, 64), "rmat18": (262144, 3939126, 16, 32),
           "rmat20": (1048576, 16087353, 16, 32), "er1k": (1000, 20000, 10, 20)}


def _work_units(workload):
    if workload not in _SHAPES:
        from oracle import oracle
        d, p, _ = oracle.workload(workload)
        _SHAPES[workload] = (d.num_nodes, d.num_edges, p.num_nodes, p.num_edges)
    dn, de, pn, pe = _SHAPES[workload]
    return _units(dn, de, pn, pe)


# ------------------------------------------------------------------- ours
def run_ours(args, ws, rank, local):
    import numpy as np
    import torch

    from application_classification_gb300 import _lib, graph, matcher
    import ctypes as C

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    t0 = time.time()
    d, p, truth = graph.workload(args.workload)
    gen_s = time.time() - t0
    _SHAPES[args.workload] = (d.num_nodes, d.num_edges, p.num_nodes, p.num_edges)

    # ---- device-resident match
    dg = matcher.DataGraph(d)
    ek = args.edge_kernel if args.precision == "mixed" else "auto"
    ck = args.cdist_kernel if args.precision == "mixed" else "auto"
    plan = matcher.Plan(dg, p, args.precision, edge_kernel=ek, cdist_kernel=ck)
    out = torch.empty((d.num_nodes, p.num_nodes), dtype=torch.float64, device=dev)
    for _ in range(args.warmup):
        plan.run(out)
    torch.cuda.synchronize()
    barrier(ws)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ms_kernels = []
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            plan.run(out)
            ms_kernels.append(None)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier(ws)
    ms_total = ev0.elapsed_time(ev1)
    st = plan.stats()  # last match of the timed region
    ms_total = max_over_ranks(ms_total, ws, dev)
    value = ms_total / (args.steps * ws)
    mu_mixed = out.cpu().numpy()

    # per-phase durations (CUDA events around each phase of every iteration,
    # on a second plan so that the timed region above carries no extra events)
    del plan
    tplan = matcher.Plan(dg, p, args.precision, kernel_timing=True, edge_kernel=ek, cdist_kernel=ck)
    tplan.run(out)
    phase = []
    for _ in range(min(args.steps, 3)):
        tplan.run(out)
        phase.append(tplan.stats())
    del tplan
    iters = max(1, int(st["num_iters"]))
    edge_ms = statistics.median(x["ms_edge_phase"] for x in phase) / iters
    vert_ms = statistics.median(x["ms_vertex_phase"] for x in phase) / iters
    peaks = measured_peaks()
    peak = peaks.get("hbm_gbs") or 6800.0
    psrc = "MEASURED_PEAKS.json hbm_gbs" if peaks.get("hbm_gbs") else "fallback 6.8 TB/s"
    achieved = st["bytes_edge_phase"] / (edge_ms * 1e-3) / 1e9
    vachieved = st["bytes_vertex_phase"] / (vert_ms * 1e-3) / 1e9
    traffic = ncu_traffic(args.workload, args.precision)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic,
                "kernel": "edge_max_kernel (edge phase of one BP iteration: segmented max "
                          "over the destination-sorted CSR, plus the hub combine)",
                "launch_ms": round(edge_ms, 4),
                "algorithmic_bytes_per_launch": st["bytes_edge_phase"], "peak_source": psrc,
                "vertex_phase": {"kernel": "vertex_update_kernel + stat_finalize",
                                 "launch_ms": round(vert_ms, 4),
                                 "algorithmic_bytes_per_launch": st["bytes_vertex_phase"],
                                 "achieved": round(vachieved, 1),
                                 "frac": round(vachieved / peak, 4)}}

    result = {
        "metric": "match ms (one whole ApplicationClassification match, "
                  f"{args.precision} precision)",
        "value": round(value, 4), "unit": "ms", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_total / args.steps, 4),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {workload_info(args.workload)[0]}",
                   "data_vertices": d.num_nodes, "data_edges": d.num_edges,
                   "pattern_vertices": p.num_nodes, "pattern_edges": p.num_edges,
                   "precision": args.precision, "bp_iterations": int(st["num_iters"]),
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                   "l2": "inputs larger than L2 (edge cost matrix "
                         f"{d.num_edges * p.num_edges * (4 if args.precision == 'mixed' else 8) / 1e9:.2f} GB "
                         "streamed every iteration)",
                   "csr_prebuilt": True, "generation_s": round(gen_s, 1)},
        "phases_ms": {k: round(st[k], 3) for k in ("ms_cdist", "ms_init", "ms_iters", "ms_total")},
        "roofline": roofline,
        "gpu_launches": int(st["launches"]) * args.steps,
        "clocks": clk.summary(),
    }

    # ---- plain FP64 on the same input
    if not args.no_fp64 and args.precision == "mixed":
        pl64 = matcher.Plan(dg, p, "fp64")
        out64 = torch.empty_like(out)
        pl64.run(out64)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.fp64_steps):
            pl64.run(out64)
        e1.record(stream)
        torch.cuda.synchronize()
        ms64 = e0.elapsed_time(e1) / args.fp64_steps
        mu64 = out64.cpu().numpy()
        s64 = pl64.stats()
        # per-phase times of the FP64 iterations (a second plan with events
        # around each phase) against their bytes and their FP64 operations:
        # the edge phase does a subtraction and a maximum per (in-edge, column)
        t64 = matcher.Plan(dg, p, "fp64", kernel_timing=True)
        t64.run(out64)
        st64 = t64.stats()
        del t64
        it64 = max(1, int(st64["num_iters"]))
        e_ms = st64["ms_edge_phase"] / it64
        v_ms = st64["ms_vertex_phase"] / it64
        fp64_ops = 2.0 * d.num_edges * p.num_edges
        fp64_nominal = 1.25e12 / 2  # FP64 instructions per second (1.25 TFLOP/s counts an FMA as 2)
        fp64_roof = {
            "edge_phase": {"launch_ms": round(e_ms, 3), "bytes": st64["bytes_edge_phase"],
                           "achieved_gbs": round(st64["bytes_edge_phase"] / (e_ms * 1e-3) / 1e9, 1),
                           "hbm_frac": round(st64["bytes_edge_phase"] / (e_ms * 1e-3) / 1e9 / peak, 4),
                           "fp64_ops": fp64_ops,
                           "fp64_ops_per_s": round(fp64_ops / (e_ms * 1e-3), 1),
                           "fp64_frac_of_nominal": round(fp64_ops / (e_ms * 1e-3) / fp64_nominal, 4)},
            "vertex_phase": {"launch_ms": round(v_ms, 3), "bytes": st64["bytes_vertex_phase"],
                             "achieved_gbs": round(st64["bytes_vertex_phase"] / (v_ms * 1e-3) / 1e9, 1),
                             "hbm_frac": round(st64["bytes_vertex_phase"] / (v_ms * 1e-3) / 1e9 / peak, 4)},
            "bound": "fp64 pipe (GB300's FP64 rate: nominal 1.25 TFLOP/s, 1/64 of its FP32 rate), "
                     "not HBM",
            "nominal_fp64": "1.25 TFLOP/s, NVIDIA's figure (no measured FP64 peak on this pool)",
        }
        diff = np.abs(mu_mixed - mu64)
        a64, am = mu64.argmax(1), mu_mixed.argmax(1)
        srt = np.sort(mu64, axis=1)
        gap = srt[:, -1] - srt[:, -2]
        tie = gap <= 2 * float(diff.max())  # unresolvable at the mixed path's precision
        result["plain_fp64"] = {
            "ms": round(ms64, 3), "speedup_mixed_vs_fp64": round(ms64 / value, 2),
            "phases_ms": {k: round(s64[k], 3) for k in ("ms_cdist", "ms_init", "ms_iters")},
            "roofline": fp64_roof,
            "max_abs_dmu": float(diff.max()), "max_abs_mu": float(np.abs(mu64).max()),
            "argmax_identical_except_ties": bool(((a64 == am) | tie).all()),
            "argmax_mismatch_rows": int((a64 != am).sum()),
            "argmax_mismatch_min_fp64_gap": float(gap[a64 != am].min()) if (a64 != am).any() else None,
            "tie_rule": "FP64 top-2 gap <= 2 x max_abs_dmu",
            "planted_recovered": int(sum(int(mu64[:, i].argmax()) == int(truth[i])
                                         for i in range(p.num_nodes))),
        }
        del pl64, out64

    # ---- end to end through the one-shot C-ABI call, host buffers
    if not args.no_e2e:
        def pinned(a):
            t = torch.from_numpy(a.view(np.int64) if a.dtype == np.uint64 else a)
            return t.pin_memory()

        hs = [pinned(x) for x in (d.node_feats, d.edge_feats, d.srcs, d.dsts,
                                  p.node_feats, p.edge_feats, p.srcs, p.dsts)]
        mu_host = torch.empty((d.num_nodes, p.num_nodes), dtype=torch.float64).pin_memory()
        opt = _lib.Options()
        _lib.lib().acg_options_default(C.byref(opt))
        opt.precision = matcher.PRECISIONS[args.precision]
        # acg_graph views of the pinned HOST arrays
        gd = matcher.DeviceGraph.from_tensors(*hs[:4]).c_graph()
        gp = matcher.DeviceGraph.from_tensors(*hs[4:]).c_graph()

        def e2e_step():
            # host graphs in, host mu out: copies, CSR build, allocation, match
            _lib.check(_lib.lib().acg_match_graphs_host(C.byref(gd), C.byref(gp), C.byref(opt),
                                                        C.c_void_p(mu_host.data_ptr()),
                                                        C.c_void_p(stream.cuda_stream)), "e2e")

        for _ in range(args.e2e_warmup):  # the library's memory pool grows to its working size
            e2e_step()
        torch.cuda.synchronize()
        barrier(ws)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step_ms = []
        for _ in range(args.e2e_steps):
            t_0 = time.perf_counter()
            e2e_step()  # returns once mu is in host memory
            step_ms.append(round((time.perf_counter() - t_0) * 1e3, 1))
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(ws)
        e2e_ms = max_over_ranks(e0.elapsed_time(e1), ws, dev) / (args.e2e_steps * ws)
        result["e2e"] = {"value": round(e2e_ms, 3), "unit": "ms",
                         "h2d_bytes_per_step": int(sum(h.numel() * h.element_size() for h in hs)),
                         "d2h_bytes_per_step": int(mu_host.numel() * 8),
                         "steps": args.e2e_steps,
                         "includes": "acg_match_graphs_host: H2D of both graphs (mixed: the edge "
                                     "features in 16 pieces, each turned into FP32 rows and edge-cost "
                                     "rows as it lands, under the CSR build and the plan), CSR build, "
                                     "allocation, match, D2H of mu",
                         "warmup": args.e2e_warmup, "step_ms_host": step_ms}
        del hs

    # ---- CPU baseline (rank 0, N=1 only)
    if rank == 0 and ws == 1 and not args.no_cpu:
        ms, info = cpu_sample(args.workload)
        result["cpu_baseline"] = {"value": round(ms, 1), "unit": "ms", "cores": info["cores"],
                                  "kind": "port", "sample": info["sample"], "cpu": cpu_model(),
                                  "validation": cpu_validation(info["sample_ms_per_unit"],
                                                               info["cores"])}
        if info["cores"] > 1:  # the same sample on one thread
            ms1, info1 = cpu_sample(args.workload, threads=1)
            result["cpu_baseline"]["single_thread"] = {
                "value": round(ms1, 1), "unit": "ms", "cores": 1,
                "sample_s": round(info1["sample_s"], 2),
                "thread_scaling": round(ms1 / ms, 2)}
    # ---- the many-pattern and gradient configurations, short runs (N=1 only)
    if ws == 1 and not args.no_configs:
        result["configs"] = other_configs(args, local)
    if rank == 0:
        print(json.dumps(result), flush=True)


def other_configs(args, local) -> dict:
    """Short runs of the batch (64 patterns against R-MAT 20) and the adjoint
    (R-MAT 16, 12 / 24 pattern) legs, carried on the main line so that one
    default run records every configuration; `bench.py --batch` / `--adjoint`
    time them with the full step counts.  A leg that fails reports its error."""
    import argparse as _ap

    out = {}
    for name, fn, steps in (("batch", batch_result, 2), ("adjoint", adjoint_result, 5)):
        a = _ap.Namespace(**vars(args))
        a.steps, a.warmup, a.fp64_sample = steps, 1, 8
        t0 = time.time()
        try:
            out[name] = fn(a, 1, local)
        except Exception as e:  # noqa: BLE001 -- the main line must still print
            out[name] = {"error": f"{type(e).__name__}: {e}"}
        out[name]["wall_s"] = round(time.time() - t0, 1)
    return out


# -------------------------------------------------------------- reference
def run_reference(args, ws, rank):
    """The CPU oracle (restatement of the reference program) on a bounded sample."""
    if rank != 0:
        return
    from oracle import oracle

    full = _work_units(args.workload)
    sample = workload_info(args.workload)[1]
    d, p, _ = oracle.workload(sample)  # the oracle's generator: no product library here
    nt = os.cpu_count() or 1
    units = _units(d.num_nodes, d.num_edges, p.num_nodes, p.num_edges)
    for _ in range(args.warmup):
        oracle.match(d, p, threads=nt)
    els = []
    t0 = time.time()
    for _ in range(args.steps):
        _, el = oracle.match(d, p, threads=nt, return_elapsed=True)
        els.append(el / 1e3)
    wall = time.time() - t0
    ms_sample = sum(els) / len(els)
    value = ms_sample * full / units
    validation = cpu_validation(ms_sample / units, nt)
    print(json.dumps({
        "impl": "reference",
        "metric": "match ms (one whole ApplicationClassification match, "
                  f"{args.precision} precision)",
        "value": round(value, 1), "unit": "ms", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_sample, 2), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {workload_info(args.workload)[0]}",
                   "precision": "fp64 (the reference computes in FP64)"},
        "cpu_baseline": {"value": round(value, 1), "unit": "ms", "cores": nt, "kind": "port",
                         "cpu": cpu_model(),
                         "sample": f"{sample}: {d.num_nodes} vertices / {d.num_edges} edges, "
                                   f"pattern {p.num_nodes}/{p.num_edges}, {ms_sample/1e3:.2f} s per "
                                   f"sample match, scaled by (De+Dn)*Pe*(Pn+1) x{full/units:.1f}",
                         "validation": validation},
        "e2e": {"value": round(value, 1), "unit": "ms", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "wall_s": round(wall, 1),
    }), flush=True)


# ------------------------------------------------------------------ batch
def run_batch(args, ws, rank, local):
    """One data graph against many patterns: one acg_batch launch (all patterns,
    one CUDA graph) against the same patterns matched one after another."""
    out = batch_result(args, ws, local)
    if rank == 0:
        print(json.dumps(out), flush=True)


def batch_result(args, ws, local) -> dict:
    """The measurements of run_batch as one dict (the bench line's fields)."""
    import numpy as np
    import torch

    from application_classification_gb300 import graph, matcher

    torch.cuda.set_device(local)
    t0 = time.time()
    d, pats, truths = graph.batch_workload(args.batch_scale, args.batch_patterns, seed=3)
    gen_s = time.time() - t0
    dg = matcher.DataGraph(d)
    prec = args.precision
    t0 = time.time()
    b = matcher.Batch(dg, pats, prec, autotune=not args.no_autotune)
    create_s = time.time() - t0
    for _ in range(max(1, args.warmup)):
        b.run()
    torch.cuda.synchronize()
    barrier(ws)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            outs = b.run()
        e1.record(stream)
        torch.cuda.synchronize()
    barrier(ws)
    ms_batch = max_over_ranks(e0.elapsed_time(e1) / args.steps, ws)
    info = b.info()
    mus = [o.cpu().numpy() for o in outs]
    del b
    greedy = None
    if not args.no_autotune:  # the default grouping, for comparison (one timed run)
        bg = matcher.Batch(dg, pats, prec)
        bg.run()
        torch.cuda.synchronize()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        bg.run()
        g1.record(stream)
        torch.cuda.synchronize()
        greedy = {"ms": round(g0.elapsed_time(g1), 2), "groups": bg.info()["groups"]}
        del bg

    def sequential(precision, subset):
        # one plan at a time (all of them at once would not fit in memory); the
        # device time of each match is summed, plan creation excluded
        total, res = 0.0, []
        for k, i in enumerate(subset):
            pl = matcher.Plan(dg, pats[i], precision)
            if k == 0:
                pl.run()  # warm-up
            torch.cuda.synchronize()
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            r = pl.run()
            s1.record(stream)
            torch.cuda.synchronize()
            total += s0.elapsed_time(s1)
            res.append(r.cpu().numpy())
            del pl, r
        return total, res

    n = len(pats)
    ms_seq, seq = sequential(prec, range(n))
    err = max(float(np.abs(a - b_).max()) for a, b_ in zip(mus, seq))
    sub = list(range(0, n, max(1, n // max(1, args.fp64_sample))))[:args.fp64_sample]
    ms64_sub, mu64 = sequential("fp64", sub)
    ms64 = ms64_sub * n / len(sub)
    err64 = max(float(np.abs(mus[i] - m).max()) for i, m in zip(sub, mu64))
    recovered = sum(int(mu64[k][:, j].argmax()) == int(truths[i][j])
                    for k, i in enumerate(sub) for j in range(pats[i].num_nodes))
    total_pn = sum(pats[i].num_nodes for i in sub)
    value = n / (ms_batch * 1e-3)
    return {
            "metric": f"patterns matched per second (one data graph, {n} patterns, batched, "
                      f"{prec} precision)",
            "value": round(value, 2), "unit": "patterns/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_batch, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if prec == "mixed" else "f64", "data": "synthetic",
            "config": {"workload": f"rmat{args.batch_scale} + {n} planted patterns (Pn 4..48, "
                                   "Pe 2..4 Pn, seeds 3000+i)",
                       "data_vertices": d.num_nodes, "data_edges": d.num_edges,
                       "pattern_vertices_total": sum(p.num_nodes for p in pats),
                       "pattern_edges_total": sum(p.num_edges for p in pats),
                       "generation_s": round(gen_s, 1), "batch_create_s": round(create_s, 1)},
            "batch": info,
            "greedy_grouping": greedy,
            "autotune_model_over_measured": (round(info["predicted_ms"] / ms_batch, 3)
                                             if info.get("autotuned") else None),
            "sequential_same_precision_ms": round(ms_seq, 2),
            "speedup_vs_sequential_same_precision": round(ms_seq / ms_batch, 3),
            "max_abs_dmu_vs_sequential": err,
            "sequential_plain_fp64_ms": round(ms64, 1),
            "sequential_plain_fp64_sample": f"{len(sub)} of {n} patterns timed, scaled x{n/len(sub):.1f}",
            "speedup_vs_sequential_plain_fp64": round(ms64 / ms_batch, 2),
            "max_abs_dmu_vs_fp64_sample": err64,
            "planted_recovered_fp64_sample": f"{recovered} of {total_pn}",
            "clocks": clk.summary(),
    }


def run_adjoint(args, ws, rank, local):
    """Forward (acg_match, and acg_match_record which also keeps checkpoints)
    against the backward (acg_backward) of one match.  Loss: the sum of mu --
    the log of the normalised assignment probability -- over the planted
    (data vertex, pattern vertex) pairs, so grad_mu is one-hot there."""
    out = adjoint_result(args, ws, local)
    if rank == 0:
        print(json.dumps(out), flush=True)


def adjoint_result(args, ws, local) -> dict:
    """The measurements of run_adjoint as one dict (the bench line's fields)."""
    import numpy as np
    import torch

    from application_classification_gb300 import graph, matcher

    torch.cuda.set_device(local)
    d, p, truth = graph.workload(args.adjoint_workload)
    dg = matcher.DataGraph(d)
    stream = torch.cuda.current_stream()
    gmu = torch.zeros((d.num_nodes, p.num_nodes), dtype=torch.float64, device="cuda")
    gmu[torch.as_tensor(np.asarray(truth, dtype=np.int64)), torch.arange(p.num_nodes)] = 1.0
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")  # 256 MB > L2

    def timed(fn, n):
        # each call alone between events, L2 flushed before it
        tot = 0.0
        for _ in range(n):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        return tot / n

    res, grads = {}, {}
    clk_summary = None
    for prec in (args.precision, "fp64"):
        pl = matcher.Plan(dg, p, prec)
        mu = pl.record(checkpoint_every=args.checkpoint_every)
        for _ in range(max(1, args.warmup)):
            pl.run(mu)
            pl.record(mu, args.checkpoint_every)
            pl.backward(gmu)
        torch.cuda.synchronize()
        barrier(ws)
        with Clocks(local) as clk:
            ms_fwd = timed(lambda: pl.run(mu), args.steps)
            ms_rec = timed(lambda: pl.record(mu, args.checkpoint_every), args.steps)
            ms_bwd = timed(lambda: pl.backward(gmu), args.steps)
        if prec == args.precision:
            clk_summary = clk.summary()
        barrier(ws)
        res[prec] = {k: round(max_over_ranks(v, ws), 3)
                     for k, v in (("forward_ms", ms_fwd), ("forward_record_ms", ms_rec),
                                  ("backward_ms", ms_bwd))}
        res[prec]["backward_over_forward"] = round(res[prec]["backward_ms"] / res[prec]["forward_ms"], 3)
        grads[prec] = [x.cpu().numpy() for x in pl.backward(gmu)]
        del pl
    names = ["data_node", "data_edge", "pattern_node", "pattern_edge"]
    rel = {n: float(np.linalg.norm(a - b) / max(1e-300, np.linalg.norm(b)))
           for n, a, b in zip(names, grads[args.precision], grads["fp64"])}
    r = res[args.precision]
    return {
            "metric": "backward time / forward time of one match (gradients of the planted-pair "
                      "log-probabilities w.r.t. all four feature arrays)",
            "value": r["backward_over_forward"], "unit": "x", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["backward_ms"], "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.precision == "mixed" else "f64", "data": "synthetic",
            "config": {"workload": workload_info(args.adjoint_workload)[0],
                       "data_vertices": d.num_nodes, "data_edges": d.num_edges,
                       "pattern": [p.num_nodes, p.num_edges],
                       "checkpoint_every": args.checkpoint_every, "precision": args.precision,
                       "l2": "flushed (256 MB write) before every timed call"},
            "timings": res,
            "grad_rel_frobenius_vs_fp64": rel,
            "clocks": clk_summary,
    }


def main():
    args = parse()
    if args.impl == "reference":
        ws, rank, _ = dist_setup("gloo")
        run_reference(args, ws, rank)
    else:
        ws, rank, local = dist_setup("nccl")
        if args.batch:
            run_batch(args, ws, rank, local)
        elif args.adjoint:
            run_adjoint(args, ws, rank, local)
        else:
            run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
