"""Benchmark of the GB300 P3 step (prints ONE JSON line on rank 0).

Workload (headline): P3 precision form, ncol=345,600 x nlev=128, dt=300 s,
state carried across steps, FP32-bulk (process rates and table interpolation
in FP32, FP64 state / residuals / fluxes).  The plain FP64 form is timed on
the same workload and reported beside it.  A "step" is one p3_main call over
all columns.  Inputs (15.9 GB per step) are larger than L2, so no flush is
needed between steps.

  value       column-levels/s of the FP32-bulk step, inputs resident in HBM
  e2e         the same step through the public API on pinned HOST arrays
              (p3x_main_host): every step copies the 23 input fields
              host->device and the 20 per-level outputs + 2 interface fluxes +
              2 surface fields back, in column chunks overlapped with the
              kernels
  roofline    HBM roofline of the P3 step (three kernels: part1+part2,
              sedimentation, part3) at 360 algorithmic bytes per column-level
              (23 FP64 inputs read, 22 FP64 outputs written), with each
              kernel's share of the step measured live with CUDA events
  batched     the batched form: 256 instances (ncol log-uniform [1,16384],
              nlev 72/128, dt 300/120 s) in one persistent launch sequence
              replayed from a captured CUDA graph, launch configuration picked
              by the autotuner, FP64 and FP32-bulk
  serving     the request loop: Poisson sessions (ncol log-uniform
              [1,65536], nlev 72/128, FP64/FP32-bulk 50/50, 1-20 steps) at
              80% of the capacity measured in the same run, 120 GB budget
  cpu_baseline  the CPU oracle (a C++/OpenMP restatement of the reference
              p3_main) on the whole workload, 10 steps with the state
              carried, all host cores
  precision   per-field rel-L2 / max-abs of both GPU forms against that
              oracle run over all columns after 1 and 10 steps, the
              oracle's own 1-ulp spread, domain-total precipitation per step
              and every column's 10-step water budget

--impl reference times the CPU oracle alone on the same whole workload (the
reference itself cannot be built: its EKAT/Kokkos submodules are empty).
Multi-GPU (torchrun): each rank runs its own 345,600 columns (weak scaling,
no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NCOL, NLEV, DT = 345_600, 128, 300.0
ALG_BYTES_PER_CL = 360.0
SEED = 1002  # seed of the 345,600-column RH-stress workload
METRIC = "P3 column-levels/sec at nlev=128 (FP32-bulk; FP64 beside it)"
DATA = "synthetic (seeded standard-atmosphere columns, RH~U(0.9,1.05) in even columns)"


def workload_config(ncol):
    """The `config` object of both arms' lines."""
    gb = ALG_BYTES_PER_CL * ncol * NLEV / 1e9  # interface fields read and written per step
    l2 = f"interface fields {gb:.1f} GB/step > L2 (no flush needed)" if gb > 0.129 else \
        f"interface fields {gb:.3f} GB/step < L2"
    return {"workload": f"P3 p3_main ncol={ncol} nlev={NLEV} dt={DT}s, state carried", "l2": l2,
            "columns_per_gpu": ncol}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def rank_seed(rank):
    """Workload seed of a rank: each rank steps its own columns (weak scaling)."""
    return SEED + 7919 * rank


def reduce_max(x):
    """Maximum of a host float over all ranks (the slowest rank sets the
    job's time); identity without a process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def weak_value(world_size, cl_per_rank_step, steps, wall_max):
    """Whole-job column-levels/s: every rank's work over the slowest rank's time."""
    return world_size * cl_per_rank_step * steps / wall_max


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def _profile_figure(kernel_tag, key):
    """A per-column-level figure of the step (``dram_bytes_per_cl``,
    ``fp64_warp_inst_per_cl``) from the committed ncu summary (profiles/), or
    None."""
    f = ROOT / "profiles" / "p3_step_traffic_65536x128.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith(kernel_tag + " " + key):
            return float(line.split()[-1])
    return None


def _traffic_per_cl(kernel_tag):
    """DRAM bytes per column-level of the column kernels, or None."""
    return _profile_figure(kernel_tag, "dram_bytes_per_cl")


# FP64-pipe issue rate of one SM on this part: one warp instruction per 16
# cycles (ncu: sm__pipe_fp64_cycles_active / sm__inst_executed_pipe_fp64)
FP64_CYCLES_PER_WARP_INST = 16.0


def fp64_ceiling(kernel_tag, cl_step, ms_per_step, sm_mhz, num_sms):
    """The step's floor set by the FP64 pipe alone: FP64-pipe warp
    instructions per column-level (committed ncu summary) x 16 cycles over
    the SMs at the sampled SM clock, and the measured step's fraction of it."""
    ipc = _profile_figure(kernel_tag, "fp64_warp_inst_per_cl")
    if ipc is None or not sm_mhz or not ms_per_step:
        return None
    floor_ms = ipc * FP64_CYCLES_PER_WARP_INST * cl_step / (num_sms * sm_mhz * 1e6) * 1e3
    return {"fp64_warp_inst_per_cl": ipc, "floor_ms": floor_ms, "frac": floor_ms / ms_per_step,
            "sm_mhz": sm_mhz, "sms": num_sms,
            "note": "floor = FP64-pipe warp instructions x 16 cycles / (SMs x SM clock); frac = floor / "
                    "measured step (1.0 would be an FP64-pipe-bound step with nothing else in the way)"}


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


PRECISION_FIELDS = ["qc", "nc", "qr", "nr", "qi", "qm", "ni", "bm", "qv", "th", "precip_liq_surf",
                    "precip_ice_surf", "precip_liq_flux", "diag_eff_radius_qc", "diag_eff_radius_qr",
                    "diag_eff_radius_qi", "rho_qi", "qv2qi_depos_tend", "precip_total_tend", "nevapr",
                    "liq_ice_exchange", "vap_liq_exchange", "vap_ice_exchange"]
RHO_W = 1000.0
GRAV = 9.80616


def carry_host(state):
    """State hand-over of the process interface between steps
    (eamxx_p3_process_interface.hpp:218,237): qv_prev <- qv, t_prev <- T."""
    state["qv_prev"][...] = state["qv"]
    state["t_prev"][...] = state["th"] / state["inv_exner"]


def column_water(st):
    return ((st["qv"] + st["qc"] + st["qr"] + st["qi"]) * st["dpres"] / GRAV).sum(axis=1)


def cpu_baseline(inputs, steps=10, keep=None, warmup=0):
    """The CPU oracle (C++/OpenMP restatement of the reference p3_main) on the
    whole workload: `steps` steps of all columns with the state carried, on
    all host cores; `warmup` untimed steps first (on the same state, then the
    state restarts from the inputs).  Timed like the reference times p3_main
    (the column loop, init excluded).  With `keep`, also stores the state after
    step 1 and after the last step, the domain-total surface precipitation of
    every step, and the same run with th moved by one ulp (the oracle's own
    round-off spread)."""
    import numpy as np
    from scream_gb300 import _lib as L
    from oracle import p3_oracle as O
    tab = L.host_tables()
    cores = os.cpu_count() or 1
    ncol, nlev = inputs["qc"].shape

    def fresh(perturb=False):
        st = {k: np.array(v, copy=True) for k, v in inputs.items()}
        st.update(O.empty_outputs(ncol, nlev))
        if perturb:
            st["th"] = np.nextafter(st["th"], np.inf)
        return st

    if warmup:
        st = fresh()
        for s in range(warmup):
            O.p3_main(st, tab, DT, it=s + 1, nthreads=cores)
            carry_host(st)
        del st
    st = fresh()
    total_us, totals = 0.0, []
    for s in range(steps):
        err, us = O.p3_main(st, tab, DT, it=s + 1, nthreads=cores)
        if err:
            raise RuntimeError(f"oracle step {s + 1} returned error bits {err}")
        total_us += us
        totals.append(float(np.sum(st["precip_liq_surf"] + st["precip_ice_surf"])))
        if keep is not None and s == 0:
            keep["step1"] = {n: st[n].copy() for n in PRECISION_FIELDS}
        carry_host(st)
    value = ncol * nlev * steps / (total_us * 1e-6)
    if keep is not None:
        keep.update(oracle=st, oracle_totals=totals)
        pert = fresh(perturb=True)
        ptot = []
        for s in range(steps):
            O.p3_main(pert, tab, DT, it=s + 1, nthreads=cores)
            ptot.append(float(np.sum(pert["precip_liq_surf"] + pert["precip_ice_surf"])))
            carry_host(pert)
        keep.update(oracle_1ulp=pert, oracle_1ulp_totals=ptot)
    return {"value": value, "unit": "column-levels/s", "cores": cores, "kind": "port",
            "sample": f"the whole workload: {ncol} columns x {nlev} levels (RH ~ U(0.9, 1.05) in even columns), "
                      f"{steps} steps with the state carried" + (f" after {warmup} untimed steps" if warmup else "")
                      + f"; oracle p3_main (scalar FP64 C++ restatement of the reference, -O2) with OpenMP "
                        f"over columns on {cores} threads; elapsed time of the column loops"}


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    from scream_gb300.p3 import generate_inputs
    ncol = args.ncol or NCOL
    inputs = generate_inputs(1, rank_seed(0), ncol, NLEV)
    cb = cpu_baseline(inputs, steps=args.steps, warmup=args.warmup)
    line = {"metric": METRIC, "value": cb["value"], "unit": "column-levels/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ncol * NLEV / cb["value"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": DATA, "config": workload_config(ncol),
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "column-levels/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def _errors(g, ref):
    import numpy as np
    rows = {}
    for n in PRECISION_FIELDS:
        den = float(np.linalg.norm(ref[n]))
        d = g[n] - ref[n]
        num = float(np.linalg.norm(d))
        rows[n] = {"rel_l2": num / den if den > 0 else num, "max_abs": float(np.max(np.abs(d)))}
    tot_g = g["precip_liq_surf"] + g["precip_ice_surf"]
    tot_r = ref["precip_liq_surf"] + ref["precip_ice_surf"]
    rows["surface_precip_total"] = {"rel_l2": float(np.linalg.norm(tot_g - tot_r) / np.linalg.norm(tot_r)),
                                    "max_abs": float(np.max(np.abs(tot_g - tot_r)))}
    return rows


def precision_report(ctx, inputs, sample, steps=10):
    """Per-field rel-L2 and max-abs error of both GPU forms against the FP64
    oracle over the whole workload, after one step and after `steps` steps
    (the oracle run the CPU baseline just timed), with two well-conditioned
    aggregates: the domain-total surface precipitation of every step, and
    every column's water budget over all steps (W_end + precipitated mass =
    W_0).  The oracle's own run with th moved by one ulp is the round-off
    spread: P3's ice fields respond at ~1e-2 to 1-ulp input changes, so
    multi-step per-field figures measure the problem's conditioning."""
    import numpy as np
    import scream_gb300 as p3
    ncol, nlev = inputs["qc"].shape
    w0 = column_water(inputs)
    ref, ref1 = sample["oracle"], sample["step1"]
    o_tot = sample["oracle_totals"]
    out = {"workload": f"all {ncol} columns x {nlev} levels, {steps} steps, state carried "
                       "(qv_prev <- qv, t_prev <- T between steps), RH-stress inputs",
           "note": "oracle_1ulp: the oracle itself with th moved by one ulp (round-off spread)",
           "step1": {}, f"step{steps}": {}, "domain_total_precip_rel_diff": {},
           "column_water_residual_max": {}}
    for prec, tag in ((p3.P3X_FP32_BULK, "fp32_bulk"), (p3.P3X_FP64, "fp64")):
        f = p3.P3Fields.from_inputs(inputs)
        acc = np.zeros(ncol)
        rel_tot = []
        for s in range(steps):
            ctx.p3_main(f, DT, prec, it=s + 1)
            pl = f.t["precip_liq_surf"].cpu().numpy()
            pi = f.t["precip_ice_surf"].cpu().numpy()
            acc += (pl + pi) * RHO_W * DT
            rel_tot.append(abs(float(np.sum(pl + pi)) - o_tot[s]) / o_tot[s])
            if s == 0:
                out["step1"][tag] = _errors({n: f.t[n].cpu().numpy() for n in PRECISION_FIELDS}, ref1)
            f.t["qv_prev"].copy_(f.t["qv"])
            f.t["t_prev"].copy_(f.t["th"] / f.t["inv_exner"])
        g = {n: f.t[n].cpu().numpy() for n in PRECISION_FIELDS + ["dpres"]}
        out[f"step{steps}"][tag] = _errors(g, ref)
        out["domain_total_precip_rel_diff"][tag] = rel_tot
        out["column_water_residual_max"][tag] = float(np.max(np.abs(column_water(g) + acc - w0) / w0))
        del f, g
    out[f"step{steps}"]["oracle_1ulp"] = _errors(sample["oracle_1ulp"], ref)
    out["domain_total_precip_rel_diff"]["oracle_1ulp"] = [abs(a - b) / b for a, b in
                                                          zip(sample["oracle_1ulp_totals"], o_tot)]
    return out


def run_batched(ctx, args):
    """Batched form: 256 instances in one persistent launch sequence under a
    captured CUDA graph, launch configuration from the autotuner; FP64 and
    FP32-bulk."""
    import numpy as np
    import torch
    import scream_gb300 as p3

    rng = np.random.default_rng(4000)
    n = args.batch_instances
    ncols = np.floor(np.exp(rng.uniform(0, np.log(16385), n))).astype(int).clip(1, 16384)
    nlevs = np.where(rng.random(n) < 0.5, 72, 128)
    dts = np.where(rng.random(n) < 0.5, 300.0, 120.0)
    inputs = [p3.generate_inputs(0, 4000 + j, int(ncols[j]), int(nlevs[j])) for j in range(n)]
    cl = float(np.sum(ncols * nlevs))
    out = {"instances": n, "columns": int(ncols.sum()), "column_levels_per_step": cl}
    stream = torch.cuda.Stream()
    for prec, tag in ((p3.P3X_FP64, "fp64"), (p3.P3X_FP32_BULK, "fp32_bulk")):
        fields = [p3.P3Fields.from_inputs(x) for x in inputs]
        batch = p3.P3Batch(ctx, fields, dts, prec)
        with torch.cuda.stream(stream):
            best, ms_best = batch.autotune(reps=1, stream=stream)  # keeps the fastest configuration
            batch.capture_graph(stream)
            for _ in range(args.warmup):
                batch.run(stream)
            stream.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            steps = max(3, args.steps // 2)
            e0.record(stream)
            for _ in range(steps):
                batch.run(stream)
            e1.record(stream)
            e1.synchronize()
        ctx.check()
        ms = e0.elapsed_time(e1) / steps
        out[tag] = {"value": cl / (ms * 1e-3), "unit": "column-levels/s", "ms_per_step": ms,
                    "graph": True, "autotuned": best, "autotune_best_ms": ms_best}
        batch.close()
        del fields
        torch.cuda.empty_cache()
    out["fp32_bulk_speedup"] = out["fp32_bulk"]["value"] / out["fp64"]["value"]
    return out


def run_serving(ctx, args):
    """Request loop at 80% of the capacity measured here: capacity = sessions
    per second completed when every session arrives at once.  Requests carry
    data (first-step state upload, every step's result download, both inside
    the latency).  Isolated service times are calibrated first, so the tail
    is also reported as slowdown (latency over the request's own isolated
    time) and per size class."""
    import scream_gb300 as p3

    srv = p3.P3Server(ctx, budget_bytes=120 * 10**9, max_inflight=4)
    try:
        srv.calibrate()
        iso = {f"{'fp64' if prec == 0 else 'fp32_bulk'}_nlev{nl}_ncol{n}": srv.isolated_ms(prec, nl, n)
               for prec in (0, 1) for nl in (72, 128) for n in (1, 4096, 65536)}
        # the throughput policy first, reported beside the default (latency) one
        srv.set_latency_policy(False)
        sat_t = srv.run_poisson(rate_hz=1e6, n_sessions=args.serve_sessions, max_ncol=65536, seed=41)
        cap_t = args.serve_sessions / sat_t["wall_s"]
        st_t = srv.run_poisson(rate_hz=args.serve_load * cap_t, n_sessions=args.serve_sessions, max_ncol=65536,
                               seed=42)
        srv.set_latency_policy(True)
        sat = srv.run_poisson(rate_hz=1e6, n_sessions=args.serve_sessions, max_ncol=65536, seed=41)
        cap_hz = args.serve_sessions / sat["wall_s"]
        rate = args.serve_load * cap_hz
        st = srv.run_poisson(rate_hz=rate, n_sessions=args.serve_sessions, max_ncol=65536, seed=42)
    finally:
        srv.close()
    keys = ("p50_ms", "p90_ms", "p99_ms", "max_ms", "slowdown_p50", "slowdown_p99", "column_levels_per_s",
            "by_size_class")
    throughput_policy = {"capacity_column_levels_per_s": sat_t["column_levels_per_s"],
                         **{k: st_t[k] for k in keys}}
    return {"load": args.serve_load, "capacity_sessions_per_s": cap_hz, "rate_sessions_per_s": rate,
            "capacity_column_levels_per_s": sat["column_levels_per_s"], "budget_bytes": 120 * 10**9,
            "max_inflight": 4, **{k: st[k] for k in ("completed", "rejected", "p50_ms", "p90_ms", "p99_ms",
                                                      "max_ms", "mean_ms", "wall_s", "column_levels_per_s",
                                                      "peak_bytes", "peak_inflight", "slowdown_p50",
                                                      "slowdown_p99", "by_size_class", "h2d_bytes",
                                                      "d2h_bytes")},
            "p99_over_p50": st["p99_ms"] / st["p50_ms"] if st["p50_ms"] > 0 else None,
            "isolated_ms": iso,
            "policy": "latency (small requests on their own dispatches and reserved slot, large steps at 87.5 % of "
                      "the resident-block capacity); both policies launch dispatches in chunks of 2^18 "
                      "column-levels",
            "throughput_policy": throughput_policy,
            "data": "every request carries data: a session's first step uploads its 23 input fields from "
                    "page-locked host memory, every step downloads 10 prognostic fields + 2 surface rates; "
                    "both inside the latency"}


def run_gpu(args):
    import numpy as np
    import torch
    import scream_gb300 as p3
    from scream_gb300 import _lib as L

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    ncol = args.ncol or NCOL
    ctx = p3.P3Context()
    inputs = p3.generate_inputs(1, rank_seed(rank), ncol, NLEV)
    stream = torch.cuda.current_stream()

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    def timed_device(precision, steps, warmup):
        """K timed steps (events on the launching stream), then two untimed
        steps with per-kernel events for the kernel shares."""
        f = p3.P3Fields.from_inputs(inputs)
        for s in range(warmup):
            ctx.p3_main(f, DT, precision, it=s + 1, sync=False)
        ctx.check()
        barrier()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        t0 = time.perf_counter()
        for s in range(steps):
            ev[s][0].record(stream)
            ctx.p3_main(f, DT, precision, it=warmup + s + 1, sync=False)
            ev[s][1].record(stream)
        barrier()
        wall = time.perf_counter() - t0
        ctx.check()
        kms = [a.elapsed_time(b) for a, b in ev]
        ctx.set_kernel_timing(True)
        parts = []
        for s in range(2):
            ctx.p3_main(f, DT, precision, it=warmup + steps + s + 1, sync=False)
            parts.append(ctx.kernel_times())
        ctx.set_kernel_timing(False)
        ctx.check()
        del f
        torch.cuda.empty_cache()
        return wall, kms, [sum(p[i] for p in parts) / len(parts) for i in range(3)]

    # FP64 plain form (reported beside the headline)
    wall64, k64, parts64 = timed_device(L.P3X_FP64, args.steps, args.warmup)
    # FP32-bulk headline, with clocks sampled during the timed region
    with ClockSampler(local) as clk:
        wall32, k32, parts32 = timed_device(L.P3X_FP32_BULK, args.steps, args.warmup)
    clocks = clk.summary()

    maxr = reduce_max
    wall32 = maxr(wall32)
    wall64 = maxr(wall64)
    cl_step = ncol * NLEV
    value = weak_value(ws, cl_step, args.steps, wall32)
    value64 = weak_value(ws, cl_step, args.steps, wall64)

    # e2e: pinned host buffers through the public API
    h2d_fields = L.INPUT_FIELDS
    d2h_fields = [n for n in L.ALL_FIELDS if n not in L.DIAG_IN_FIELDS]
    hf = p3.P3Fields.allocate_host(ncol, NLEV)
    for n in h2d_fields:
        hf.t[n].copy_(torch.from_numpy(np.ascontiguousarray(inputs[n])))
    h2d_bytes = sum(hf.t[n].numel() * 8 for n in h2d_fields)
    d2h_bytes = sum(hf.t[n].numel() * 8 for n in d2h_fields)

    def e2e_step(it):
        # host arrays in, host arrays out (state carried in host memory)
        ctx.p3_main_host(hf, DT, L.P3X_FP32_BULK, it=it)

    e2e_steps = max(2, min(args.steps, 5))
    for s in range(min(args.warmup, 2)):
        e2e_step(s + 1)
    barrier()
    t0 = time.perf_counter()
    for s in range(e2e_steps):
        e2e_step(s + 1)
    barrier()
    e2e_wall = maxr(time.perf_counter() - t0)
    ctx.check()
    e2e_value = weak_value(ws, cl_step, e2e_steps, e2e_wall)
    del hf
    torch.cuda.empty_cache()

    batched = run_batched(ctx, args) if not args.no_batched else None
    serving = run_serving(ctx, args) if not args.no_serving else None

    if rank != 0:
        return 0
    hbm_peak, peak_kind = _peaks()
    kmean32 = sum(k32) / len(k32) * 1e-3
    achieved = ALG_BYTES_PER_CL * cl_step / kmean32 / 1e9
    tpc = _traffic_per_cl("fp32")
    names32 = ["p3_part12_kernel", "p3_sed_bulk_kernel", "p3_part3_kernel"]
    names64 = ["p3_part12_kernel", "p3_sed_kernel", "p3_part3_kernel"]

    def shares(parts, names):
        tot = sum(parts)
        return {n: {"ms": p, "share": p / tot} for n, p in zip(names, parts)}

    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved / hbm_peak, "peak_source": peak_kind,
            "traffic": (tpc * cl_step if tpc is not None else None),
            "kernel": "P3 step <float>: p3_part12_kernel + p3_sed_bulk_kernel + p3_part3_kernel, one launch "
                      "sequence per step; achieved = 360 B/cl x cl / mean event-timed step",
            "alg_bytes_per_cl": ALG_BYTES_PER_CL,
            "kernels": shares(parts32, names32),
            "fp64_pipe": fp64_ceiling("fp32", cl_step, kmean32 * 1e3, (clocks or {}).get("sm_mhz"),
                                      torch.cuda.get_device_properties(0).multi_processor_count)}
    kmean64 = sum(k64) / len(k64) * 1e-3
    sample = {}
    cb = cpu_baseline(inputs, steps=10, keep=sample) if not args.no_cpu else None
    precision = precision_report(ctx, inputs, sample) if sample else None
    sample.clear()
    line = {
        "metric": METRIC,
        "value": value, "unit": "column-levels/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": wall32 / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32-bulk (f64 state/residuals/fluxes)",
        "data": DATA,
        "config": workload_config(ncol),
        "fp64": {"value": value64, "unit": "column-levels/s", "ms_per_step": wall64 / args.steps * 1e3,
                 "kernel_ms": kmean64 * 1e3,
                 "hbm_gbs_alg": ALG_BYTES_PER_CL * cl_step / kmean64 / 1e9,
                 "fp32_bulk_speedup": value / value64, "kernels": shares(parts64, names64)},
        "roofline": roof,
        "e2e": {"value": e2e_value, "unit": "column-levels/s", "h2d_bytes_per_step": h2d_bytes,
                "d2h_bytes_per_step": d2h_bytes, "steps": e2e_steps,
                "path": "pinned host arrays -> P3Context.p3_main_host (libp3x C ABI p3x_main_host: column "
                        "chunks through three device buffers, uploads/kernels/downloads overlapped) -> "
                        "pinned host arrays"},
        "gpu_launches": 3 * args.steps,
        "batched": batched,
        "serving": serving,
        "clocks": clocks,
        "cpu_baseline": cb,
        "precision": precision,
    }
    print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ncol", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--batch-instances", type=int, default=256)
    ap.add_argument("--serve-sessions", type=int, default=120)
    ap.add_argument("--serve-load", type=float, default=0.8)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
