#!/usr/bin/env python3
"""Throughput of the nlchains hot path on GB300: FP64 site-steps/s.

Workload (one GPU): the register-resident DNKG ensemble, N = 128 sites, 65536 copies, m = 1,
beta = 1, dt = 0.05, seeded random-phase initial state with energy density 0.5 in the lowest 8% of
modes; a bench *step* is one fused launch of kernel_batching = 100 Yoshida steps over the whole
ensemble plus one diagnostics sample (linear-mode energies + entropies), i.e. one iteration of the
reference's main loop.  Toda (alpha = 0.5) on the same shape is measured as a second line item.

  value   device-resident throughput: state already in HBM, CUDA events on the launching stream,
          L2 flushed (256 MiB write) before every timed step;
  e2e     through the C ABI job API with host buffers: every step uploads the ensemble from pinned
          host memory, advances, reads back the diagnostics and downloads the ensemble;
  roofline  the integrator kernel against the FP64 FMA rate measured in this run by the engine's
          own DFMA loop kernel (nlc_fp64_peak); flops per site-step = 70 (DNKG/dDNKG), 56 + 7 exp (Toda);
  cpu_baseline  the reference's CPU algorithm (the oracle port of DNKG_FPUT_Toda/cpu-implementation,
          one OpenMP thread per host core over copies) on a bounded sample.

`--impl reference` runs only the reference's CPU implementation (the oracle port; the reference
itself cannot be built in this image) on the same metric and prints its line.

Multi-GPU (torchrun): one process per GPU, each integrating its own shard of copies of the same
size (weak scaling); the only exchange is the reference's all_reduce of the N linear energies per
sample (results_entropy.cpp:13), done here on the host over torch.distributed.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(name="DNKG N=128 copies=65536 (register-resident tier)", model="DNKG", n=128, copies=65536,
                dt=0.05, params=dict(m=1.0, beta=1.0), batching=100, eps=0.5, fraction=0.08, include_zero=True)
TODA = dict(name="Toda N=128 copies=65536", model="Toda", n=128, copies=65536, dt=0.05,
            params=dict(alpha=0.5), batching=100, eps=0.5, fraction=0.08, include_zero=False)
FLOPS_PER_SITE_STEP = {"DNKG": 70, "dDNKG": 70, "FPUT": 91, "Toda": 56}
L2_FLUSH_BYTES = 256 << 20


def initial_state(w, copies, first_copy, seed=12345):
    from nlchains_gb300 import ic
    modes = ic.low_modes(w["n"], w["fraction"], include_zero=w["include_zero"])
    return ic.real_ensemble(w["n"], copies, w["eps"], modes, m=w["params"].get("m", 0.0), seed=seed,
                            first_copy=first_copy)


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (getattr(self, "out", "") or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    return rank, local, world


def allreduce(values, op="sum"):
    """Host-side all_reduce over torch.distributed (no-op with one process)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor(np.asarray(values, dtype=np.float64))
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return t.numpy()


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def measure_engine(w, steps, warmup, rank, world, local):
    import torch

    import nlchains_gb300 as nlc

    torch.cuda.set_device(local)
    nlc.lib()
    n, copies, b = w["n"], w["copies"], w["batching"]
    state = initial_state(w, copies, first_copy=rank * copies)
    model = nlc.Model(w["model"], n, copies, w["dt"], **w["params"])
    plan = nlc.Plan(model)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    dev = torch.from_numpy(state).cuda()
    lin = torch.zeros(n, dtype=torch.float64, device="cuda")
    ent = torch.zeros(2, dtype=torch.float64, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def one_step():
        plan.move(dev.data_ptr(), b, sp)
        plan.linenergies(dev.data_ptr(), lin.data_ptr(), ent.data_ptr(), sp)

    for _ in range(warmup):
        one_step()
    torch.cuda.synchronize()
    e_step = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    e_move = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    barrier()
    torch.cuda.synchronize()
    launches0 = nlc.kernel_launches()
    with Clocks(local) as clk:
        wall0 = time.perf_counter()
        for i in range(steps):
            flush.zero_()   # outside the events: the state (128 MiB) does not exceed L2 by itself
            e_step[i][0].record(stream)
            e_move[i][0].record(stream)
            plan.move(dev.data_ptr(), b, sp)
            e_move[i][1].record(stream)
            plan.linenergies(dev.data_ptr(), lin.data_ptr(), ent.data_ptr(), sp)
            e_step[i][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    launches = nlc.kernel_launches() - launches0
    barrier()
    step_ms = sum(a.elapsed_time(z) for a, z in e_step)
    move_ms = sum(a.elapsed_time(z) for a, z in e_move) / steps
    step_ms = float(allreduce([step_ms], "max")[0])
    site_steps = float(n) * copies * b * steps * world
    value = site_steps / (step_ms * 1e-3)
    lin_h = lin.cpu().numpy()
    # ensemble average over ranks: the reference's all_reduce of linenergies (equal shards)
    lin_all = allreduce(lin_h) / world
    shape = plan.shape()
    return dict(value=value, step_ms=step_ms / steps, move_ms=move_ms, wall_s=wall, launches=launches,
                clocks=clk.summary(), shape=shape, plan=plan, lin=lin_all, entropies=ent.cpu().numpy().tolist(),
                state_after=dev.cpu().numpy(), state_before=state)


def measure_e2e(w, steps, warmup, rank, local):
    import torch

    import nlchains_gb300 as nlc

    n, copies, b = w["n"], w["copies"], w["batching"]
    host_in = torch.empty((copies, n, 2), dtype=torch.float64, pin_memory=True).numpy()
    host_out = torch.empty((copies, n, 2), dtype=torch.float64, pin_memory=True).numpy()
    host_in[...] = initial_state(w, copies, first_copy=rank * copies)
    ctx = nlc.Context(local)
    job = ctx.job(nlc.Model(w["model"], n, copies, w["dt"], **w["params"]), b)

    def one_step():
        job.upload(host_in)
        job.advance(b)
        job.linenergies()
        job.download(host_out)

    for _ in range(warmup):
        one_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        one_step()
    t = float(allreduce([time.perf_counter() - t0], "max")[0])
    job.close()
    ctx.close()
    bi = host_in.nbytes
    bo = host_out.nbytes + (n + 2) * 8
    return dict(value=float(n) * copies * b * steps / t, h2d=bi, d2h=bo)


def cpu_baseline(w, target_s=10.0, threads=None, sample_copies=None, steps_per_call=None):
    """The reference CPU algorithm (oracle port, reference arithmetic) on a bounded sample."""
    import oracle as O
    threads = threads or os.cpu_count() or 1
    n, b = w["n"], w["batching"]
    copies = sample_copies or max(threads * 16, 256)
    state = initial_state(w, copies, first_copy=0)
    mdl = O.Model(w["model"], n, copies, w["dt"], order=O.ORDER_REFERENCE, **w["params"])
    t0 = time.perf_counter()
    O.advance(mdl, state, b, b, threads=threads)
    probe = time.perf_counter() - t0
    reps = steps_per_call or max(1, int(target_s / max(probe, 1e-3)))
    t0 = time.perf_counter()
    st = state
    for _ in range(reps):
        st = O.advance(mdl, st, b, b, threads=threads)
    t = time.perf_counter() - t0
    value = float(n) * copies * b * reps / t
    return {"value": value, "unit": "site-steps/s", "cores": threads, "kind": "port",
            "sample": f"{w['model']} n={n}, {copies} of the {w['copies']} copies, {reps} x {b} steps "
                      f"({t:.1f} s), oracle reference-order port, OpenMP over copies"}


def energy_drift(w, before, after):
    import oracle as O
    sel = slice(0, 2048)
    mdl = O.Model(w["model"], w["n"], 2048, w["dt"], **w["params"])
    e0 = O.energies(mdl, np.ascontiguousarray(before[sel]))
    e1 = O.energies(mdl, np.ascontiguousarray(after[sel]))
    return float(np.abs(e1 / e0 - 1).max())


def read_traffic(kernel_key):
    """DRAM bytes per launch from the committed ncu summary (profiles/traffic.tsv), or None."""
    path = os.path.join(ROOT, "profiles", "traffic.tsv")
    if not os.path.exists(path):
        return None
    for line in open(path):
        f = line.rstrip("\n").split("\t")
        if len(f) >= 2 and f[0] == kernel_key:
            try:
                return float(f[1])
            except ValueError:
                return None
    return None


def run_engine(args):
    rank, local, world = dist_setup()
    import nlchains_gb300 as nlc
    import torch
    torch.cuda.set_device(local)
    peak = nlc.fp64_peak_tflops(ms=300.0)
    w = WORKLOAD
    r = measure_engine(w, args.steps, args.warmup, rank, world, local)
    e2e = measure_e2e(w, max(2, args.steps // 2), 1, rank, local)
    toda = measure_engine(TODA, max(2, args.steps // 2), 2, rank, world, local)
    flops = FLOPS_PER_SITE_STEP[w["model"]] * w["n"] * w["copies"] * w["batching"]
    achieved = flops / (r["move_ms"] * 1e-3) / 1e12
    out = {
        "metric": "site-steps/s FP64",
        "value": r["value"],
        "unit": "site-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": r["step_ms"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded random-phase low-mode ensemble, reference -i layout)",
        "config": {"workload": w["name"], "model": w["model"], "chain_length": w["n"], "copies": w["copies"],
                   "dt": w["dt"], **w["params"], "kernel_batching": w["batching"],
                   "step": "one fused launch of 100 Yoshida steps + one linenergies/entropy sample",
                   "l2": "flushed (256 MiB write) before every timed step",
                   "integrator_shape": r["shape"]},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": read_traffic("real_move_dnkg_n128"),
                     "kernel": "real_move_kernel_t<DNKG, E, beta==1>",
                     "flops_per_site_step": FLOPS_PER_SITE_STEP[w["model"]],
                     "peak_source": "measured in this run: engine DFMA loop kernel (nlc_fp64_peak), FMA = 2 flops",
                     "kernel_ms": r["move_ms"]},
        "e2e": {"value": e2e["value"], "unit": "site-steps/s", "h2d_bytes_per_step": e2e["h2d"],
                "d2h_bytes_per_step": e2e["d2h"]},
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
        "energy_drift": energy_drift(w, r["state_before"], r["state_after"]) if rank == 0 else None,
        "toda": {"value": toda["value"], "unit": "site-steps/s", "workload": TODA["name"],
                 "roofline_frac": FLOPS_PER_SITE_STEP["Toda"] * TODA["n"] * TODA["copies"] * TODA["batching"] /
                 (toda["move_ms"] * 1e-3) / 1e12 / peak, "kernel_ms": toda["move_ms"],
                 "shape": toda["shape"]},
    }
    if rank == 0 and world == 1:
        out["cpu_baseline"] = cpu_baseline(w)
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    w = WORKLOAD
    threads = os.cpu_count() or 1
    copies = max(threads * 64, 1024)   # a bounded sample of the 65536 copies per step
    import oracle as O
    for _ in range(args.warmup):
        cpu_baseline(w, threads=threads, sample_copies=copies, steps_per_call=1)
    t0 = time.perf_counter()
    vals = [cpu_baseline(w, threads=threads, sample_copies=copies, steps_per_call=1)["value"] for _ in range(args.steps)]
    wall = time.perf_counter() - t0
    value = float(w["n"]) * copies * w["batching"] * args.steps / wall
    out = {
        "metric": "site-steps/s FP64", "value": value, "unit": "site-steps/s", "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded random-phase low-mode ensemble, reference -i layout)",
        "config": {"workload": w["name"], "model": w["model"], "chain_length": w["n"], "copies": w["copies"],
                   "dt": w["dt"], **w["params"], "kernel_batching": w["batching"],
                   "sample_copies_per_step": copies},
        "cpu_baseline": {"value": value, "unit": "site-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{copies} of the {w['copies']} copies x {w['batching']} steps per bench step; "
                                   "the reference CPU code (DNKG_FPUT_Toda/cpu-implementation) needs Boost, MPI, "
                                   "FFTW3 and Armadillo, absent here, so its oracle port runs, OpenMP over copies"},
        "e2e": {"value": value, "unit": "site-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "per_step_values": vals,
    }
    del O
    print(json.dumps(out), flush=True)


def run_profile_case(args):
    """Small case of the headline kernels for ncu captures: 16384 copies, 4 launches of 10 steps."""
    import torch

    import nlchains_gb300 as nlc
    w = dict(WORKLOAD, copies=16384)
    if args.profile == "toda":
        w = dict(TODA, copies=16384)
    state = initial_state(w, w["copies"], 0)
    plan = nlc.Plan(nlc.Model(w["model"], w["n"], w["copies"], w["dt"], flags=nlc.FLAG_NO_TUNE, **w["params"]))
    dev = torch.from_numpy(state).cuda()
    lin = torch.zeros(w["n"], dtype=torch.float64, device="cuda")
    ent = torch.zeros(2, dtype=torch.float64, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream
    for _ in range(4):
        plan.move(dev.data_ptr(), 10, sp)
        plan.linenergies(dev.data_ptr(), lin.data_ptr(), ent.data_ptr(), sp)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": w["name"].replace("65536", str(w["copies"])), "shape": plan.shape(),
                      "entropies": ent.cpu().numpy().tolist()}))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--profile", choices=["dnkg", "toda"], default=None,
                    help="run only a small case of the integrator + diagnostics (for ncu captures)")
    args = ap.parse_args()
    if args.profile:
        return run_profile_case(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
