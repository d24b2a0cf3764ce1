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

`--impl reference` runs only the reference's CPU implementation (the oracle port, bit-identical in its
strict build to the reference's own CPU program compiled from its sources, which exist only where the
reference is checked out) on the same metric and prints its line.  `plain_reference_gpu` times the
reference's own GPU kernels, compiled unmodified for sm_103a, on the same workloads.

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
FLOPS_PER_SITE_STEP = {"DNKG": 70, "dDNKG": 70, "FPUT": 91, "Toda": 56, "DNLS": 812}
# FP64 instructions the engine issues per site-step for these workloads (7 sub-steps, the drift
# merged across steps): DNKG / dDNKG with beta = 1: 5 per sub-step; FPUT with alpha = 0, beta = 1: 6;
# Toda with 2 alpha = 1: 12 (8 of them the table exp); DNLS at n = 1024, dt = 0.01: 47 per sub-step
# (the 17-operation phase rotation of an angle below 2^-4, the propagator's radius-7 real-space
# stencil in 30) plus the closing rotation of a 10-step launch.  Against the measured FMA issue rate
# they give the fraction of the FP64 pipe's issue rate the integrator sustains, whatever the
# operation mix.
FP64_OPS_PER_SITE_STEP = {"DNKG": 35, "dDNKG": 35, "FPUT": 42, "Toda": 84, "DNLS": 7 * 47 + 17 / 10}
# the other workloads of the reference's benchmark list, measured as secondary line items
OTHERS = [
    dict(name="FPUT-beta N=64 copies=1024 (small ensemble)", model="FPUT", n=64, copies=1024, dt=0.1,
         params=dict(alpha=0.0, beta=1.0), batching=100, eps=0.1, kmax=4, include_zero=False),
    dict(name="DNLS N=1024 copies=8192", model="DNLS", n=1024, copies=8192, dt=0.01, params=dict(beta=1.0),
         batching=10, eps=1.0, fraction=0.1, include_zero=True),
    dict(name="dDNKG N=256 copies=4096", model="dDNKG", n=256, copies=4096, dt=0.05, params=dict(beta=1.0),
         batching=100, eps=0.5, nmodes=20, include_zero=True),
]
L2_FLUSH_BYTES = 256 << 20


def masses(w):
    from nlchains_gb300 import ic
    return ic.masses_uniform(w["n"], seed=777) if w["model"] == "dDNKG" else None


def initial_state(w, copies, first_copy, seed=12345):
    from nlchains_gb300 import ic
    if w["model"] == "dDNKG":
        return ic.ddnkg_ensemble(masses(w), copies, w["eps"], w["nmodes"], seed=seed, first_copy=first_copy)
    modes = ic.low_modes(w["n"], w.get("fraction"), kmax=w.get("kmax"), include_zero=w["include_zero"])
    if w["model"] == "DNLS":
        psi = ic.dnls_ensemble(w["n"], copies, w["eps"], modes, seed=seed, first_copy=first_copy)
        return np.ascontiguousarray(psi).view(np.float64).reshape(copies, w["n"], 2)
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
    model = nlc.Model(w["model"], n, copies, w["dt"], masses=masses(w), **w["params"])
    plan = nlc.Plan(model)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    dev = torch.from_numpy(state).cuda()
    lin = torch.zeros(n, dtype=torch.float64, device="cuda")
    ent = torch.zeros(2, dtype=torch.float64, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    # per-chain energies before and after the run (nlc_energies): the drift of the integrator
    e_before = torch.zeros(copies, dtype=torch.float64, device="cuda")
    e_after = torch.zeros(copies, dtype=torch.float64, device="cuda")
    plan.energies(dev.data_ptr(), e_before.data_ptr(), sp)

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
    # ensemble average over ranks and its entropies: the reference's all_reduce of linenergies
    from nlchains_gb300 import shards
    lin_all, wt, inf = shards.sample(lin.cpu().numpy(), copies, copies * world, model.a0is0)
    shape = plan.shape()
    plan.energies(dev.data_ptr(), e_after.data_ptr(), sp)
    drift = float((e_after / e_before - 1).abs().max().item())
    return dict(value=value, step_ms=step_ms / steps, move_ms=move_ms, wall_s=wall, launches=launches, energy_drift=drift,
                clocks=clk.summary(), shape=shape, plan=plan, lin=lin_all, entropies=[wt, inf],
                state_after=dev.cpu().numpy(), state_before=state)


def measure_e2e(w, steps, warmup, rank, local):
    import torch

    import nlchains_gb300 as nlc

    n, copies, b = w["n"], w["copies"], w["batching"]
    host_in = torch.empty((copies, n, 2), dtype=torch.float64, pin_memory=True).numpy()
    host_out = torch.empty((copies, n, 2), dtype=torch.float64, pin_memory=True).numpy()
    host_in[...] = initial_state(w, copies, first_copy=rank * copies)
    host_out2 = torch.empty((copies, n, 2), dtype=torch.float64, pin_memory=True).numpy()
    ctx = nlc.Context(local)
    # two jobs, each on its own stream: step i + 1's upload runs during step i's integration and
    # step i's read-back during step i + 1's (every step still copies its input in and its state
    # and energies out); the integrations stay in sequence (Job.after), so that step i + 1's
    # persistent launch does not hold the SMs that step i's diagnostics wait for
    jobs = [ctx.job(nlc.Model(w["model"], n, copies, w["dt"], **w["params"]), b) for _ in range(2)]
    outs = [host_out, host_out2]

    def issue(i):
        job = jobs[i % 2]
        job.upload(host_in, wait=False)
        if i:
            job.after(jobs[(i - 1) % 2])
        job.advance(b)
        job.sample_async(0)

    def finish(i):
        job = jobs[i % 2]
        job.sample_wait(0)
        job.download(outs[i % 2])

    def run(count):
        issue(0)
        for i in range(count):
            if i + 1 < count:
                issue(i + 1)
            finish(i)

    run(max(warmup, 2))
    barrier()
    t0 = time.perf_counter()
    run(steps)
    t = float(allreduce([time.perf_counter() - t0], "max")[0])
    for job in jobs:
        job.close()
    ctx.close()
    bi = host_in.nbytes
    bo = host_out.nbytes + (n + 2) * 8
    return dict(value=float(n) * copies * b * steps / t, h2d=bi, d2h=bo)


SERVED_PARAMS = {"FPUT": (0.1, dict(alpha=0.0, beta=1.0)), "Toda": (0.05, dict(alpha=0.5)),
                 "DNKG": (0.05, dict(m=1.0, beta=1.0)), "dDNKG": (0.05, dict(beta=1.0)), "DNLS": (0.01, dict(beta=1.0))}
# the served mixed stream at its stated ranges, with few enough requests for a bench run of minutes
SERVED_FULL = dict(count=24, seed=2024, n_range=(32, 4096), copies_range=(64, 16384), steps_range=(1000, 100000),
                   mean_gap_ms=500.0)
# the smaller stream of earlier measurements (one hundredth of the work per request)
SERVED_SMALL = dict(count=48, seed=2024, n_range=(32, 1024), copies_range=(64, 4096), steps_range=(100, 2000),
                    mean_gap_ms=15.0)


def served_stream(count=48, seed=2024, n_range=(32, 1024), copies_range=(64, 4096), steps_range=(100, 2000),
                  batching=100, mean_gap_ms=15.0):
    """A seeded mixed request stream: model uniform over the five, chain length, copies and steps
    log-uniform over the given ranges (steps rounded to a multiple of kernel_batching), energy density
    U[0.1, 1], seeded random-phase low-mode initial states, Poisson arrivals."""
    from nlchains_gb300 import ic
    rng = np.random.default_rng(seed)
    names = ["FPUT", "Toda", "DNKG", "dDNKG", "DNLS"]
    reqs, t = [], 0.0
    for i in range(count):
        name = names[rng.integers(len(names))]
        n = int(round(np.exp(rng.uniform(*np.log(n_range)))))
        copies = int(round(np.exp(rng.uniform(*np.log(copies_range)))))
        steps = max(batching, int(round(np.exp(rng.uniform(*np.log(steps_range))) / batching)) * batching)
        eps = rng.uniform(0.1, 1.0)
        dt, params = SERVED_PARAMS[name]
        masses = ic.masses_uniform(n, seed=seed + i) if name == "dDNKG" else None
        if name == "DNLS":
            st = np.ascontiguousarray(ic.dnls_ensemble(n, copies, eps, ic.low_modes(n, 0.1), seed=seed + i))
            st = st.view(np.float64).reshape(copies, n, 2)
        elif name == "dDNKG":
            st = ic.ddnkg_ensemble(masses, copies, eps, max(1, n // 10), seed=seed + i)
        else:
            st = ic.real_ensemble(n, copies, eps, ic.low_modes(n, 0.1, include_zero=params.get("m", 0) > 0),
                                  m=params.get("m", 0.0), seed=seed + i)
        t += rng.exponential(mean_gap_ms)
        reqs.append(dict(name=name, n=n, copies=copies, steps=steps, b=batching, dt=dt, params=params,
                         masses=masses, state=st, arrival_ms=t))
    return reqs


def run_alone(nlc, ctx, model, r):
    """One request alone through the job API with the sampling of the reference's main loop (a sample
    every kernel_batching steps), pipelined as the command line runs it: each batch and its sample go
    out as one graph replay into one of two result slots while the host waits for the previous one,
    so the GPU never idles on a host round trip."""
    job = ctx.job(model, r["b"])
    t1 = time.perf_counter()
    job.upload(r["state"])
    rounds = r["steps"] // r["b"]
    job.sample_async(0)
    for i in range(rounds):
        job.step_async((i + 1) % 2)
        job.sample_wait(i % 2)
    job.sample_wait(rounds % 2)
    job.download()
    t = time.perf_counter() - t1
    job.close()
    return t


def measure_served(local, stream):
    """Continuous batching (nlc_server) against the same requests run alone, one after the other."""
    import nlchains_gb300 as nlc
    reqs = served_stream(**stream)
    site_steps = sum(float(r["n"]) * r["copies"] * r["steps"] for r in reqs)

    def model(r):
        return nlc.Model(r["name"], r["n"], r["copies"], r["dt"], masses=r["masses"], **r["params"])

    # warm the plans' code paths once
    srv = nlc.Server(local)
    w = reqs[0]
    srv.wait(srv.submit(model(w), w["b"], w["b"], w["state"]), 120000)
    srv.close()

    srv = nlc.Server(local)
    ids = []
    t0 = time.perf_counter()
    for r in reqs:
        delay = r["arrival_ms"] / 1e3 - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        ids.append(srv.submit(model(r), r["b"], r["steps"], r["state"]))
    lat, prep = [], []
    for rid in ids:
        srv.wait(rid, 1800000)
        st = srv.poll(rid)
        lat.append(st["finish_ms"] - st["submit_ms"])
        prep.append(st["ready_ms"] - st["submit_ms"])
        srv.result(rid)
    makespan = time.perf_counter() - t0
    srv.close()

    # the same requests alone, one at a time through the job API (the plain per-model path)
    ctx = nlc.Context(local)
    alone = [run_alone(nlc, ctx, model(r), r) for r in reqs]
    ctx.close()
    alone_s = sum(alone)
    slowdown = np.array(lat) / (np.array(alone) * 1e3)
    # the plain path as a queue: the same arrivals, each request run alone when the previous is done
    queue_lat, free_at = [], 0.0
    for r, al in zip(reqs, alone):
        start = max(r["arrival_ms"] / 1e3, free_at)
        free_at = start + al
        queue_lat.append((free_at - r["arrival_ms"] / 1e3) * 1e3)
    per_model = {}
    for r, lt, al in zip(reqs, lat, alone):
        m = per_model.setdefault(r["name"], {"requests": 0, "site_steps": 0.0, "alone_s": 0.0, "latency_ms": []})
        m["requests"] += 1
        m["site_steps"] += float(r["n"]) * r["copies"] * r["steps"]
        m["alone_s"] += al
        m["latency_ms"].append(lt)
    for m in per_model.values():
        m["p50_latency_ms"] = float(np.percentile(m.pop("latency_ms"), 50))
    return {"value": site_steps / makespan, "unit": "site-steps/s", "alone_value": site_steps / alone_s,
            "speedup_vs_alone": alone_s / makespan, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "slowdown_p50": float(np.percentile(slowdown, 50)),
            "slowdown_p99": float(np.percentile(slowdown, 99)),
            "alone_queue_p50_ms": float(np.percentile(queue_lat, 50)), "alone_queue_p99_ms": float(np.percentile(queue_lat, 99)),
            "alone_queue_makespan_s": free_at, "speedup_vs_alone_queue": free_at / makespan,
            "ready_p50_ms": float(np.percentile(prep, 50)), "ready_p99_ms": float(np.percentile(prep, 99)),
            "requests": len(reqs), "makespan_s": makespan,
            "alone_s": alone_s, "largest_request_alone_s": float(max(alone)), "per_model": per_model,
            "stream": f"{stream['count']} requests, model uniform over FPUT/Toda/DNKG/dDNKG/DNLS, N log-uniform "
                      f"{list(stream['n_range'])}, copies log-uniform {list(stream['copies_range'])}, steps log-uniform "
                      f"{list(stream['steps_range'])} (multiples of 100), kernel_batching 100 with a sample every batch, "
                      f"Poisson arrivals (mean gap {stream['mean_gap_ms']:g} ms), seed {stream['seed']}",
            "alone": "each request by itself through the job API, batch + sample replayed as one CUDA graph, "
                     "two result slots (no host round trip between batches)",
            "slowdown": "latency over the request's own alone time",
            "ready": "submit to prepared (plan, tables, eigensystem, upload)",
            "alone_queue": "latency percentiles and makespan of the plain path run as a first-come-first-served "
                           "queue on the same arrivals, from the measured alone times (both makespans run from the "
                           "stream's start, so both include the GPU's idle time before arrivals)"}


def measure_mixed_concurrency(local, full_rates, rounds=20):
    """Different models sharing the GPU: four small ensembles (DNKG, FPUT, Toda, dDNKG, each about
    a quarter of the GPU's resident chains) submitted to the request server together, which runs each
    model's class kernel on its own stream, against (a) the same four run one after the other and
    (b) the time their work takes at each model's full-GPU rate (`full_rates`, site-steps/s of this
    bench's full-size workloads).  occupancy = (b) / served makespan: 1.0 means the concurrent
    per-model launches keep the FP64 pipes as busy as one launch over all four would."""
    import nlchains_gb300 as nlc
    from nlchains_gb300 import ic
    cases = [("DNKG", 128, 4096, 0.05, dict(m=1.0, beta=1.0)), ("FPUT", 64, 8192, 0.1, dict(alpha=0.0, beta=1.0)),
             ("Toda", 128, 4096, 0.05, dict(alpha=0.5)), ("dDNKG", 256, 2048, 0.05, dict(beta=1.0))]
    b = 100
    reqs = []
    for i, (name, n, copies, dt, params) in enumerate(cases):
        masses = ic.masses_uniform(n, seed=777) if name == "dDNKG" else None
        if name == "dDNKG":
            st = ic.ddnkg_ensemble(masses, copies, 0.5, 20, seed=i)
        else:
            st = ic.real_ensemble(n, copies, 0.5, ic.low_modes(n, 0.08, include_zero=params.get("m", 0) > 0),
                                  m=params.get("m", 0.0), seed=i)
        reqs.append((nlc.Model(name, n, copies, dt, masses=masses, **params), st, float(n) * copies * b * rounds))

    def serve(subset):
        srv = nlc.Server(local)
        t0 = time.perf_counter()
        ids = [srv.submit(m, b, b * rounds, st) for m, st, _ in subset]
        for rid in ids:
            srv.wait(rid, 600000)
            srv.result(rid)
        t = time.perf_counter() - t0
        srv.close()
        return t

    serve(reqs[:1])   # warm-up
    together = serve(reqs)
    alone = sum(serve([r]) for r in reqs)
    ideal = sum(work / full_rates[m.name] for m, _, work in reqs)
    return {"ensembles": [f"{m.name} n={m.chain_length} copies={m.copies}" for m, _, _ in reqs],
            "steps_each": b * rounds, "served_together_s": together, "served_one_by_one_s": alone,
            "at_full_gpu_rates_s": ideal, "occupancy": ideal / together,
            "gain_over_one_by_one": alone / together}


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
                      f"({t:.1f} s), oracle port of the reference CPU loop, -Ofast like the reference's CPU build, OpenMP over copies"}


def measure_projection(w, local, evolve_steps=1000):
    """One diagnostics sample of the dDNKG workload (its initial state advanced by 1000 steps; at the
    initial state most modes hold rounding-level energy and the WT entropy, a sum of their logs, is
    ill-conditioned) with the mode projection on the FP64 CUDA cores, on the tensor cores (7 slices,
    the default) and as BF16x3 (3 slices): times, and the differences of the mode energies and of
    both entropies against the FP64 projection."""
    import torch

    import nlchains_gb300 as nlc
    n, copies = w["n"], w["copies"]
    dev = torch.from_numpy(initial_state(w, copies, 0)).cuda()
    sp = torch.cuda.current_stream().cuda_stream
    res = {}
    for name, flag in (("fp64", nlc.FLAG_FP64_PROJECTION), ("tensor", nlc.FLAG_TENSOR_PROJECTION),
                       ("bf16x3", nlc.FLAG_BF16X3_PROJECTION)):
        plan = nlc.Plan(nlc.Model(w["model"], n, copies, w["dt"], masses=masses(w), flags=flag, **w["params"]))
        if name == "fp64":
            plan.move(dev.data_ptr(), evolve_steps, sp)
        lin = torch.zeros(n, dtype=torch.float64, device="cuda")
        ent = torch.zeros(2, dtype=torch.float64, device="cuda")
        for _ in range(3):
            plan.linenergies(dev.data_ptr(), lin.data_ptr(), ent.data_ptr(), sp)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(20):
            plan.linenergies(dev.data_ptr(), lin.data_ptr(), ent.data_ptr(), sp)
        e1.record()
        torch.cuda.synchronize()
        res[name] = (e0.elapsed_time(e1) / 20, lin.cpu().numpy(), ent.cpu().numpy())
        plan.close()
    ref, eref = res["fp64"][1], res["fp64"][2]
    diff = float(np.abs(res["tensor"][1] - ref).max() / np.abs(ref).max())
    diff3 = float(np.abs(res["bf16x3"][1] - ref).max() / np.abs(ref).max())

    def ent_diffs(name):
        e = res[name][2]
        return {"wt_abs_diff": float(abs(e[0] - eref[0])), "inf_rel_diff": float(abs(e[1] - eref[1]) / abs(eref[1]))}

    return {"fp64_ms": res["fp64"][0], "tensor_ms": res["tensor"][0], "speedup": res["fp64"][0] / res["tensor"][0],
            "state": f"the workload's initial state after {evolve_steps} steps",
            "max_rel_diff": diff, "tensor_entropies": ent_diffs("tensor"), "bf16x3_ms": res["bf16x3"][0],
            "bf16x3_max_rel_diff": diff3, "bf16x3_entropies": ent_diffs("bf16x3"),
            "flops": 4.0 * copies * n * n,
            # the 28 BF16 slice products of the 7-slice form, over the whole sample (split, projection
            # and finish kernels), against the measured cuBLAS BF16 rate
            "bf16_tflops": 28 * 4.0 * copies * n * n / (res["tensor"][0] * 1e-3) / 1e12,
            "bf16_frac_of_measured_peak": 28 * 4.0 * copies * n * n / (res["tensor"][0] * 1e-3) / 1e12 / bf16_peak(),
            "method": "tcgen05 BF16 MMA (M = N = 128), 7-slice split of X and of the eigenvectors, FP32 accumulation "
                      "in TMEM read out every 256 sites, exact integer recombination, energy epilogue fused"}


def bf16_peak():
    """The measured burst BF16 rate of this GPU type (TFLOP/s), or the stated fallback."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"])
    except (OSError, KeyError, ValueError):
        return 1900.0


def measure_eigensystem(w, sizes=(1024, 2048)):
    """Set-up cost of the dDNKG eigensystem on this machine's host cores (nlc_eigensystem with no
    device: the divide-and-conquer solver plans use below 4096 sites), best of three wall-clock
    times at the workload's chain length and at the given ones.  A failure is reported, not raised."""
    try:
        import nlchains_gb300 as nlc
        from nlchains_gb300 import ic
        out = {"solver": "host divide and conquer (nlc_eigensystem, device -1)"}
        for n in sorted({w["n"], *sizes}):
            m = ic.masses_uniform(n, seed=777)
            best = float("inf")
            for _ in range(3):
                t0 = time.perf_counter()
                nlc.eigensystem(m, device=-1)
                best = min(best, time.perf_counter() - t0)
            out[f"ms_n{n}"] = best * 1e3
        out["host_threads"] = os.cpu_count()
        return out
    except Exception as e:   # the set-up figure is informational
        return {"error": f"{type(e).__name__}: {e}"}


def measure_fp32_diagnostics(w, local, evolve_steps=1000):
    """One diagnostics sample of the DNLS workload (its initial state advanced by 1000 steps, so that
    energy has spread beyond the initial modes) with the FP64 transform and with
    NLC_FLAG_FP32_DIAGNOSTICS: times, and the FP32 path's error against FP64 for the mode energies
    (largest difference over the largest energy) and both entropies."""
    import torch

    import nlchains_gb300 as nlc
    n, copies = w["n"], w["copies"]
    dev = torch.from_numpy(initial_state(w, copies, 0)).cuda()
    sp = torch.cuda.current_stream().cuda_stream
    plans = {name: nlc.Plan(nlc.Model(w["model"], n, copies, w["dt"], flags=flag, **w["params"]))
             for name, flag in (("fp64", 0), ("fp32", nlc.FLAG_FP32_DIAGNOSTICS))}
    plans["fp64"].move(dev.data_ptr(), evolve_steps, sp)
    res = {}
    for name, plan in plans.items():
        lin = torch.zeros(n, dtype=torch.float64, device="cuda")
        ent = torch.zeros(2, dtype=torch.float64, device="cuda")
        for _ in range(3):
            plan.linenergies(dev.data_ptr(), lin.data_ptr(), ent.data_ptr(), sp)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(20):
            plan.linenergies(dev.data_ptr(), lin.data_ptr(), ent.data_ptr(), sp)
        e1.record()
        torch.cuda.synchronize()
        res[name] = (e0.elapsed_time(e1) / 20, lin.cpu().numpy(), ent.cpu().numpy())
        plan.close()
    (t64, l64, s64), (t32, l32, s32) = res["fp64"], res["fp32"]
    return {"state": f"the workload's initial state after {evolve_steps} steps", "fp64_ms": t64, "fp32_ms": t32,
            "speedup": t64 / t32, "energies_max_diff_over_max": float(np.abs(l32 - l64).max() / np.abs(l64).max()),
            "wt_abs_diff": float(abs(s32[0] - s64[0])), "inf_rel_diff": float(abs(s32[1] - s64[1]) / abs(s64[1])),
            "method": "per-chain FFT and mode energies in FP32, sum over chains in FP64"}


def measure_reference_gpu(local, engine_kernel_ms, launches=3):
    """The plain reference GPU path on this GB300: the reference's own integration kernels
    (move_chain_in_warp<model>, dDNKG::move_chain_in_warp, and DNLS's evolve_* kernels with cuFFT),
    compiled unmodified for sm_103a from its sources (oracle/_ref/ref_gpu_n<N>.fatbin), on each
    workload's full ensemble; `launches` launches of kernel_batching steps timed with CUDA events on
    the launching stream after one warm-up launch.  The reference's per-process copy count is 16-bit
    (common/configuration.hpp:24), so 65536 copies run as two launches of 32768, as two of its MPI
    ranks would.  engine_kernel_ms: the engine's integrator time per launch of the same workload."""
    import torch

    import oracle as O
    out = {}
    for w in (WORKLOAD, TODA, OTHERS[0], OTHERS[2], OTHERS[1]):
        key = w["model"]
        n_opt = 64 if w["model"] == "DNLS" else w["n"]
        if not O.RefGPU.available(n_opt):
            out[key] = {"unavailable": f"oracle/_ref/ref_gpu_n{n_opt}.fatbin was not built from the reference's sources"}
            continue
        n, copies, b = w["n"], w["copies"], w["batching"]
        ref = O.RefGPU(n_opt)
        state = torch.from_numpy(initial_state(w, copies, 0)).cuda()
        stream = torch.cuda.current_stream()
        sp = stream.cuda_stream
        chunk = 32768
        parts = [(c0, min(chunk, copies - c0)) for c0 in range(0, copies, chunk)]
        mp2 = None
        if w["model"] == "dDNKG":
            mp2 = torch.from_numpy(masses(w) + 2).cuda()
        mdl0 = O.Model(w["model"], n, parts[0][1], w["dt"], masses=masses(w), **w["params"])

        def launch_all():
            for c0, cn in parts:
                ptr = state.data_ptr() + c0 * n * 16
                if w["model"] == "DNLS":
                    ref.dnls_advance(O.Model("DNLS", n, cn, w["dt"], **w["params"]), ptr, b, b, sp, sync=False)
                else:
                    ref.move_warp_async(mdl0.model, ptr, n, cn, b, 1, mp2.data_ptr() if mp2 is not None else None, sp)

        if w["model"] != "DNLS":
            ref.advance(mdl0, state.data_ptr(), 0, b, stream=sp)   # the constants, no steps
        launch_all()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(launches):
            launch_all()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / launches
        ref.close()
        eng_ms = engine_kernel_ms.get(key)
        out[key] = {"workload": w["name"], "value": float(n) * copies * b / (ms * 1e-3), "unit": "site-steps/s",
                    "kernel_ms_per_launch": ms, "steps_per_launch": b,
                    "launches_per_step": len(parts) * (14 * b + b + 1 if w["model"] == "DNLS" else 1),
                    "kernel": ("DNLS evolve_nonlinear/evolve_linear + cuFFT Z2Z (no callbacks)" if w["model"] == "DNLS"
                               else ("dDNKG::" if w["model"] == "dDNKG" else "DNKG_FPUT_Toda::") +
                               f"move_chain_in_warp, optimized_chain_length={n}"),
                    "engine_kernel_ms_per_launch": eng_ms, "engine_speedup": (ms / eng_ms) if eng_ms else None}
    return out


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
    e2e = measure_e2e(w, max(4, args.steps), 2, rank, local)
    toda = measure_engine(TODA, max(2, args.steps // 2), 2, rank, world, local)
    others = {}
    for ow in OTHERS:
        o = measure_engine(ow, max(3, args.steps // 2), 3, rank, world, local)
        others[ow["model"]] = {"workload": ow["name"], "value": o["value"], "unit": "site-steps/s",
                               "ms_per_step": o["step_ms"], "kernel_ms": o["move_ms"],
                               "steps_per_launch": ow["batching"], "shape": o["shape"],
                               "fp64_frac_of_peak": FLOPS_PER_SITE_STEP[ow["model"]] * ow["n"] * ow["copies"] *
                               ow["batching"] / (o["move_ms"] * 1e-3) / 1e12 / peak,
                               "fp64_issue_frac": FP64_OPS_PER_SITE_STEP[ow["model"]] * ow["n"] * ow["copies"] *
                               ow["batching"] / (o["move_ms"] * 1e-3) / (peak * 1e12 / 2)}
        if ow["model"] == "dDNKG" and rank == 0:
            others["dDNKG"]["projection"] = measure_projection(ow, local)
            others["dDNKG"]["projection_n1024"] = measure_projection(
                dict(ow, name="dDNKG N=1024 copies=4096", n=1024, nmodes=80), local)
            others["dDNKG"]["eigensystem_setup"] = measure_eigensystem(ow)
        if ow["model"] == "DNLS" and rank == 0:
            others["DNLS"]["fp32_diagnostics"] = measure_fp32_diagnostics(ow, local)
            others["DNLS"]["note"] = ("fp64_frac_of_peak counts the reference algorithm's 812 flops per site-step "
                                      "(radix-2 transforms); the engine applies the same propagator as a real-space "
                                      "stencil in 331 FP64 operations per site-step, so that ratio can pass 1; "
                                      "fp64_issue_frac is the FP64 pipe's measure")
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
        "energy_drift": r["energy_drift"] if rank == 0 else None,
        "toda": {"value": toda["value"], "unit": "site-steps/s", "workload": TODA["name"],
                 # one figure: the FP64 operations the integrator issues per site-step (84: 12 per
                 # sub-step, 8 of them the table exp) against the measured FMA issue rate
                 "roofline": {"bound": "fp64", "ops_per_site_step": FP64_OPS_PER_SITE_STEP["Toda"],
                              "frac": FP64_OPS_PER_SITE_STEP["Toda"] * TODA["n"] * TODA["copies"] * TODA["batching"] /
                              (toda["move_ms"] * 1e-3) / (peak * 1e12 / 2),
                              "note": "the reference algorithm's count without its 7 exp (56 flops) would read "
                                      "as a third of this; every exp costs 8 FP64 operations here"},
                 "kernel_ms": toda["move_ms"], "shape": toda["shape"]},
        "other_workloads": others,
    }
    if rank == 0:
        out["plain_reference_gpu"] = measure_reference_gpu(
            local, {"DNKG": r["move_ms"], "Toda": toda["move_ms"],
                    **{k: v["kernel_ms"] for k, v in others.items()}})
    if world == 1:
        out["served"] = measure_served(local, SERVED_FULL)
        out["served_small"] = measure_served(local, SERVED_SMALL)
        out["mixed_models"] = measure_mixed_concurrency(
            local, {"DNKG": r["value"], "Toda": toda["value"], "FPUT": others["FPUT"]["value"],
                    "dDNKG": others["dDNKG"]["value"]})
    if rank == 0 and world == 1:
        out["cpu_baseline"] = cpu_baseline(w)
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    import oracle as O
    w = WORKLOAD
    n, b = w["n"], w["batching"]
    threads = os.cpu_count() or 1
    copies = max(threads * 256, 1024)   # a bounded sample of the 65536 copies per step
    mdl = O.Model(w["model"], n, copies, w["dt"], order=O.ORDER_REFERENCE, **w["params"])
    st = initial_state(w, copies, first_copy=0)
    for _ in range(args.warmup):
        st = O.advance(mdl, st, b, b, threads=threads)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):   # one step: kernel_batching steps of the sample, as one reference launch
        t1 = time.perf_counter()
        st = O.advance(mdl, st, b, b, threads=threads)
        vals.append(float(n) * copies * b / (time.perf_counter() - t1))
    wall = time.perf_counter() - t0
    value = float(n) * copies * b * args.steps / wall
    out = {
        "metric": "site-steps/s FP64", "value": value, "unit": "site-steps/s", "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded random-phase low-mode ensemble, reference -i layout)",
        "config": {"workload": w["name"], "model": w["model"], "chain_length": w["n"], "copies": w["copies"],
                   "dt": w["dt"], **w["params"], "kernel_batching": w["batching"],
                   "sample_copies_per_step": copies},
        "cpu_baseline": {"value": value, "unit": "site-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{copies} of the {w['copies']} copies x {w['batching']} steps per bench step "
                                   "(a bounded sample of the workload, not all 65536 copies); the oracle port of the "
                                   "reference's CPU loop (DNKG_FPUT_Toda/cpu-implementation), whose strict build "
                                   "reproduces the reference's own CPU program bit for bit (tests/test_reference_pin.py), "
                                   "here built -Ofast like the reference's CPU code, OpenMP over copies; the reference's "
                                   "program itself is built from its sources only where they are, not on this host"},
        "e2e": {"value": value, "unit": "site-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "per_step_values": vals,
    }
    print(json.dumps(out), flush=True)


def run_reference_profile_case():
    """The reference's own DNKG warp kernel (move_chain_in_warp<DNKG>, compiled unmodified for sm_103a)
    on the small DNKG profile case: 16384 of the 65536 copies, 4 launches of 10 steps."""
    import torch

    import oracle as O
    w = dict(WORKLOAD, copies=16384)
    if not O.RefGPU.available(w["n"]):
        print(json.dumps({"profile_case": "reference", "unavailable": "no reference fatbin"}))
        return
    ref = O.RefGPU(w["n"])
    state = torch.from_numpy(initial_state(w, w["copies"], 0)).cuda()
    mdl = O.Model(w["model"], w["n"], w["copies"], w["dt"], **w["params"])
    ref.advance(mdl, state.data_ptr(), 0, 10)   # the constants
    sp = torch.cuda.current_stream().cuda_stream
    for _ in range(4):
        ref.move_warp_async(mdl.model, state.data_ptr(), w["n"], w["copies"], 10, 1, None, sp)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": "reference move_chain_in_warp<DNKG> N=128 copies=16384",
                      "state_norm": float(state.norm().item())}))
    ref.close()


def run_profile_case(args):
    """Small cases of the headline kernels for ncu captures: 4 launches (10 steps; DNLS 2 steps),
    each followed by one diagnostics sample.  DNKG / Toda: 16384 of the 65536 copies (33.5 MB);
    DNLS: the full 8192 copies of N = 1024 (134 MB, above the L2); dnlslong: 512 DNLS chains of 16384
    sites in windows (6 steps: two launches of 3); dDNKG: the full 4096 x 256;
    long: 256 FPUT chains of 65535 sites (windowed tier, 268 MB)."""
    import torch

    import nlchains_gb300 as nlc
    w, steps = dict(WORKLOAD, copies=16384), 10
    if args.profile == "toda":
        w = dict(TODA, copies=16384)
    if args.profile == "dnls":
        w, steps = dict(OTHERS[1]), 2
    if args.profile == "dnlslong":   # DNLS beyond one block: the stencil form in windows (134 MB of state)
        w, steps = dict(OTHERS[1], name="DNLS N=16384 copies=512 (windowed)", n=16384, copies=512), 6
    if args.profile == "ddnkg":   # the full dDNKG workload: 4096 chains of 256 sites, tensor-core projection
        w = dict(OTHERS[2])
    if args.profile == "ddnkg1024":   # 4096 chains of 1024 sites: four read-outs per projection tile
        w, steps = dict(OTHERS[2], name="dDNKG N=1024 copies=4096", n=1024, nmodes=80), 2
    if args.profile == "long":    # chains beyond one block: the windowed tier (268 MB of state)
        w = dict(name="FPUT-beta N=65535 copies=256 (windowed tier)", model="FPUT", n=65535, copies=256, dt=0.1,
                 params=dict(alpha=0.0, beta=1.0), batching=10, eps=0.1, kmax=4, include_zero=False)
    state = initial_state(w, w["copies"], 0)
    plan = nlc.Plan(nlc.Model(w["model"], w["n"], w["copies"], w["dt"], masses=masses(w), flags=nlc.FLAG_NO_TUNE,
                              **w["params"]))
    dev = torch.from_numpy(state).cuda()
    lin = torch.zeros(w["n"], dtype=torch.float64, device="cuda")
    ent = torch.zeros(2, dtype=torch.float64, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream
    for _ in range(4):
        plan.move(dev.data_ptr(), steps, sp)
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
    ap.add_argument("--profile", choices=["dnkg", "toda", "dnls", "dnlslong", "ddnkg", "ddnkg1024", "long", "refdnkg"],
                    default=None,
                    help="run only a small case of the integrator + diagnostics (for ncu captures)")
    args = ap.parse_args()
    if args.profile == "refdnkg":
        return run_reference_profile_case()
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
