"""Benchmark of the hydro flux path on one GB300.

Headline workload (the reference benchmark configuration that fits one GPU): 3D Kelvin-Helmholtz,
256^3 periodic unit box as 64 meshblocks of 64^3 with 4 ghost cells, PPM + HLLC, RK2,
CFL 0.3, gamma 5/3, FP64, synthetic initial data.  A "step" is one full RK2 step of the
whole pack (2 stages + the CFL dt reduction).

Arithmetic mode (--mode): exact (the default) computes the reference's FP64 operations in the
reference's order with one rounding each and is bit-identical to the oracle, so it carries
the parity claim; fast (fused multiply-adds, shared reciprocals, constant adiabatic indices)
is timed beside it as other_mode and is not parity-carrying (the reference's PPM limiter
switches branches on its one-ulp differences).

value   zone-updates/s of the batched path (one persistent launch per stage over all 64
        meshblocks, the step replayed as a CUDA graph), state resident in HBM.
e2e     the same through the C ABI with the state in pinned host memory as the packed
        interiors (aph_stepper_load_interiors / _store_interiors, one kernel each way across
        the host link): every step loads its input from the host, steps, and stores its
        result back to the host.
plain   the per-meshblock launch path (one launch per kernel per meshblock).
roofline  HBM roofline of the stage kernel with the algorithmic 200 B per zone-update
        (stage 1: read U^n, write U^1; stage 2: read U^1 and U^n, write U^n+1), and the
        FP64-pipe roofline that actually binds it.
cpu_baseline  the oracle (C++ FP64 restatement of the reference's CPU path) on the host
        cores, a bounded sample of the same workload.

amr     the uneven refined pack (2D Rayleigh-Taylor, 256 x 768 base grid, two static levels:
        1440 meshblocks of 32^2 and 16^2, PPM+HLLC, RK2, gravity): the batched stepper
        against the plain per-pack and per-meshblock launch paths (the latter host-driven,
        and replayed from a CUDA graph as its best case).
ensemble the batched blast ensemble (64 independent 2D blast problems, grids from
        {128..512}^2 in 64^2 blocks, gamma ~ U[1.4, 5/3], PPM+HLLC, RK2) run to t = 0.1 in one
        stepper (one persistent launch per stage over all 1814 blocks, each member with its own
        gamma, CFL dt and clock; finished members are skipped); zone-updates/s counts every
        member's own steps.
adjoint the adjoint/forward time ratio on the differentiable rollout (2D KH 512^2 as 64
        blocks of 64^2, PLM+HLLE, RK2, checkpoint every 20 steps): reverse sweep (with
        recomputation) per step over the batched forward step.

--impl reference times that CPU path alone (all host threads) on the same workload.
Under torchrun (N > 1) every rank runs its own replica of the workload (the hydro step
shards by meshblocks, but this build drives one GPU per replica and exchanges nothing);
the step time is the max over ranks.
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "zone-updates/s (PPM+HLLC, FP64) batched vs plain; adjoint/forward time ratio"
UNIT = "zone-updates/s"
WORKLOAD = ("kh3d 256^3: 64 meshblocks of 64^3, 4 ghost cells, PPM+HLLC, RK2, CFL 0.3, "
            "gamma 5/3, FP64")
BYTES_PER_ZONE_UPDATE = 200.0   # RK2 with 5 FP64 conserved variables
# FP64 work of the stage kernel per RK2 zone-update on this workload: the DADD + DMUL + DFMA
# thread instructions the kernel executes (ncu sass counters of one stage launch of each kind
# on a 128^3 pack of 64^3 blocks, per zone), by arithmetic mode
FP64_LANE_OPS_PER_ZONE_UPDATE = {"fast": 1981.0, "exact": 2364.0}
FP64_LANES_PER_CLK_PER_SM = 2.0    # DFMA lanes per clock per SM on GB300 (measured)
# DRAM bytes (read + write) per zone per stage launch, same captures (the 256^3 launches
# process 8x the blocks of the 128^3 capture, so traffic is scaled by zones)
TRAFFIC_BYTES_PER_ZONE_LAUNCH = {"fast": 628.3, "exact": 612.7}
TRAFFIC_LAUNCH = {"fast": "8 lines, dynamic schedule (not the tuned launch)",
                  "exact": "256 threads, 3 lines, dynamic schedule, 80-register build: the tuned launch"}
PARITY = {
    "exact": "bit-identical to the oracle (the reference's FP64 CPU path): one step of this "
             "256^3 pack with this launch, 50 steps of 128^3, the refined RT pack over 100 "
             "steps and blast members to t = 0.1 (tests/test_gpu_headline.py)",
    "fast": "not parity-carrying: PPM limiter branches switch on one-ulp differences (50 of "
            "16.7M cells off by up to 8e-7 after one step of this pack; end-of-run L1(rho) "
            "< 1e-10 on KH, 1.5e-4 on blast members)",
}


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return None


def workload_config(cfg, ws):
    """The config object of the JSON line (the same in both arms)."""
    return {"workload": WORKLOAD, "zones": cfg.zones(), "meshblocks": cfg.nblocks,
            "parallelism": "replica per rank" if ws > 1 else "none (one pack)",
            "l2": "no flush: inputs larger than L2 (state 1.0 GB, ~4 GB working set)"}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured", d
    return 6800.0, "fallback", {}


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        ClockSampler.count = getattr(ClockSampler, "count", 0) + 1
        self.path = "/tmp/aph_clocks_%d_%d.csv" % (os.getpid(), ClockSampler.count)

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
            # let nvidia-smi finish starting (its driver initialisation stalls other processes'
            # CUDA calls for a moment) before the timed region begins
            time.sleep(1.0)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("APH_BENCH_BACKEND") != "gloo" else "gloo")
        return dist, rank, ws
    return None, 0, 1


def cpu_baseline(cfg, cons, nsteps, threads=None, warmup=1):
    """Oracle (C++ FP64 restatement of the reference path) on the host cores."""
    from oracle import oracle as O
    if threads:
        O.set_num_threads(threads)
    m = O.Mesh(cfg)
    m.set_cons(cons)
    m.run(nsteps=warmup)
    t0 = time.perf_counter()
    m.run(nsteps=nsteps)
    el = time.perf_counter() - t0
    return cfg.zones() * nsteps / el, O.num_threads(), el


def amr_leg(args, warmup):
    """The uneven refined pack: batched stepper vs the plain launch paths (rank 0)."""
    import torch
    from apophis_gb300 import amr, hydro
    cfg, cons = amr.rt2d_amr()
    zones = cfg.zones()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def timed(fn, n):
        torch.cuda.synchronize()
        a, b = ev(), ev()
        a.record()
        fn(n)
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / n

    st = amr.AmrStepper(cfg, cons, exact=args.exact)
    if args.launch:  # a given launch configuration, as for the headline
        c = st.config
        c.update(json.loads(args.launch))
        st.set_config(c)
        tune = {"config": st.config}
    else:
        tune = None if args.no_tune else st.autotune(trial_steps=2)
    st.step(warmup)
    st.status()
    stage_ms = st.profile(nsteps=2)
    nsteps = 100
    bms = timed(st.step, nsteps)
    status = st.status()
    st.close()
    out = {"mode": "exact" if args.exact else "fast",
           "workload": "rt2d_amr: 1440 meshblocks (160 of 32^2 at level 0, 256 + 1024 of 16^2 "
                       "at levels 1-2), 491,520 zones, PPM+HLLC, RK2, gravity -0.1, FP64",
           "batched": {"value": zones / (bms * 1e-3), "ms_per_step": bms, "steps": nsteps,
                       "stage_ms": stage_ms, "launches_per_step": 3,
                       "launch": tune["config"] if tune else None, "sim_time": status["time"]}}
    if not args.no_plain:
        drv = amr.AmrDriver(cfg, cons, exact=args.exact)
        drv.run(nsteps=2)
        pms = timed(lambda n: drv.run(nsteps=n), 20)
        out["plain_per_pack"] = {"value": zones / (pms * 1e-3), "ms_per_step": pms}
        drv.md.close()
        del drv
        # per meshblock, host-driven: each kernel launched once per block through the C ABI
        drv = amr.AmrDriver(cfg, cons, exact=args.exact, per_block=True)
        drv.run(nsteps=1)
        hms = timed(lambda n: drv.run(nsteps=n), 2)
        # the same launches replayed from one CUDA graph (no host cost): fixed dt, each block's
        # dt estimate written to the device
        dts = torch.empty(cfg.nblocks, dtype=torch.float64, device="cuda")
        from apophis_gb300 import _capi

        def body():
            drv.step(1e-5)
            for b, p in enumerate(drv.md.block_packs):
                _capi.call("aph_hydro_estimate_timestep_async", p,
                           ctypes.c_void_p(dts.data_ptr() + 8 * b), hydro.stream_handle())
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            body()
        torch.cuda.current_stream().wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            body()
        g.replay()
        gms = timed(lambda n: [g.replay() for _ in range(n)], 10)
        launches = cfg.nblocks * (2 * 5 + 3) + 2
        out["plain_per_meshblock"] = {"value": zones / (hms * 1e-3), "ms_per_step": hms,
                                      "launches_per_step": launches, "driver": "host (ctypes)"}
        out["plain_per_meshblock_graph"] = {"value": zones / (gms * 1e-3), "ms_per_step": gms,
                                            "launches_per_step": launches,
                                            "driver": "one CUDA graph per step"}
        del g
        drv.md.close()
        del drv
        torch.cuda.empty_cache()
        out["batched_vs_plain_per_meshblock_graph"] = gms / bms
        out["batched_vs_plain_per_meshblock"] = hms / bms
        out["batched_vs_plain_per_pack"] = pms / bms
    bytes_per_launch = BYTES_PER_ZONE_UPDATE * zones / len(stage_ms)
    out["hbm_achieved_gbs"] = bytes_per_launch / (sum(stage_ms) / len(stage_ms) * 1e-3) / 1e9
    return out


def ensemble_leg(args):
    """The batched blast ensemble to t = 0.1 (rank 0)."""
    import torch
    from apophis_gb300 import ensemble
    ens, flat = ensemble.blast_ensemble()
    st = ensemble.EnsembleStepper(ens, flat, exact=args.exact)
    tune = None if args.no_tune else st.autotune(trial_steps=2)
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    a, b = ev(), ev()
    torch.cuda.synchronize()
    a.record()
    launched = st.run_to_end(chunk=16)
    b.record()
    torch.cuda.synchronize()
    sec = a.elapsed_time(b) / 1e3
    ms = st.member_status()
    st.close()
    zu = sum(c.zones() * k for c, k in zip(ens.members, ms["ncycle"]))
    return {"mode": "exact" if args.exact else "fast",
            "workload": "64 blast2d members (%d blocks of 64^2, %d zones), PPM+HLLC, RK2, "
                        "CFL 0.3, to t = 0.1" % (ens.nblocks, ens.zones()),
            "value": zu / sec, "unit": UNIT, "seconds": sec, "zone_updates": zu,
            "member_steps_min_max": [min(ms["ncycle"]), max(ms["ncycle"])],
            "steps_launched": launched, "launches_per_step": 3,
            "launch": tune["config"] if tune else None,
            "end_time_min_max": [min(ms["time"]), max(ms["time"])]}


def ensemble_adjoint_leg(ckpt=20):
    """The blast ensemble's reverse sweep with respect to every member's initial state (the
    gradient with respect to initial pressure is lambda_E / (gamma - 1) of it), all members
    in the same launches: the members' dt schedules are recorded from a forward run to
    t = 0.1, then the checkpointed rollout and its reverse sweep are timed (rank 0)."""
    import torch
    from apophis_gb300 import ensemble
    from apophis_gb300.adjoint import EnsembleAdjoint
    ens, flat = ensemble.blast_ensemble()
    st = ensemble.EnsembleStepper(ens, flat, exact=False)
    st.autotune(trial_steps=1)
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    a, b = ev(), ev()
    torch.cuda.synchronize()
    a.record()
    st.run_to_end(chunk=16)
    b.record()
    torch.cuda.synchronize()
    fwd_s = a.elapsed_time(b) / 1e3
    st.close()
    st = ensemble.EnsembleStepper(ens, flat, exact=False)
    dts = []
    while True:
        ms = st.member_status()
        if max(ms["dt"]) == 0.0:
            break
        dts.append(ms["dt"])
        st.step(1)
    st.close()
    del st
    torch.cuda.empty_cache()
    adj = EnsembleAdjoint(ens)
    u0 = torch.from_numpy(flat).cuda()
    adj.autotune(u0)
    a, b, c = ev(), ev(), ev()
    a.record()
    uT = adj.forward_members(u0, dts, ckpt)
    b.record()
    lam = torch.zeros_like(uT)
    lam.copy_(uT)  # d(0.5 |U(T)|^2)/dU(T)
    lam0 = adj.backward(lam)
    c.record()
    torch.cuda.synchronize()
    ok = bool(torch.isfinite(lam0).all())
    tape_s, bwd_s = a.elapsed_time(b) / 1e3, b.elapsed_time(c) / 1e3
    adj.close()
    return {"workload": "64-member blast ensemble to t = 0.1 (%d steps), PPM+HLLC, RK2, "
                        "checkpoint every %d" % (len(dts), ckpt),
            "forward_s": fwd_s, "checkpointed_forward_s": tape_s, "backward_s": bwd_s,
            "ratio": bwd_s / fwd_s, "finite": ok,
            "note": "backward includes the recomputation of each checkpoint segment; forward "
                    "is the batched stepper run to t = 0.1"}


def adjoint_leg(nsteps=40):
    """Adjoint/forward time ratio on the differentiable rollout (rank 0)."""
    import torch
    from apophis_gb300 import problems
    from apophis_gb300.adjoint import Adjoint
    from apophis_gb300.stepper import Stepper
    cfg, cons = problems.kh2d(n=512, block=64, ng=2, recon="plm", rsolver="hlle")
    u0 = torch.from_numpy(cons).cuda()
    adj = Adjoint(cfg)
    adj.autotune(u0)
    dts = [2e-4] * nsteps
    adj.forward(u0, dts[:4], 2)
    adj.backward(torch.ones_like(u0))
    torch.cuda.synchronize()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    a, b, c = ev(), ev(), ev()
    a.record()
    uT = adj.forward(u0, dts, 20)
    b.record()
    adj.backward(torch.ones_like(uT))
    c.record()
    torch.cuda.synchronize()
    fwd_tape = a.elapsed_time(b) / nsteps
    bwd = b.elapsed_time(c) / nsteps
    adj.close()
    st = Stepper(cfg, cons, exact=False, fixed_dt=2e-4)
    st.autotune(trial_steps=1)
    st.step(3)
    st.status()
    a, b = ev(), ev()
    a.record()
    st.step(nsteps)
    b.record()
    torch.cuda.synchronize()
    fwd = a.elapsed_time(b) / nsteps
    st.close()
    return {"workload": "kh2d 512^2 (64 blocks of 64^2), PLM+HLLE, RK2, %d steps, checkpoint "
                        "every 20" % nsteps,
            "forward_ms_per_step": fwd, "checkpointed_forward_ms_per_step": fwd_tape,
            "backward_ms_per_step": bwd, "ratio": bwd / fwd,
            "note": "backward includes the recomputation of each checkpoint segment"}


def cpu_baseline_amr(nsteps=2):
    """The refined-mesh oracle on the RT pack (host cores)."""
    from apophis_gb300 import amr
    from oracle import oracle as O
    cfg, cons = amr.rt2d_amr()
    m = O.AmrMesh(cfg)
    m.set_cons(cons)
    m.run(nsteps=1)
    t0 = time.perf_counter()
    m.run(nsteps=nsteps)
    el = time.perf_counter() - t0
    return {"value": cfg.zones() * nsteps / el, "unit": UNIT, "cores": O.num_threads(),
            "kind": "port", "sample": "%d RK2 steps of the RT pack after 1 warm-up" % nsteps}


def table_leg(args):
    """Zone-updates/s of every configuration on every path, for the results table: the CPU
    oracle (host cores), the plain path per meshblock and per pack, and the batched stepper
    (rank 0; bounded samples)."""
    import torch
    from apophis_gb300 import ensemble, hydro, problems
    from apophis_gb300.stepper import Stepper
    from oracle import oracle as O

    def gpu_time(fn, n):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn(n)
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / n

    def uniform_rows(name, cfg, cons, nsteps, fixed_dt=0.0):
        zones = cfg.zones()
        out = {"workload": name, "zones": zones}
        m = O.Mesh(cfg)
        m.set_cons(cons)
        m.run(nsteps=1, fixed_dt=fixed_dt)
        t = time.perf_counter()
        m.run(nsteps=nsteps, fixed_dt=fixed_dt)
        out["cpu_oracle"] = zones * nsteps / (time.perf_counter() - t)
        out["cpu_cores"] = O.num_threads()
        for label, per_block, n in (("gpu_plain_per_meshblock", True, max(1, nsteps // 2)),
                                    ("gpu_plain_per_pack", False, nsteps)):
            d = hydro.Driver(cfg, cons, exact=args.exact, per_block=per_block)
            d.run(nsteps=1, fixed_dt=fixed_dt)
            out[label] = zones / gpu_time(lambda k: d.run(nsteps=k, fixed_dt=fixed_dt), n)
            d.md.close()
        st = Stepper(cfg, cons, exact=args.exact, fixed_dt=fixed_dt)
        st.autotune(trial_steps=1)
        st.step(3)
        st.status()
        out["gpu_batched_graph"] = zones / gpu_time(lambda k: (st.step(k), st.status()), 4 * nsteps)
        st.close()
        torch.cuda.empty_cache()
        return out

    rows = []
    cfg, cons = problems.sod(nx=256, recon="plm", rsolver="hlle", integrator="rk2", cfl=0.4)
    rows.append(uniform_rows("sod 1D 256 cells, PLM+HLLE, RK2", cfg, cons, 50))
    cfg, cons = problems.kh2d(n=512, block=64, ng=2, recon="plm", rsolver="hlle")
    rows.append(uniform_rows("kh2d 512^2 (64 x 64^2), PLM+HLLE, RK2", cfg, cons, 10, fixed_dt=2e-4))
    # the blast ensemble: every member on the CPU oracle and the per-pack plain path
    ens, flat = ensemble.blast_ensemble()
    zones = ens.zones()
    t_cpu = 0.0
    t_pack = 0.0
    for m_i, mcfg in enumerate(ens.members):
        mcons = ens.unpack(flat, m_i)
        m = O.Mesh(mcfg)
        m.set_cons(mcons)
        t = time.perf_counter()
        m.run(nsteps=1)
        t_cpu += time.perf_counter() - t
        d = hydro.Driver(mcfg, mcons, exact=args.exact)
        d.run(nsteps=1)
        t_pack += gpu_time(lambda k: d.run(nsteps=k), 2)
        d.md.close()
    rows.append({"workload": "blast ensemble, 64 members, PPM+HLLC, RK2 (one step of every member)",
                 "zones": zones, "cpu_oracle": zones / t_cpu, "cpu_cores": O.num_threads(),
                 "gpu_plain_per_pack": zones / t_pack})
    return rows


def run_reference(args, cfg, cons):
    dist, rank, ws = dist_init()
    if rank != 0:
        return
    # K full RK2 steps of the 256^3 pack after W warm-up steps (about 2 s each on 16 host cores)
    nsteps = max(1, args.steps)
    zps, cores, el = cpu_baseline(cfg, cons, nsteps, warmup=args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": zps, "unit": UNIT, "n_gpus": ws,
            "steps": nsteps, "warmup": args.warmup, "ms_per_step": el / nsteps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": workload_config(cfg, ws),
            "cpu_baseline": {"value": zps, "unit": UNIT, "cores": cores, "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": "%d full RK2 steps of the 256^3 pack after %d warm-up steps"
                                       % (nsteps, args.warmup)},
            "e2e": {"value": zps, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def timed_stepper(cfg, cons, exact, args, dist, local):
    """Autotune (or set) the launch, warm up, and time args.steps graph-replayed steps with
    CUDA events on the launching stream; returns (stepper, ms per step, stage ms, clocks,
    launch)."""
    import torch
    from apophis_gb300.stepper import Stepper
    st = Stepper(cfg, cons, exact=exact)
    if args.launch:
        c = st.config
        c.update(json.loads(args.launch))
        st.set_config(c)
    elif not args.no_tune:
        st.autotune(trial_steps=2)  # two timed steps per candidate: a steadier choice
    stream = torch.cuda.current_stream()
    st.step(args.warmup)
    st.status()
    stage_ms = st.profile(nsteps=2)  # per-stage kernel durations (roofline time)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        e0.record(stream)
        st.step(args.steps)
        e1.record(stream)
        barrier()
    ms = e0.elapsed_time(e1) / args.steps
    if dist is not None:
        t = torch.tensor([ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return st, ms, stage_ms, clk.summary(), st.config


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--n", type=int, default=256, help="mesh cells per side")
    ap.add_argument("--mode", default="exact", choices=["exact", "fast"],
                    help="arithmetic mode of the headline (exact: bit-identical to the oracle)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--launch", default=None,
                    help="JSON launch configuration of the stepper (keys of aph_stepper_config); "
                         "used instead of the autotuner, e.g. for reproducible profiles")
    ap.add_argument("--no-plain", action="store_true", help="skip the per-meshblock path")
    ap.add_argument("--no-fast", action="store_true", help="skip the other arithmetic mode's leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--no-amr", action="store_true", help="skip the refined-pack leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint ratio leg")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the blast-ensemble leg")
    ap.add_argument("--only", choices=["amr", "ensemble", "adjoint", "ensemble_adjoint", "table"],
                    help="run one extra leg alone and print its object (for profiling)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    exact = args.mode == "exact"
    if args.only:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        from apophis_gb300 import _build
        _build.build()
        args.exact = exact
        out = {"amr": lambda: amr_leg(args, args.warmup), "ensemble": lambda: ensemble_leg(args),
               "adjoint": adjoint_leg, "ensemble_adjoint": ensemble_adjoint_leg,
               "table": lambda: table_leg(args)}[args.only]()
        print(json.dumps({"only": args.only, args.only: out}), flush=True)
        return

    from apophis_gb300 import problems
    cfg, cons = problems.kh3d(n=args.n, block=64 if args.n >= 64 else args.n // 2, ng=4)
    if args.impl == "reference":
        run_reference(args, cfg, cons)
        return

    import torch
    dist, rank, ws = dist_init()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    from apophis_gb300 import _build, hydro
    _build.build()

    zones = cfg.zones()
    st, ms, stage_ms, clocks, launch = timed_stepper(cfg, cons, exact, args, dist, local)
    status = st.status()
    value = zones * ws / (ms * 1e-3)
    launches_per_step = 3  # two stage kernels + the dt-policy kernel

    # e2e: the state in pinned host memory as the packed interiors, through the C ABI
    # (aph_stepper_load_interiors / _store_interiors): every step loads its input from the
    # host and stores its result back, inside the timed region
    e2e = None
    if not args.no_e2e:
        stream = torch.cuda.current_stream()
        host = torch.empty(st.interior_shape(), dtype=torch.float64, pin_memory=True)
        st.store_interiors(host)
        nbytes = host.numel() * 8

        def e2e_step():
            st.load_interiors(host)
            st.step(1)
            st.store_interiors(host)

        def barrier():
            if dist is not None:
                dist.barrier()
            torch.cuda.synchronize()

        for _ in range(max(1, min(args.warmup, 2))):  # first transfers of a fresh pinned buffer
            e2e_step()
        with ClockSampler(local) as clk_e2e:
            barrier()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                e2e_step()
            barrier()
            t1 = time.perf_counter()  # before the sampler stops (its shutdown is not the step's)
        e2e_ms = (t1 - t0) * 1e3 / args.steps
        if dist is not None:
            t = torch.tensor([e2e_ms], device="cuda", dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e2e_ms = float(t.item())
        # the host link's share of an e2e step: the load and the store alone (CUDA events)
        link = {}
        for name, fn in (("load", lambda: st.load_interiors(host)),
                         ("store", lambda: st.store_interiors(host))):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(3):
                fn()
            b.record(stream)
            torch.cuda.synchronize()
            t = a.elapsed_time(b) / 3
            link[name + "_ms"] = t
            link[name + "_gbs"] = nbytes / (t * 1e-3) / 1e9
        e2e = {"value": zones * ws / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes, "ms_per_step": e2e_ms, "mode": args.mode,
               "host_link": link, "clocks": clk_e2e.summary()}
        del host
    st.close()
    del st
    torch.cuda.empty_cache()

    # the other arithmetic mode, same workload and timing
    other = None
    if not args.no_fast:
        omode = "fast" if exact else "exact"
        ost, oms, ostage, oclk, olaunch = timed_stepper(cfg, cons, not exact, args, dist, local)
        ost.close()
        del ost
        torch.cuda.empty_cache()
        other = {"mode": omode, "value": zones * ws / (oms * 1e-3), "ms_per_step": oms,
                 "stage_ms": ostage, "launch": olaunch, "clocks": oclk, "parity": PARITY[omode]}

    # plain per-meshblock launch path, bounded sample
    plain = None
    if rank == 0 and not args.no_plain:
        drv = hydro.Driver(cfg, cons, exact=exact, per_block=True)
        drv.run(nsteps=1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        drv.run(nsteps=2)
        torch.cuda.synchronize()
        pms = (time.perf_counter() - t0) * 1e3 / 2
        plain = {"value": zones / (pms * 1e-3), "ms_per_step": pms, "mode": args.mode,
                 "launches_per_step": 2 * cfg.nblocks * (1 + 3 + 1) + 2 + 2 + cfg.nblocks,
                 "driver": "one launch per kernel per meshblock"}
        del drv
        torch.cuda.empty_cache()
        # reference-style granularity: one launch per kernel per pack (the Kokkos kernels over a
        # MeshBlockPack)
        drv = hydro.Driver(cfg, cons, exact=exact, per_block=False)
        drv.run(nsteps=1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        drv.run(nsteps=2)
        torch.cuda.synchronize()
        kms = (time.perf_counter() - t0) * 1e3 / 2
        plain_pack = {"value": zones / (kms * 1e-3), "ms_per_step": kms, "mode": args.mode,
                      "launches_per_step": 2 * (1 + 3 + 1) + 2 + 2 + 1,
                      "driver": "one launch per kernel per pack"}
        del drv
        torch.cuda.empty_cache()

    hbm, peak_kind, pk = peaks()
    stage_sum = sum(stage_ms)
    per_launch_bytes = BYTES_PER_ZONE_UPDATE * zones / len(stage_ms)
    achieved = per_launch_bytes / (stage_sum / len(stage_ms) * 1e-3) / 1e9
    sm_mhz = clocks.get("sm_mhz") or pk.get("sm_max_mhz", 2070.0)
    fp64_peak = FP64_LANES_PER_CLK_PER_SM * 152 * sm_mhz * 1e6 / 1e9  # G lane-ops/s
    traffic = TRAFFIC_BYTES_PER_ZONE_LAUNCH[args.mode]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(cfg, ws),
        "mode": args.mode, "parity": PARITY[args.mode], "launch": launch,
        "e2e": e2e,
        "gpu_launches": launches_per_step * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm,
                     "traffic": traffic * zones / len(stage_ms) if traffic else None,
                     "traffic_note": ("ncu DRAM bytes per zone of one stage launch on a 128^3 "
                                      "pack (%s) x zones" % TRAFFIC_LAUNCH[args.mode])
                                     if traffic else "no capture of this mode's launch",
                     "kernel": "k_stage (batched stage, %s mode)" % args.mode,
                     "stage_ms": stage_ms, "peak_source": peak_kind},
        "fp64_pipe": {"note": "the FP64 pipe binds this kernel; achieved counts the DADD/DMUL/DFMA "
                              "it executes (ncu)",
                      "peak_source": "2 DFMA lanes/clk/SM x 152 SMs x sampled SM clock"},
        "clocks": clocks,
        "time_check": {"sim_time": status["time"], "ncycle": status["ncycle"]},
    }
    ops = FP64_LANE_OPS_PER_ZONE_UPDATE[args.mode]
    if ops:
        ach = ops * zones / (stage_sum * 1e-3) / 1e9
        line["fp64_pipe"].update({"achieved": ach, "peak": fp64_peak, "unit": "G lane-ops/s",
                                  "frac": ach / fp64_peak, "ops_per_zone_update": ops})
        # the bound that binds, beside the HBM figures of the roofline object
        line["roofline"]["fp64_pipe_frac"] = ach / fp64_peak
    if other is not None:
        line["other_mode"] = other
    if plain is not None:
        line["plain"] = plain
        line["plain_per_pack"] = plain_pack
        line["batched_vs_plain"] = value / ws / plain["value"]
        line["batched_vs_plain_per_pack"] = value / ws / plain_pack["value"]
    args.exact = exact
    if rank == 0 and not args.no_amr:
        line["amr"] = amr_leg(args, args.warmup)
        line["gpu_launches_amr_batched_step"] = 3
    if rank == 0 and not args.no_ensemble:
        line["ensemble"] = ensemble_leg(args)
    if rank == 0 and not args.no_adjoint:
        line["adjoint"] = adjoint_leg()
        if not args.no_ensemble:
            line["ensemble_adjoint"] = ensemble_adjoint_leg()
    if rank == 0 and not args.no_cpu:
        runs = [cpu_baseline(cfg, cons, 1) for _ in range(5)]
        zps, cores, el = sorted(runs)[2]
        line["cpu_baseline"] = {"value": zps, "unit": UNIT, "cores": cores, "kind": "port",
                                "cpu_model": cpu_model(),
                                "sample": "median of 5 runs of 1 full RK2 step of the 256^3 pack, "
                                          "each after 1 warm-up step (%.1f s per run)" % el}
        if "amr" in line:
            line["amr"]["cpu_baseline"] = cpu_baseline_amr()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
