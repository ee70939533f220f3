"""Benchmark of the PIHM right-hand side on GB300.

Workload (the configuration the headline metric is quoted on): one synthetic
watershed of 1,000,000 triangular elements and 30,000 river segments (the
generator of pihm_gpu.watershed, seed 0), evaluated on 100 perturbed states
(a wet reference state with every storage jittered x U(0.9, 1.1), seeded per
state: pihm_gpu.workloads.rhs_state, shared with the reference arm and the
parity tests).  One "step" evaluates the right-hand side once on every state
of the set, in order; 100 states are 2.4 GB of y, far more than the 129 MB
L2, so no L2 flush is needed between evaluations.

Printed (one JSON line, rank 0):
  value     element-evals/s with the states resident in HBM (device pointers,
            internal order), the states spread over four contexts of the mesh
            on their own streams, CUDA events from the first launch to the
            last stream's end
  e2e       the same metric through the host-buffer C-ABI calls, every
            state copied from pinned host memory and every derivative back
            inside the timed region: the faster of pihm_gpu_rhs_host one
            evaluation at a time (sync_value) and pihm_gpu_rhs_host_async on
            four contexts of the mesh, whose transfers run beside each other's
            kernels, with one or four evaluations queued per context
            (pipelined); mode says which
  roofline  the right-hand-side evaluation against the measured HBM copy
            bandwidth: algorithmic bytes (332 B per element + 184 B per
            segment) / device time of one evaluation
  cpu_baseline  the CPU restatement of the reference ODE() (oracle/, OpenMP
            build on all host cores, and the 1-thread build) on a bounded
            sample of the same states

`--impl reference` times that CPU implementation alone as the reference arm,
on the same states in the same order.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "pihm-cuda_gb300"))

NELEM, NRIVER = 1_000_000, 30_000
NSTATES = 100
STATES_PER_STEP = 100      # a step is one pass over the whole state set
YDOT_RING = 12             # derivative buffers cycled through (a multiple of the context count)
PIPE_DEPTH = 4             # evaluations queued per context in the pipelined end-to-end leg
E2E_REPS = 3               # timed passes per pipelined configuration (the median is kept)
BYTES_PER_ELEM, BYTES_PER_SEG = 332, 184
METRIC = "RHS element-evals/s"
UNIT = "elem-evals/s"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, world: int, device=None) -> float:
    """The largest x over the ranks (the slowest rank's time); x itself on one
    rank.  `device`: where the collective's tensor lives (the GPU under NCCL,
    the host under gloo)."""
    if world <= 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device or "cpu")
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world: int, units_per_rank: float, ms: float) -> float:
    """Whole-job throughput of `world` replicas that each processed
    units_per_rank in at most ms milliseconds (the slowest rank's time)."""
    return world * units_per_rank / (ms * 1e-3)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region: the sampler starts, its
    first sample is awaited, and only the samples stamped between entering
    and leaving the block are kept."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.stamped = []
        self.lines = []
        self.t0 = self.t1 = 0.0

    def _read(self):
        for line in self.proc.stdout:
            if line.strip():
                self.stamped.append((time.monotonic(), line))

    def __enter__(self):
        import threading
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
            deadline = time.monotonic() + 10.0
            while not self.stamped and time.monotonic() < deadline and self.proc.poll() is None:
                time.sleep(0.02)
        except Exception:
            self.proc = None
        self.t0 = time.monotonic()
        return self

    def __exit__(self, *a):
        self.t1 = time.monotonic()
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.reader.join(timeout=5)
        self.lines = [l for t, l in self.stamped if self.t0 <= t <= self.t1]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm),
                "window_s": round(self.t1 - self.t0, 3)}


def workload_config(world: int) -> dict:
    """The `config` both arms print (the same workload, so the same dict)."""
    return {"workload": f"rhs_{NELEM}elem_{NRIVER}seg", "nelem": NELEM, "nriver": NRIVER,
            "states": NSTATES, "evals_per_step": STATES_PER_STEP,
            "states_source": "pihm_gpu.workloads.rhs_state(base, k), k = 0..states-1, in order",
            "l2": "inputs larger than L2 (100 states x 24.5 MB per step)",
            "parallelism": "replicas" if world > 1 else "single"}


def host_cores() -> dict:
    n = os.cpu_count() or 1
    try:
        avail = len(os.sched_getaffinity(0))
    except Exception:
        avail = n
    return {"host_cores": n, "host_cores_available": avail}


def cpu_time_oracle(ws, state_of, threads, omp=True, max_seconds=12.0, min_evals=2, max_evals=200):
    """Time the CPU restatement (test infrastructure) on a bounded sample of
    the benchmark's states, in order; returns (evaluations, seconds, threads)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    from pihm_gpu import workloads as WL
    o = Oracle(ws, omp=omp, threads=threads if omp else None)
    o.set_forcing(*WL.rhs_forcing(ws))
    base = WL.rhs_base_state(ws)
    o.set_ws0_surf(base[:ws.nelem])
    pre = [state_of(k) for k in range(min(NSTATES, 4))]
    o.rhs(pre[0])  # warm
    n = 0
    t0 = time.perf_counter()
    while True:
        o.rhs(pre[n % len(pre)])
        n += 1
        el = time.perf_counter() - t0
        if (el >= max_seconds and n >= min_evals) or n >= max_evals:
            break
    thr = o.threads if omp else 1
    o.close()
    return n, el, thr


def run_reference_arm(args):
    """CPU implementation of the path (the OpenMP restatement of the
    reference ODE() on all host cores) on the same workload: each step
    evaluates the same states in the same order as the GPU arm's step (a
    fixed subsample of them when the whole run would not end within a few
    minutes), same metric."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    import pihm_gpu.watershed as W
    from pihm_gpu import workloads as WL
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    ws = W.generate(NELEM, NRIVER, seed=WL.RHS_SEED)
    base = WL.rhs_base_state(ws)
    states = [WL.rhs_state(base, k) for k in range(NSTATES)]
    threads = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    o = Oracle(ws, omp=True, threads=threads)
    o.set_forcing(*WL.rhs_forcing(ws))
    o.set_ws0_surf(base[:ws.nelem])
    # warm-up: one evaluation per warm-up step; it also sizes the sample
    t0 = time.perf_counter()
    for w in range(max(1, args.warmup)):
        o.rhs(states[w % NSTATES])
    per_eval = (time.perf_counter() - t0) / max(1, args.warmup)
    budget_s = 180.0
    stride = 1
    while args.steps * (STATES_PER_STEP // stride) * per_eval > budget_s and stride < STATES_PER_STEP:
        stride += 1
    picked = list(range(0, STATES_PER_STEP, stride))
    t0 = time.perf_counter()
    for s in range(args.steps):
        for e in picked:
            o.rhs(states[(s * STATES_PER_STEP + e) % NSTATES])
    el = time.perf_counter() - t0
    n_evals = len(picked) * args.steps
    value = NELEM * n_evals / el
    cores = o.threads
    sample = (f"every state of each step ({len(picked)} evaluations of the {NELEM}-element mesh)"
              if stride == 1 else
              f"{len(picked)} of each step's {STATES_PER_STEP} states (every {stride}th, in order)")
    o.close()
    # the 1-thread build on a bounded sample of the same states
    serial = None
    try:
        n1, el1, _ = cpu_time_oracle(ws, lambda k: states[k], 1, omp=False, max_seconds=8.0, min_evals=2)
        serial = {"value": NELEM * n1 / el1, "unit": UNIT, "cores": 1, "kind": "port",
                  "sample": f"{n1} evaluations, {el1:.1f} s, 1-thread build"}
    except Exception as exc:
        serial = {"error": repr(exc)}
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3 * (STATES_PER_STEP / len(picked)),
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(1),
        "cpu_baseline": dict({"value": value, "unit": UNIT, "cores": cores,
                              "kind": "port", "sample": sample, "serial": serial}, **host_cores()),
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


BATCH_N, BATCH_LO, BATCH_HI, BATCH_STEPS, BATCH_SEQ_SAMPLE = 256, 2000, 200000, 10, 256
SERVE_N, SERVE_LO, SERVE_HI, SERVE_STEPS, SERVE_LOAD = 48, 1000, 500000, 10, 0.8
SERVE_ARENA_BYTES, SERVE_MAX_REQ = 4 << 30, 64  # the arena's device-memory budget (about 3M elements)


def _pct(a, q):
    import numpy as np
    return float(np.percentile(np.asarray(a), q)) if len(a) else None


def bench_batched():
    """256 watersheds integrated together vs one by one through the plain path."""
    import numpy as np
    import torch
    from pihm_gpu import workloads as WL
    from pihm_gpu.batch import Batch, limits_for
    from pihm_gpu.single import solve_alone
    t = time.perf_counter()
    cases = WL.make_cases(WL.batched_specs(BATCH_N, BATCH_LO, BATCH_HI, BATCH_STEPS))
    gen_s = time.perf_counter() - t
    torch.cuda.synchronize()
    b = Batch(limits_for([c["ws"] for c in cases], BATCH_STEPS))
    t0 = time.perf_counter()
    ids = b.add_many(cases, threads=min(16, os.cpu_count() or 1))
    assert all(i is not None for i in ids)
    t1 = time.perf_counter()
    b.step()
    t2 = time.perf_counter()
    res = [b.result(i) for i in ids]
    t3 = time.perf_counter()
    inf = b.info()
    b.close()
    evals = sum(c["ws"].nelem * (r["stats"].nfe + r["stats"].nfes) for c, r in zip(cases, res))
    sizes = np.array([c["ws"].nelem for c in cases])
    pick = np.argsort(sizes)[np.linspace(0, BATCH_N - 1, BATCH_SEQ_SAMPLE).astype(int)]
    seq_s, same = 0.0, 0
    for k in pick:
        ts = time.perf_counter()
        r = solve_alone(cases[k])
        seq_s += time.perf_counter() - ts
        same += int(np.array_equal(r["y"], res[k]["y"]) and np.array_equal(r["outlet"], res[k]["outlet"]))
    seq_all = seq_s * BATCH_N / len(pick)
    full = len(set(pick.tolist())) == BATCH_N
    return {
        "metric": "batched solves/s", "unit": "solves/s",
        "value": BATCH_N / (t2 - t1), "e2e_value": BATCH_N / (t3 - t0),
        "workload": f"{BATCH_N} watersheds, {int(sizes.sum())} elements (log-uniform {BATCH_LO}..{BATCH_HI}), "
                    f"{BATCH_STEPS} model steps of 60 s each from RelaxIc",
        "solve_s": t2 - t1, "admit_s": t1 - t0, "readback_s": t3 - t2, "generate_s": gen_s,
        "elem_evals_per_s": evals / (t2 - t1), "rounds": inf.rounds, "rhs_rounds": inf.rhs_rounds,
        "gpu_launches": inf.launches, "launches_per_round": inf.launches / max(inf.rounds, 1),
        "tuner": {"program_variant": int(inf.program_variant), "program_tuning": bool(inf.tuning),
                  "rhs_shape": ["512x2", "256x4", "128x8"][int(inf.rhs_shape)], "rhs_tuning": bool(inf.rhs_tuning)},
        "sequential": {"value": BATCH_N / seq_all, "unit": "solves/s",
                       "sample": (f"all {BATCH_N} watersheds one by one through the plain path (create, "
                                  f"solve, read back), {seq_s:.2f} s" if full else
                                  f"{len(pick)} of {BATCH_N} watersheds stratified by size, plain path "
                                  f"(create, solve, read back), {seq_s:.2f} s, scaled to all")},
        "speedup_e2e": (BATCH_N / (t3 - t0)) / (BATCH_N / seq_all),
        "bit_identical_to_plain_path": f"{same}/{len(pick)}",
    }


SCAT_STATES, SCAT_EVALS = 20, 60
RHS_CONTEXTS = 4  # contexts of the mesh the states are spread over (value and pipelined e2e)


def bench_scattered():
    """The headline right-hand side on an unstructured mesh of the same size:
    the Delaunay triangulation of 1,000,000 elements' scattered nodes
    (pihm_gpu.watershed.generate(mesh="scattered"): irregular node degrees
    and element sizes, as a mesh generator's output), jittered states,
    device-resident, CUDA events."""
    import torch
    import pihm_gpu.watershed as W
    from pihm_gpu.capi import GpuRhs
    t = time.perf_counter()
    ws = W.generate(NELEM, NRIVER, seed=1, mesh="scattered")
    gen_s = time.perf_counter() - t
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.Stream(device=dev)
    g = GpuRhs(ws, stream=stream.cuda_stream)
    g.set_forcing(*W.random_forcing(ws, 3))
    base = W.reference_state(ws, 2)
    g.set_ws0_surf(base[:ws.nelem])
    with torch.cuda.stream(stream):
        st = torch.empty((SCAT_STATES, ws.neq), dtype=torch.float64, device=dev)
        stage = torch.empty(ws.neq, dtype=torch.float64, device=dev)
        for k in range(SCAT_STATES):
            stage.copy_(torch.from_numpy(W.jitter(base, 300 + k)))
            g.to_internal(stage.data_ptr(), st[k].data_ptr())
        yd = torch.empty((2, ws.neq), dtype=torch.float64, device=dev)
    for k in range(3):
        g.rhs_device(st[k].data_ptr(), yd[k % 2].data_ptr())
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(SCAT_EVALS):
        g.rhs_device(st[k % SCAT_STATES].data_ptr(), yd[k % 2].data_ptr())
    e1.record(stream)
    e1.synchronize()
    assert g.status() == 0
    ms = e0.elapsed_time(e1) / SCAT_EVALS
    g.set_profiling(True)
    g.rhs_device(st[0].data_ptr(), yd[0].data_ptr())
    kt = g.kernel_times()
    g.close()
    return {"metric": "RHS element-evals/s", "unit": "elem-evals/s", "value": ws.nelem / (ms * 1e-3),
            "ms_per_eval": ms, "generate_s": gen_s,
            "workload": f"{ws.nelem} elements, {ws.nriver} segments, Delaunay mesh of scattered nodes, "
                        f"{SCAT_STATES} jittered states, {SCAT_EVALS} evaluations",
            "kernel_ms": {k: v[0] / v[1] for k, v in kt.items()}}


FLUX_NELEM, FLUX_LAYERS, FLUX_STATES, FLUX_STEPS, FLUX_LSM = 200_000, 4, 40, 60, 3600.0


def bench_flux_pihm():
    """Flux-PIHM (the c2 configuration, 200,000 elements, 4 Noah soil
    layers): the right-hand side with Noah's outputs fused into the element
    kernel beside the plain right-hand side on the same states; the Noah
    land-surface step and its post-model-step update (include/pihm_noah.h)
    timed alone; and a coupled run of the reference's Flux-PIHM model-step
    loop on the device (pihm_gpu.single.NoahWatershed: hourly forcing, Noah
    every land-surface step of an hour, the integration of each 60 s model
    step, Summary and NoahHydrol) for FLUX_STEPS model steps of the
    configuration's 3 days."""
    import numpy as np
    import torch
    import pihm_gpu.watershed as W
    from pihm_gpu import noah as N
    from pihm_gpu import workloads as WL
    from pihm_gpu.capi import GpuRhs
    from pihm_gpu.single import NoahWatershed
    from pihm_gpu.solver import StepControl, run_steps
    ws = W.generate(FLUX_NELEM, WL.river_count(FLUX_NELEM), seed=2)
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.Stream(device=dev)
    base = W.reference_state(ws, 3)
    params, state = N.synthetic_noah(ws, seed=2, nlayers=FLUX_LAYERS)
    gen = torch.Generator(device=dev)
    gen.manual_seed(99)
    res, noah_ms = {}, {}
    for mode in ("plain", "noah"):
        g = GpuRhs(ws, stream=stream.cuda_stream)
        g.set_forcing(*W.random_forcing(ws, 5))
        g.set_ws0_surf(base[:ws.nelem])
        with torch.cuda.stream(stream):
            b = torch.from_numpy(base).to(dev)
            ref = torch.stack([b * (0.9 + 0.2 * torch.rand(ws.neq, generator=gen, device=dev, dtype=torch.float64))
                               for _ in range(FLUX_STATES)])
            st = torch.empty_like(ref)
            for k in range(FLUX_STATES):
                g.to_internal(ref[k].data_ptr(), st[k].data_ptr())
            yd = torch.empty((1, ws.neq), dtype=torch.float64, device=dev)
        if mode == "noah":
            # the right-hand side's Noah inputs from the device Noah itself
            g.noah_init(params, state)
            g.noah_begin(st[0].data_ptr())
            g.noah_set_forcing(N.forcing(ws, 12, seed=2))
            g.noah_step(FLUX_LSM)
        for k in range(3):
            g.rhs_device(st[k].data_ptr(), yd[0].data_ptr())
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(FLUX_STATES):
            g.rhs_device(st[k].data_ptr(), yd[0].data_ptr())
        e1.record(stream)
        e1.synchronize()
        assert g.status() == 0
        res[mode] = FLUX_NELEM * FLUX_STATES / (e0.elapsed_time(e1) * 1e-3)
        if mode == "noah":
            # Noah's land-surface step and its post-step alone, CUDA events
            for name, fn in (("noah_step", lambda k: g.noah_step(FLUX_LSM)),
                             ("noah_post_step", lambda k: g.noah_post_step(st[k].data_ptr(), 60.0))):
                fn(0)
                stream.synchronize()
                e0.record(stream)
                for k in range(5):
                    fn(k)
                e1.record(stream)
                e1.synchronize()
                noah_ms[name] = e0.elapsed_time(e1) / 5
            assert g.status() == 0
        g.close()
    # the coupled run
    m = NoahWatershed(ws, W.relax_state(ws), params, state, lambda h: N.forcing(ws, h, seed=2),
                      lsm_step=FLUX_LSM)
    torch.cuda.synchronize()
    t = time.perf_counter()
    r = run_steps(m, StepControl(), FLUX_STEPS, m.set_forcing, outlet=int(np.where(ws.arrays["down"] < 0)[0][0]))
    torch.cuda.synchronize()
    solve_s = time.perf_counter() - t
    noah_steps = m.noah_steps
    sneqv = m.g.noah_get("sneqv")
    y_plain = m.read_state()
    m.close()
    evals = int(r["stats"].nfe + r["stats"].nfes)
    hours = FLUX_STEPS * 60.0 / 3600.0
    # the same hour as a batch of one in the batch engine (Noah on the device
    # there too; each round's vector operations fused per watershed)
    engine = None
    try:
        from pihm_gpu.batch import Batch, limits_for
        forcings = [N.forcing(ws, h, seed=2) for h in range(int(hours) + 1)]
        b = Batch(limits_for([ws], FLUX_STEPS))
        torch.cuda.synchronize()
        t = time.perf_counter()
        i = b.add_noah(ws, W.relax_state(ws), StepControl(), params, state, forcings, FLUX_LSM, FLUX_STEPS)
        b.step()
        got = b.result(i)
        torch.cuda.synchronize()
        ewall = time.perf_counter() - t
        b.close()
        engine = {"wall_s": ewall, "bit_identical_to_plain_path": bool(np.array_equal(got["y"], y_plain))}
    except Exception as exc:
        engine = {"error": repr(exc)}
    return {"metric": "Flux-PIHM RHS element-evals/s", "unit": "elem-evals/s", "value": res["noah"],
            "plain_rhs_value": res["plain"],
            "workload": f"{FLUX_NELEM} elements, {ws.nriver} segments, {FLUX_LAYERS} Noah soil layers, Noah on the "
                        f"device (pihm_gpu_noah_*), {FLUX_STATES} jittered states",
            "noah_ms": noah_ms,
            "noah_element_steps_per_s": FLUX_NELEM / (noah_ms["noah_step"] * 1e-3),
            "coupled_run": {"model_steps": FLUX_STEPS, "simulated_hours": hours, "wall_s": solve_s,
                            "noah_steps": noah_steps, "integrator_steps": int(r["stats"].nst), "rhs_evals": evals,
                            "elem_evals_per_s": FLUX_NELEM * evals / solve_s,
                            "simulated_hours_per_wall_hour": hours * 3600.0 / solve_s,
                            "fraction_of_the_3_day_run": hours / 72.0,
                            "snow_covered_elements": int((sneqv > 0).sum()),
                            "batch_engine": engine,
                            "workload": "RelaxIc, hourly synthetic Noah forcing (pihm_gpu.noah.forcing), land-surface "
                                        f"step {int(FLUX_LSM)} s, model step 60 s, reltol 1e-4"}}


LAND_STEPS = 96            # one day of 900 s land-surface steps
LAND_BYTES_PER_ELEM = 260  # algorithmic: 196 B read (with the monthly aerodynamic term), 64 B written


def bench_land(ws):
    """The land-surface step (forcing interpolation, snow, interception,
    evapotranspiration; include/pihm_land.h) on the headline mesh: 64
    stations, 8 LAI series, a day of 900 s steps, timed with CUDA events on
    the launching stream; the OpenMP restatement on the host cores on a
    bounded sample of the same steps."""
    import numpy as np
    import torch
    import pihm_gpu.land as L
    from pihm_gpu.capi import GpuRhs
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.Stream(device=dev)
    land = L.synthetic_land(ws, hours=LAND_STEPS // 4 + 2, nstations=64, nlai=8, seed=21)
    g = GpuRhs(ws, stream=stream.cuda_stream)
    g.land_init(land)
    # a soil state with the water table anywhere in the column
    rng = np.random.default_rng(5)
    depth = np.asarray(ws.arrays["depth"])
    gw = depth * rng.uniform(0.0, 1.0, depth.size)
    unsat = (depth - gw) * rng.uniform(-0.1, 1.2, depth.size)
    y = np.zeros(ws.neq)
    ne = ws.nelem
    y[ne:2 * ne], y[2 * ne:3 * ne] = unsat, gw
    with torch.cuda.stream(stream):
        yr = torch.from_numpy(y).to(dev)
        yi = torch.empty_like(yr)
        g.to_internal(yr.data_ptr(), yi.data_ptr())
    t0 = L.epoch("2009-01-01 00:00")
    for k in range(3):
        g.land_step(t0 + 900 * k, 900.0, yi.data_ptr())
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(LAND_STEPS):
        g.land_step(t0 + 900 * k, 900.0, yi.data_ptr())
    e1.record(stream)
    e1.synchronize()
    assert g.status() == 0
    ms = e0.elapsed_time(e1) / LAND_STEPS
    value = ne / (ms * 1e-3)
    g.close()
    cpu = None
    try:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        o = oracle.OracleLand(land, ws, omp=True)
        n, t = 0, time.perf_counter()
        while n < 3 or (time.perf_counter() - t < 10.0 and n < LAND_STEPS):
            assert o.step(t0 + 900 * n, 900.0, unsat, gw) == 0
            n += 1
        cpu_s = time.perf_counter() - t
        cpu = {"value": ne * n / cpu_s, "unit": "element-steps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{n} land-surface steps of the {ne}-element mesh (OpenMP restatement)"}
        o.close()
    except Exception as exc:
        cpu = {"error": repr(exc)}
    peak, _ = peaks()
    achieved = LAND_BYTES_PER_ELEM * ne / (ms * 1e-3) / 1e9
    return {"metric": "land-surface element-steps/s", "unit": "element-steps/s", "value": value,
            "ms_per_step": ms,
            "workload": f"{ne} elements, 64 meteorological stations, 8 LAI series, {LAND_STEPS} steps of 900 s",
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "alg_bytes_per_elem": LAND_BYTES_PER_ELEM},
            "cpu_baseline": cpu}


def bench_solve(ws, hours):
    """A solve on the headline 1M-element mesh (the c1 configuration's solve):
    from RelaxIc, 60 s model steps with hourly synthetic forcing, the
    integrator over device N_Vectors with the right-hand side on the device
    (pihm_gpu.single.GpuWatershed through pihm_gpu.solver.run_steps, the
    reference's model-step loop).  Wall time on the host clock around the
    whole solve."""
    import numpy as np
    import torch
    import pihm_gpu.watershed as W
    from pihm_gpu import workloads as WL
    from pihm_gpu.single import GpuWatershed
    from pihm_gpu.solver import StepControl, run_steps
    nsteps = int(hours * 60)
    pcp, edir, ett = WL.step_forcing(ws, nsteps, 60.0, seed=8)
    m = GpuWatershed(ws, W.relax_state(ws), pcp, edir, ett)
    m.g.set_diagnostics(False)
    outlet = int(np.where(np.asarray(ws.arrays["down"]) < 0)[0][0])
    torch.cuda.synchronize()
    t = time.perf_counter()
    r = run_steps(m, StepControl(), nsteps, m.set_forcing, outlet=outlet, record_every=nsteps)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t
    # the right-hand side's own device time in a repeat of the first model
    # steps with per-kernel events (not part of the timed solve)
    rhs_ms = None
    try:
        m2 = GpuWatershed(ws, W.relax_state(ws), pcp, edir, ett)
        m2.g.set_diagnostics(False)
        m2.g.set_profiling(True)
        k2 = min(nsteps, 10)
        r2 = run_steps(m2, StepControl(), k2, m2.set_forcing)
        kt = m2.g.kernel_times()
        rhs_ms = {"model_steps": k2, "rhs_evals": int(r2["stats"].nfe + r2["stats"].nfes),
                  "kernel_ms": {k: v[0] for k, v in kt.items()}}
        m2.close()
    except Exception as exc:
        rhs_ms = {"error": repr(exc)}
    m.close()
    st = r["stats"]
    evals = int(st.nfe + st.nfes)
    # GMRES scalars on the device (the default) against the plain iteration
    # that reads every norm, dot product and status back: the first model
    # steps of the same solve both ways, host clock
    gmres = None
    try:
        k3 = min(nsteps, 10)
        runs = {}
        for mode in (-1, 0):
            m3 = GpuWatershed(ws, W.relax_state(ws), pcp, edir, ett)
            m3.g.set_diagnostics(False)
            torch.cuda.synchronize()
            t = time.perf_counter()
            r3 = run_steps(m3, StepControl(), k3, m3.set_forcing, record_every=k3, deferred_scalars=mode)
            torch.cuda.synchronize()
            runs[mode] = (time.perf_counter() - t, r3)
            m3.close()
        (td, rd), (tp, rp) = runs[-1], runs[0]
        gmres = {"model_steps": k3, "integrator_steps": int(rd["stats"].nst), "gmres_iters": int(rd["stats"].nli),
                 "device_scalars_s": td, "plain_s": tp, "speedup": tp / td,
                 "bit_identical": bool(np.array_equal(rd["states"], rp["states"])),
                 "mode": int(rd["deferred_scalars"])}
    except Exception as exc:
        gmres = {"error": repr(exc)}
    # the same solve as a batch of one in the batch engine (each round's
    # vector operations fused per watershed, bit-identical to the plain path)
    engine = None
    try:
        from pihm_gpu.batch import Batch, limits_for
        b = Batch(limits_for([ws], nsteps))
        torch.cuda.synchronize()
        t = time.perf_counter()
        i = b.add(ws, W.relax_state(ws), StepControl(), pcp, edir, ett, outlet=outlet)
        b.step()
        res = b.result(i)
        torch.cuda.synchronize()
        ewall = time.perf_counter() - t
        b.close()
        engine = {"wall_s": ewall, "value": ws.nelem * evals / ewall,
                  "bit_identical_to_plain_path": bool(np.array_equal(res["y"], r["states"][-1]) and
                                                      np.array_equal(res["outlet"], r["outlet"]))}
    except Exception as exc:
        engine = {"error": repr(exc)}
    # the CPU restatements on the host cores (OpenMP right-hand side, the same
    # integrator over host vectors) on the first model step of the same solve
    cpu = None
    try:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from backends import OracleBackend
        k1 = 1
        m1 = GpuWatershed(ws, W.relax_state(ws), pcp, edir, ett)
        m1.g.set_diagnostics(False)
        torch.cuda.synchronize()
        t = time.perf_counter()
        r1 = run_steps(m1, StepControl(), k1, m1.set_forcing)
        torch.cuda.synchronize()
        g1 = time.perf_counter() - t
        m1.close()
        ob = OracleBackend(ws, W.relax_state(ws), pcp, edir, ett, omp=True)
        t = time.perf_counter()
        rc1 = run_steps(ob, StepControl(), k1, ob.set_forcing)
        c1 = time.perf_counter() - t
        ob.close()
        cpu = {"scope": "a sample: the first model step of the solve on both paths, not the whole solve",
               "sample": f"the first model step ({int(rc1['stats'].nst)} integrator steps, "
                         f"{int(rc1['stats'].nfe + rc1['stats'].nfes)} evaluations)",
               "cpu_s": c1, "gpu_s": g1, "speedup": c1 / g1, "cores": os.cpu_count(), "kind": "port",
               "same_step_count": int(rc1["stats"].nst) == int(r1["stats"].nst)}
    except Exception as exc:
        cpu = {"error": repr(exc)}
    return {"metric": "solve: RHS element-evals/s inside the solve", "unit": "elem-evals/s",
            "value": ws.nelem * evals / wall, "batch_engine": engine, "rhs_device_time": rhs_ms,
            "gmres_scalars": gmres,
            "cpu_baseline": cpu,
            "workload": f"{ws.nelem} elements, {ws.nriver} segments, {nsteps} model steps of 60 s "
                        f"({hours} simulated hours) from RelaxIc, hourly synthetic forcing, reltol 1e-4",
            "wall_s": wall, "simulated_hours_per_wall_hour": hours * 3600.0 / wall,
            "integrator_steps": int(st.nst), "rhs_evals": evals, "newton_iters": int(st.nni),
            "linear_iters": int(st.nli), "final_outlet_flux": float(r["outlet"][-1])}


def bench_serving():
    """Poisson stream of calibration requests at SERVE_LOAD of measured capacity."""
    import numpy as np
    import torch
    from pihm_gpu import workloads as WL
    from pihm_gpu.batch import DONE, Batch, limits_for_memory
    from pihm_gpu.single import solve_alone
    t = time.perf_counter()
    cases = WL.make_cases(WL.serving_specs(SERVE_N, SERVE_LO, SERVE_HI, SERVE_STEPS))
    gen_s = time.perf_counter() - t

    def limits():
        # the largest arena in the memory budget: admission is gated by it
        lim = limits_for_memory(SERVE_ARENA_BYTES, rivers_per_elem=0.1, edges_per_elem=1.6,
                                records_per_elem=0.0, max_systems=SERVE_MAX_REQ)
        lim.max_record = SERVE_N * SERVE_STEPS
        return lim

    def serve(arrivals):
        torch.cuda.synchronize()
        b = Batch(limits())
        tk = [b.submit(c["ws"], c["y0"], c["ctrl"], c["pcp"], c["edir"], c["ett"], arrival=float(a),
                       outlet=c["outlet"]) for c, a in zip(cases, arrivals)]
        b.serve(workers=8)
        recs = [b.record(k) for k in tk]
        out = [b.served(k) for k in tk]
        inf = b.info()
        b.close()
        return recs, out, inf

    # capacity: everything queued at t = 0
    recs, _, _ = serve(np.zeros(SERVE_N))
    makespan = max(r.t_done for r in recs)
    mu = SERVE_N / makespan
    # the open-loop run
    arr = WL.poisson_arrivals(SERVE_N, SERVE_LOAD * mu)
    recs, out, inf = serve(arr)
    failed = sum(r.status != DONE for r in recs)
    lat = np.array([r.t_done - r.t_arrival for r in recs if r.status == DONE])
    span = max(r.t_done for r in recs)
    # the plain path one request at a time, first come first served
    service, same = [], 0
    for c, o in zip(cases, out):
        ts = time.perf_counter()
        r = solve_alone(c)
        service.append(time.perf_counter() - ts)
        same += int(np.array_equal(r["y"], o["y"]) and np.array_equal(r["outlet"], o["outlet"]))
    seq_lat, seq_end = WL.fifo_latencies(arr, service)
    return {
        "metric": "served solves/s", "unit": "solves/s", "value": SERVE_N / span,
        "p50_s": _pct(lat, 50), "p99_s": _pct(lat, 99), "mean_s": float(lat.mean()),
        "workload": f"{SERVE_N} requests, {SERVE_LO}..{SERVE_HI} elements (log-uniform), Ksat x U(0.3,3), "
                    f"Manning n x U(0.5,2), model step of 30, 60, 90, 120 or 180 s, {SERVE_STEPS} model steps each, "
                    f"Poisson arrivals at {SERVE_LOAD} of the measured capacity {mu:.2f} solves/s",
        "arena_elements": int(limits().max_elem), "arena_bytes": SERVE_ARENA_BYTES,
        "admission": "by the arena's device-memory budget (pihm_batch_limits_for_memory)",
        "rounds": inf.rounds, "generate_s": gen_s,
        "sequential": {"value": SERVE_N / seq_end, "unit": "solves/s", "p50_s": _pct(seq_lat, 50),
                       "p99_s": _pct(seq_lat, 99), "service_s_total": float(sum(service)),
                       "note": "plain path, one request at a time, first come first served, same arrivals"},
        "bit_identical_to_plain_path": f"{same}/{SERVE_N}", "failed": failed,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--nelem", type=int, default=NELEM, help="smaller meshes for profiling only")
    ap.add_argument("--nriver", type=int, default=NRIVER)
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-watersheds leg")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving leg")
    ap.add_argument("--no-flux", action="store_true", help="skip the Flux-PIHM leg")
    ap.add_argument("--no-land", action="store_true", help="skip the land-surface leg")
    ap.add_argument("--no-scattered", action="store_true", help="skip the scattered-node mesh leg")
    ap.add_argument("--contexts", type=int, default=RHS_CONTEXTS, choices=[1, 2, 3, 4],
                    help="contexts of the mesh the states are spread over")
    ap.add_argument("--shape", type=int, default=1, choices=[0, 1, 2],
                    help="k_elem_main block shape of the headline contexts: 512x2, 256x4, 128x8 per SM")
    ap.add_argument("--solve-hours", type=float, default=0.5,
                    help="simulated hours of the 1M-element solve leg (0 skips it)")
    args = ap.parse_args()
    globals()["NELEM"], globals()["NRIVER"] = args.nelem, args.nriver
    if args.impl == "reference":
        return run_reference_arm(args)

    import numpy as np
    import torch
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    import pihm_gpu.watershed as W
    from pihm_gpu import workloads as WL
    from pihm_gpu.capi import GpuRhs
    t_setup = time.perf_counter()
    ws = W.generate(NELEM, NRIVER, seed=WL.RHS_SEED)
    stream = torch.cuda.Stream(device=dev)
    g = GpuRhs(ws, stream=stream.cuda_stream)
    g.set_forcing(*WL.rhs_forcing(ws))
    base = WL.rhs_base_state(ws)
    g.set_ws0_surf(base[:ws.nelem])
    # the state set, made on the host (the reference arm evaluates the same
    # arrays) and moved once into HBM in internal order
    with torch.cuda.stream(stream):
        states = torch.empty((NSTATES, ws.neq), dtype=torch.float64, device=dev)
        stage = torch.empty(ws.neq, dtype=torch.float64, device=dev)
        for k in range(NSTATES):
            stage.copy_(torch.from_numpy(WL.rhs_state(base, k)))
            g.to_internal(stage.data_ptr(), states[k].data_ptr())
        ydot = torch.empty((YDOT_RING, ws.neq), dtype=torch.float64, device=dev)
        del stage
    stream.synchronize()
    # RHS_CONTEXTS contexts of the mesh, each on its own stream, take the
    # states in turn: independent evaluations fill each other's kernel tails
    # and launch gaps (1: 2.62, 2: 3.16, 3: 3.23, 4: 3.19 G element-evals/s
    # measured), and in the pipelined end-to-end leg each context's copies
    # run under the others' kernels (2: 1.39-2.45, 3: 2.56, 4: 2.64 G)
    streams = [stream] + [torch.cuda.Stream(device=dev) for _ in range(args.contexts - 1)]
    ctxs = [g]
    for st in streams[1:]:
        gx = GpuRhs(ws, stream=st.cuda_stream)
        gx.set_forcing(*WL.rhs_forcing(ws))
        gx.set_ws0_surf(base[:ws.nelem])
        ctxs.append(gx)
    for c in ctxs:
        c.set_kernel_shape(args.shape)
    setup_s = time.perf_counter() - t_setup

    def step(s):
        # ydot ring slots e % YDOT_RING: the ring is a multiple of the context
        # count, so each context keeps to its own slots
        for e in range(STATES_PER_STEP):
            k = (s * STATES_PER_STEP + e) % NSTATES
            ctxs[e % len(ctxs)].rhs_device(states[k].data_ptr(), ydot[e % YDOT_RING].data_ptr())

    def sync_all():
        for st in streams:
            st.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---- device-resident throughput ----
    for s in range(args.warmup):
        step(s)
    sync_all()
    assert all(c.status() == 0 for c in ctxs), "NaN in warm-up evaluations"
    ev0 = torch.cuda.Event(enable_timing=True)
    ev_end = [torch.cuda.Event(enable_timing=True) for _ in streams]
    launches0 = sum(c.launch_count() for c in ctxs)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for st in streams[1:]:
            st.wait_event(ev0)
        for s in range(args.steps):
            step(args.warmup + s)
        for e, st in zip(ev_end, streams):
            e.record(st)
        for e in ev_end:
            e.synchronize()
    barrier()
    torch.cuda.synchronize()
    launches = sum(c.launch_count() for c in ctxs) - launches0
    ms = max_over_ranks(max(ev0.elapsed_time(e) for e in ev_end), world, dev)
    evals = args.steps * STATES_PER_STEP
    value = replica_throughput(world, NELEM * evals, ms)
    ms_per_eval = ms / evals
    assert all(c.status() == 0 for c in ctxs), "NaN in timed evaluations"

    # ---- per-kernel device time (separate pass, events around each kernel) ----
    g.set_profiling(True)
    step(0)
    kt = g.kernel_times()
    g.set_profiling(False)
    tot = sum(v[0] for v in kt.values())
    kernels = {k: {"ms_per_call": v[0] / v[1], "share": v[0] / tot} for k, v in kt.items()}
    dominant = max(kernels, key=lambda k: kernels[k]["share"])

    # ---- end to end through the host-buffer C-ABI call ----
    # one step (every state once) per host path; the states in pinned host
    # memory in reference order, the derivatives into a ring of pinned buffers
    e2e_evals = STATES_PER_STEP
    y_host = torch.empty((NSTATES, ws.neq), dtype=torch.float64, pin_memory=True)
    for k in range(NSTATES):
        y_host[k].copy_(torch.from_numpy(WL.rhs_state(base, k)))
    yd_host = torch.empty((YDOT_RING, ws.neq), dtype=torch.float64, pin_memory=True)
    import ctypes
    f64p = ctypes.POINTER(ctypes.c_double)
    lib = g.lib
    def e2e_one(k):
        rc = lib.pihm_gpu_rhs_host(g.h, 0.0, ctypes.cast(y_host[k].data_ptr(), f64p),
                                   ctypes.cast(yd_host[k % YDOT_RING].data_ptr(), f64p))
        assert rc == 0, rc
    def time_e2e(mode):
        # mode 0: the library default (direct host access where possible),
        # 1: copies through device staging
        g.set_host_path(mode)
        for k in range(2):
            e2e_one(k)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        for k in range(e2e_evals):
            e2e_one(k % NSTATES)
        e1.record(stream)
        e1.synchronize()
        ms_ = max_over_ranks(e0.elapsed_time(e1), world, dev)
        return replica_throughput(world, NELEM * e2e_evals, ms_)
    e2e_copy_value = time_e2e(1)
    e2e_value = time_e2e(0)
    direct, pageable = g.host_path_info()
    # pipelined: the contexts of the mesh, each on its own stream, take the
    # states in turn through pihm_gpu_rhs_host_async / pihm_gpu_wait, so one
    # evaluation's host-link transfers run beside the others' kernels
    # (independent evaluations: an ensemble, not a CVODE
    # sequence); same copies, same host buffers, host clock
    pipelined = None
    try:
        nc = len(ctxs)

        def submit(k):
            c = ctxs[k % nc]
            rc = lib.pihm_gpu_rhs_host_async(c.h, 0.0, ctypes.cast(y_host[k % NSTATES].data_ptr(), f64p),
                                             ctypes.cast(yd_host[k % YDOT_RING].data_ptr(), f64p))
            assert rc == 0, rc

        def run(n, depth):
            # up to depth evaluations queued per context: pihm_gpu_wait
            # drains one context while the others' queues keep the device busy
            queued = [0] * nc
            for k in range(n):
                c = k % nc
                if queued[c] >= depth:
                    assert lib.pihm_gpu_wait(ctxs[c].h) == 0
                    queued[c] = 0
                submit(k)
                queued[c] += 1
            for c in ctxs:
                assert lib.pihm_gpu_wait(c.h) == 0
        by_path = {}
        for mode, name in ((0, "direct"), (1, "copy")):
            # direct: the kernels read and write host memory (SM time on the
            # link); copy: each context's copy streams move it, beside the
            # other contexts' kernels.  Each path is timed with one and with
            # PIPE_DEPTH evaluations queued per context (a wait drains a
            # whole context, so the best depth depends on the path)
            for c in ctxs:
                c.set_host_path(mode)
            for depth in (1, PIPE_DEPTH):
                run(2 * nc, depth)
                reps = []
                for _ in range(E2E_REPS):
                    barrier()
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    run(e2e_evals, depth)
                    torch.cuda.synchronize()
                    ms_p = max_over_ranks((time.perf_counter() - t0) * 1e3, world, dev)
                    reps.append(replica_throughput(world, NELEM * e2e_evals, ms_p))
                by_path[f"{name}, depth {depth}"] = statistics.median(reps)
        g.set_host_path(0)
        best = max(by_path, key=by_path.get)
        pipelined = {"value": by_path[best], "unit": UNIT, "contexts": nc, "best": best,
                     "statistic": f"median of {E2E_REPS} passes of {e2e_evals} evaluations per configuration",
                     "by_host_path_and_depth": by_path,
                     "evals": e2e_evals, "api": "pihm_gpu_rhs_host_async + pihm_gpu_wait, host clock"}
    except Exception as exc:
        pipelined = {"error": repr(exc)}
    # the headline e2e: the faster way through the C ABI for these 100
    # independent states, every copy of every state inside the timed region
    e2e_best, e2e_mode = e2e_value, "sync: pihm_gpu_rhs_host, one evaluation at a time"
    if pipelined and "value" in pipelined and pipelined["value"] > e2e_value:
        e2e_best = pipelined["value"]
        e2e_mode = (f"pipelined: pihm_gpu_rhs_host_async on {pipelined['contexts']} contexts of the mesh, "
                    f"{pipelined['best']} queued per context")
    host_path = ("direct: k_elem_prep reads y from and the reordering kernel writes ydot to pinned host memory"
                 if direct else "copy through device staging") + (
                 "; the device can access pageable host memory" if pageable else "")
    bytes_state = ws.neq * 8

    # ---- roofline of one right-hand-side evaluation ----
    peak, peak_kind = peaks()
    alg_bytes = NELEM * BYTES_PER_ELEM + NRIVER * BYTES_PER_SEG
    achieved = alg_bytes / (ms_per_eval * 1e-3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "rhs_traffic.json")
    if os.path.exists(tp):
        try:
            traffic = json.load(open(tp)).get("dram_bytes_per_eval")
        except Exception:
            traffic = None
    # The FP64 pipe, not HBM, bounds these kernels: GB300 retires 2 FP64
    # lanes per clock per SM, so one warp-wide FP64 instruction holds it for
    # 16 cycles.  The per-evaluation FP64 instruction counts come from an ncu
    # capture (profiles/rhs_fp64.json); the time and clock are this run's.
    fp64 = None
    fp = os.path.join(ROOT, "profiles", "rhs_fp64.json")
    if os.path.exists(fp) and NELEM == 1_000_000 and NRIVER == 30_000:
        try:
            cnt = json.load(open(fp))
            sm_mhz = clk.summary().get("sm_mhz") or 2070.0
            peak_slots = torch.cuda.get_device_properties(dev).multi_processor_count * 2 * sm_mhz * 1e6
            slots = cnt["fp64_warp_instr_per_eval"] * 32 / (ms_per_eval * 1e-3)
            lanes = cnt["fp64_lane_ops_per_eval"] / (ms_per_eval * 1e-3)
            fp64 = {"achieved": slots / 1e9, "peak": peak_slots / 1e9, "unit": "G FP64 lane slots/s",
                    "frac": slots / peak_slots, "useful_frac": lanes / peak_slots,
                    "sm_mhz": sm_mhz, "counts": "profiles/rhs_fp64.json",
                    "note": "frac: FP64 pipe busy over the evaluation; useful_frac: predicated-on lanes only"}
        except Exception as exc:
            fp64 = {"error": repr(exc)}

    # ---- CPU baseline (rank 0, N = 1 only) ----
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        state_of = lambda k: WL.rhs_state(base, k)  # noqa: E731
        try:
            n, el, thr = cpu_time_oracle(ws, state_of, os.cpu_count() or 1)
            cpu = dict({"value": NELEM * n / el, "unit": UNIT, "cores": thr, "kind": "port",
                        "sample": f"{n} RHS evaluations of the {NELEM}-element mesh (the benchmark's first "
                                  f"states, in order), {el:.1f} s wall, OpenMP restatement of the reference ODE()"},
                       **host_cores())
        except Exception as exc:  # the baseline is reported, never required
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"failed: {exc}"}
        try:
            n1, el1, _ = cpu_time_oracle(ws, state_of, 1, omp=False, max_seconds=8.0)
            cpu["serial"] = {"value": NELEM * n1 / el1, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": f"{n1} RHS evaluations, {el1:.1f} s wall, 1-thread build of the restatement"}
        except Exception as exc:
            cpu["serial"] = {"error": repr(exc)}

    # ---- batched watersheds and serving (N = 1 only) ----
    batched = serving = flux = land = solve = scattered = None
    if rank == 0 and world == 1:
        for c in ctxs:
            c.close()
        if not args.no_scattered:
            try:
                scattered = bench_scattered()
            except Exception as exc:
                scattered = {"error": repr(exc)}
        if args.solve_hours > 0:
            try:
                solve = bench_solve(ws, args.solve_hours)
            except Exception as exc:
                solve = {"error": repr(exc)}
        if not args.no_land:
            try:
                land = bench_land(ws)
            except Exception as exc:
                land = {"error": repr(exc)}
        if not args.no_batched:
            try:
                batched = bench_batched()
            except Exception as exc:
                batched = {"error": repr(exc)}
        if not args.no_serving:
            try:
                serving = bench_serving()
            except Exception as exc:
                serving = {"error": repr(exc)}
        if not args.no_flux:
            try:
                flux = bench_flux_pihm()
            except Exception as exc:
                flux = {"error": repr(exc)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": workload_config(world),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "peak_kind": peak_kind, "scope": "one RHS evaluation (all its kernels)",
                         "alg_bytes_per_eval": alg_bytes, "ms_per_eval": ms_per_eval,
                         "limit": "FP64 pipe (see fp64_pipe), not HBM", "fp64_pipe": fp64},
            "kernels": kernels, "dominant_kernel": dominant,
            "rhs_contexts": {"count": len(ctxs), "k_elem_main_shape": ("512x2", "256x4", "128x8")[args.shape], "note": "the states are spread round-robin over contexts of the "
                             "mesh on their own streams; kernels and their shares are one context's"},
            "e2e": {"value": e2e_best, "unit": UNIT, "h2d_bytes_per_step": bytes_state * STATES_PER_STEP,
                    "d2h_bytes_per_step": bytes_state * STATES_PER_STEP, "evals": e2e_evals, "mode": e2e_mode,
                    "sync_value": e2e_value, "host_path": host_path, "copy_path_value": e2e_copy_value,
                    "pipelined": pipelined},
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "cpu_baseline": cpu,
            "setup_s": setup_s,
            "batched": batched,
            "serving": serving,
            "flux_pihm": flux,
            "land_surface": land,
            "solve": solve,
            "scattered_mesh": scattered,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
