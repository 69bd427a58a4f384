"""Benchmark: timesteps/s of the xcore.jl time step at 1024^2 on GB300.

One "step" is one outer time step of run! (src/run.jl:204-274): store_previous!,
store_noise!, three Picard sweeps of phsevo! -> fluidmech! -> noise! ->
update_phase_velocities! -> update! -> compute_resnorm, then update_dt.
Workload: 1024x1024 grid, crystal fraction seeded lognormal (median 0.1,
sigma 0.5, clipped to [0, 0.4]), etacntr 1e4, WENO5, BD2, Stokes solved to
relative residual 1e-9 with the mixed FP32/FP64 solver; the plain FP64 GPU
solve (FGMRES to 1e-9) is timed beside it for the speed-up the metric names.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun each rank runs an independent replica (the path does not shard
across GPUs) and rank 0 prints one JSON line.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "timesteps/s at 1024², learned+mixed vs plain FP64 GPU at Stokes rel-res 1e-9"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--N", type=int, default=1024)
    ap.add_argument("--sweeps", type=int, default=3)
    ap.add_argument("--solver", default="mixed", choices=["mixed", "fgmres64"])
    ap.add_argument("--learned", type=int, default=-1,
                    help="preconditioner of the mixed solver's FP32 inner solves: 0 multigrid, 1 the learned "
                         "network in its place (multigrid fallback), 2 the network after the V-cycle; -1 "
                         "(default): the learned mode the committed weights record as best, 0 without weights")
    ap.add_argument("--weights", default=None, help="learned preconditioner parameters (.npz)")
    ap.add_argument("--rtol", type=float, default=1e-9)
    ap.add_argument("--ensemble", type=int, default=0,
                    help="time an ensemble of this many independent instances instead (grid sides drawn from "
                         "64..512, per-member noise seed, amplitude and initial crystal fraction; member-steps/s)")
    ap.add_argument("--ensemble-graphs", action="store_true",
                    help="with --ensemble: one CUDA graph launch per explicit stage for all members "
                         "(xc_ensemble_step) instead of one host thread per member")
    ap.add_argument("--weno-weights", type=int, default=1, choices=[0, 1],
                    help="WENO5 weights: 0 the reference's four-division form (bit for bit), 1 over a common "
                         "denominator (one division per reconstruction; within the 1e-12 stencil tolerance, "
                         "measured 2%% faster per step)")
    ap.add_argument("--plain-steps", type=int, default=None,
                    help="time steps of the plain FP64 comparison loop (default: --steps, the same steps)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--roofline-kernel", type=int, default=2)
    ap.add_argument("--knob", action="append", default=[],
                    help="extra solver option key=value for the timed solves (e.g. pressure_sweeps=2)")
    ap.add_argument("--profile-kernel", type=int, default=None,
                    help="initialise, run the warm-up steps, then launch only this kernel (xc_bench_kernel "
                         "index) 3 times inside the NVTX range 'xc_profile' and exit (for ncu)")
    return ap.parse_args()


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def workload_params(N):
    """Parameters of the 1024^2 mixed-precision configuration (L0 = l0 = 3h)."""
    import xcore_gb300 as xc
    D = 10.0
    h = D / N
    return xc.Parameters(D=D, N=N, L=D, etam0=10.0, x0=0.1, Da=0.0, L0=3 * h, l0=3 * h, etacntr=1e4,
                         ADVN="weno5", TINT="bd2im")


def initial_fields(N, seed=0):
    rng = np.random.default_rng(seed)
    x0 = np.clip(np.exp(np.log(0.1) + 0.5 * rng.standard_normal((N, N))), 0.0, 0.4)
    return x0, rng


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        if self.proc is None or not getattr(self, "out", ""):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_port_step_seconds(N, sweeps=3, steps=1, seed=0):
    """Seconds per time step of the CPU oracle port (numpy stencils + SciPy
    SuperLU Stokes solve), measured on this host."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import xcore_oracle as O
    D = 10.0
    h = D / N
    par = O.Params(D=D, N=N, L=D, etam0=10.0, x0=0.1, Da=0.0, L0=3 * h, l0=3 * h, etacntr=1e4, ADVN="weno5",
                   TINT="bd2im")
    g = O.make_grid(par)
    sc = O.compute_scales(par, g)
    ns = O.NoiseStatic(g, sc)
    x0, rng = initial_fields(N, seed)
    st = O.initialize(g, par, sc, ns, x0, rng.standard_normal((N, N)), rng.standard_normal((N, N)))
    dt = sc["dt0"]
    times = []
    for step in range(1, steps + 1):
        re, rs = rng.standard_normal((N, N)), rng.standard_normal((N, N))
        t0 = time.perf_counter()
        dt, _ = O.timestep(st, g, par, sc, ns, step, dt, re, rs, sweeps=sweeps)
        times.append(time.perf_counter() - t0)
    return times


CPU_GRID = 128   # largest grid whose sparse-LU steps fit a few-minute run on the host


def cpu_note(N):
    return (f"measured at {N}^2, not at the GPU workload's grid: the port's sparse LU (SciPy SuperLU) grows "
            f"much faster than the cell count (about 10 s per factorisation at 256^2 and 100 s at 400^2 on an "
            f"x86 core), so a 1024^2 CPU step is not measured and no cell-count extrapolation is reported")


def run_reference(a):
    """--impl reference: the CPU port of the reference path on the host cores,
    real time steps of the same workload at CPU_GRID^2."""
    rank, world, _ = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        if rank != 0:
            dist.barrier()
            return
    N = CPU_GRID
    times = cpu_port_step_seconds(N, a.sweeps, steps=a.warmup + a.steps)[a.warmup:]
    per_step = float(np.mean(times))
    value = 1.0 / per_step
    sample = (f"{a.steps} timed {a.sweeps}-sweep time steps at {N}^2 after {a.warmup} warm-up steps, "
              f"{per_step:.2f} s each; " + cpu_note(N))
    out = {"metric": METRIC, "value": value, "unit": "timesteps/s", "n_gpus": a.gpus, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
           "config": {"workload": f"xcore time step {N}x{N}, {a.sweeps} Picard sweeps, WENO5, BD2, "
                                  "lognormal crystal fraction, etacntr 1e4",
                      "grid": f"{N}x{N}", "sweeps": a.sweeps,
                      "gpu_workload_grid": f"{a.N}x{a.N} (CPU steps at that grid unmeasured)",
                      "implementation": "CPU port of the reference path: numpy stencils + SciPy SuperLU "
                                        "(the Julia reference and UMFPACK are not installed); both are "
                                        "single-threaded, so one core does the work"},
           "cpu_baseline": {"value": value, "unit": "timesteps/s", "cores": 1, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": "timesteps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def gpu_steps_per_second(xc, N, sweeps, steps, sopt, seed=5, weno_weights=0):
    """Timesteps/s of the GPU path on the same workload at N^2 (the CPU
    baseline's grid), CUDA events on the library stream, after 3 warm-up steps."""
    import torch
    par = workload_params(N)
    st = xc.State(par, weno_weights=weno_weights)
    x0, rng = initial_fields(N, seed)
    st.initialize(x0, rng.standard_normal((N, N)), rng.standard_normal((N, N)))
    stream = torch.cuda.ExternalStream(st.stream_handle())
    dt = st.scales["dt0"]
    total = 0.0
    for k in range(3 + steps):
        re, rs = rng.standard_normal((N, N)), rng.standard_normal((N, N))
        st["re"], st["rs"] = re, rs
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        info = st.step(k + 1, dt, None, None, sweeps=sweeps, **sopt)
        e1.record(stream)
        e1.synchronize()
        if k >= 3:
            total += e0.elapsed_time(e1)
        dt = info["dt_next"]
    st.close()
    return 1e3 * steps / total


def run_ensemble(a):
    """member-steps/s of xcore_gb300.Ensemble (one context and stream per
    member; one host thread per member, or with --ensemble-graphs one graph
    launch per explicit stage for all members) on instances of the
    batched-ensemble configuration:
    grid sides drawn from {64, 128, 192, 256, 384, 512}, each member with its
    own noise seed, noise amplitude Xi in [1e-4, 1e-2] and uniform initial
    crystal fraction in [0.02, 0.2]; 3 Picard sweeps, mixed Stokes to 1e-9."""
    import torch
    import xcore_gb300 as xc
    xc.build()
    rng = np.random.default_rng(42)
    sides = rng.choice([64, 128, 192, 256, 384, 512], size=a.ensemble)
    members, dts, gens = [], [], []
    for q, N in enumerate(sides):
        N = int(N)
        D = 10.0
        h = D / N
        par = xc.Parameters(D=D, N=N, L=D, etam0=10.0, x0=0.1, Da=0.0, L0=3 * h, l0=3 * h, etacntr=1e4,
                            ADVN="weno5", TINT="bd2im", Xi=float(10 ** rng.uniform(-4, -2)))
        st = xc.State(par, weno_weights=a.weno_weights)
        g = np.random.default_rng(1000 + q)
        x0 = np.full((N, N), g.uniform(0.02, 0.2))
        st.initialize(x0, g.standard_normal((N, N)), g.standard_normal((N, N)))
        members.append(st)
        dts.append(st.scales["dt0"])
        gens.append(g)
    ens = xc.Ensemble(members, graphs=a.ensemble_graphs)
    solver = dict(solver="mixed", rtol=1e-9, maxit=400, inner_rtol=5e-2, inner_maxit=30, pressure_sweeps=1)

    def step(k):
        draws = [(g.standard_normal((m.grid.Nz, m.grid.Nx)), g.standard_normal((m.grid.Nz, m.grid.Nx)))
                 for m, g in zip(members, gens)]
        infos = ens.step([k] * len(members), dts, draws, **solver)
        for q, i in enumerate(infos):
            dts[q] = i["dt_next"]
    for k in range(a.warmup):
        step(k + 1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(a.steps):
        step(a.warmup + k + 1)
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    cells = float(sum(int(N) * int(N) for N in sides))
    out = {"metric": "member-steps/s of an uneven ensemble (3 Picard sweeps, mixed Stokes to 1e-9)",
           "value": a.ensemble * a.steps / sec, "unit": "member-steps/s", "n_gpus": 1, "steps": a.steps,
           "warmup": a.warmup, "ms_per_ensemble_step": 1e3 * sec / a.steps, "higher_is_better": True,
           "cell_steps_per_s": cells * a.steps / sec, "dtype": "f64+f32", "data": "synthetic",
           "config": {"workload": f"{a.ensemble} instances, sides {sorted(set(int(s) for s in sides))}",
                      "members_per_side": {str(int(s)): int((sides == s).sum()) for s in sorted(set(sides))},
                      "implementation": ("one device context and CUDA stream per member; every explicit stage one "
                                         "CUDA graph launch for all members, the Stokes solves on one host thread "
                                         "per member" if a.ensemble_graphs else
                                         "one device context, CUDA stream and host thread per member"),
                      "timing": "host wall clock over the K ensemble steps (host draws included)"}}
    print(json.dumps(out), flush=True)
    ens.close()


def main():
    a = parse()
    if a.ensemble > 0:
        return run_ensemble(a)
    if a.plain_steps is None:
        a.plain_steps = a.steps
    if a.impl == "reference":
        return run_reference(a)
    import torch
    import xcore_gb300 as xc

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    xc.build()
    N = a.N
    par = workload_params(N)
    st = xc.State(par, weno_weights=a.weno_weights)
    x0, rng = initial_fields(N, seed=1234 + rank)
    # every timed loop replays draws k0, k0 + 1, ... of the same saved state
    nstep_total = a.warmup + max(a.steps, a.plain_steps)
    # white-noise draws for every step, in pinned host memory laid out column-major
    draws = []
    for _ in range(nstep_total + 1):
        pair = []
        for _ in range(2):
            t = torch.empty((N, N), dtype=torch.float64).pin_memory()
            t.copy_(torch.from_numpy(rng.standard_normal((N, N))))
            pair.append(t.numpy().T)   # F-contiguous [z, x] view of the pinned buffer
        draws.append(pair)
    st.initialize(x0, draws[0][0], draws[0][1])
    sopt = dict(solver=a.solver, rtol=a.rtol, maxit=400, inner_rtol=5e-2, inner_maxit=30, pressure_sweeps=1)
    # the learned preconditioner (committed weights, trained by xcore.jl_gb300/learned.py)
    import xcore_gb300.learned as learned_mod
    wpath = a.weights or learned_mod.WEIGHTS
    learned_info = {"weights": None, "mode": 0}
    if a.solver == "mixed" and os.path.exists(wpath) and a.learned != 0:
        with np.load(wpath) as z:
            best = int(z["best_mode"]) if "best_mode" in z.files else 2
            for key in z.files:
                if key != "params" and z[key].ndim == 0:
                    v = z[key].item()
                    learned_info[key] = v if not isinstance(v, float) or math.isfinite(v) else None
        mode = best if a.learned < 0 else a.learned
        if mode > 0:
            learned_mod.use(st, learned_mod.load_params(wpath))
            sopt["learned"] = mode
        learned_info["weights"] = os.path.relpath(wpath, ROOT)
        learned_info["mode"] = mode
    for kv in a.knob:
        key, val = kv.split("=", 1)
        sopt[key] = float(val) if any(ch in val for ch in ".e") else int(val)
    dt = st.scales["dt0"]
    step = 0
    k = 1
    for _ in range(a.warmup):
        step += 1
        info = st.step(step, dt, draws[k][0], draws[k][1], sweeps=a.sweeps, **sopt)
        dt = info["dt_next"]
        k += 1
    if a.profile_kernel is not None:
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("xc_profile")
        st.bench_kernel(a.profile_kernel, iters=2)
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        print(json.dumps({"profiled_kernel": a.profile_kernel, "N": N}), flush=True)
        return
    stream = torch.cuda.ExternalStream(st.stream_handle())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    # Both timed loops below run the same K steps of the same trajectory: the
    # state is saved here and restored before the end-to-end loop, and both use
    # draws k, k+1, ... -- same work, same iteration counts, same bits.
    snap = st.checkpoint()
    step0, dt0, k0 = step, dt, k
    # ---- device-resident: each step's draws uploaded to the device before its
    # timed interval (CUDA events on the library stream around each step) ------------
    iters, resid = 0, 0.0
    intervals = []
    barrier()
    launches0 = xc.launch_count()
    with ClockSampler(local) as clk:
        for _ in range(a.steps):
            step += 1
            st["re"], st["rs"] = draws[k][0], draws[k][1]
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            info = st.step(step, dt, None, None, sweeps=a.sweeps, **sopt)
            e1.record(stream)
            intervals.append((e0, e1))
            dt = info["dt_next"]
            k += 1
            iters += info["solver_iterations"]
            resid = max(resid, info["solver_rel_residual"])
        barrier()
    launches = xc.launch_count() - launches0
    ms = sum(e0.elapsed_time(e1) for e0, e1 in intervals) / a.steps
    # ---- end to end: host draws in, crystal fraction out, every step ------------------
    st.restore(snap)
    step, dt, k = step0, dt0, k0
    xout = torch.empty((N, N), dtype=torch.float64).pin_memory()
    xout_np = xout.numpy().T
    iters_e2e = 0
    barrier()
    ev0.record(stream)
    for _ in range(a.steps):
        step += 1
        info = st.step(step, dt, draws[k][0], draws[k][1], sweeps=a.sweeps, **sopt)
        dt = info["dt_next"]
        k += 1
        iters_e2e += info["solver_iterations"]
        xc.lib().xc_field_download(st._h, st._ids["x"], xout_np.ctypes.data)
    ev1.record(stream)
    barrier()
    ms_e2e = ev0.elapsed_time(ev1) / a.steps
    # ---- plain FP64 GPU drop-in on the same state -------------------------------------
    # from the same saved state with the same draws as the two loops above
    ms_plain = None
    field_err = None
    if a.plain_steps > 0:
        st.restore(snap)
        step, dt, k = step0, dt0, k0
        intervals = []
        barrier()
        for _ in range(a.plain_steps):
            step += 1
            st["re"], st["rs"] = draws[k][0], draws[k][1]
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            info = st.step(step, dt, None, None, sweeps=a.sweeps, solver="fgmres64", rtol=a.rtol, maxit=1500)
            e1.record(stream)
            intervals.append((e0, e1))
            dt = info["dt_next"]
            k += 1
        barrier()
        ms_plain = sum(e0.elapsed_time(e1) for e0, e1 in intervals) / a.plain_steps
        # the same steps with the mixed solver, untimed: per-field deviation
        # of the mixed trajectory from the plain FP64 one
        plain_fields = {f: st[f] for f in ("W", "U", "P", "x")}
        st.restore(snap)
        step, dt, k = step0, dt0, k0
        for _ in range(a.plain_steps):
            step += 1
            info = st.step(step, dt, draws[k][0], draws[k][1], sweeps=a.sweeps, **sopt)
            dt = info["dt_next"]
            k += 1
        field_err = {f: float(np.abs(st[f] - v).max() / max(np.abs(v).max(), 1e-300))
                     for f, v in plain_fields.items()}
    # ---- the learned preconditioner's modes beside the headline -------------------------
    # each mode of the committed network the headline does not use, timed on the
    # same steps from the same saved state (device-resident, as `value`)
    learned_runs = {}
    if learned_info["weights"] and a.solver == "mixed":
        if "learned" not in sopt:
            learned_mod.use(st, learned_mod.load_params(wpath))
        for mode in (1, 2):
            if sopt.get("learned", 0) == mode:
                continue
            st.restore(snap)
            step, dt, k = step0, dt0, k0
            intervals, its_l = [], 0
            barrier()
            try:
                for _ in range(a.steps):
                    step += 1
                    st["re"], st["rs"] = draws[k][0], draws[k][1]
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    info = st.step(step, dt, None, None, sweeps=a.sweeps, **dict(sopt, learned=mode))
                    e1.record(stream)
                    intervals.append((e0, e1))
                    dt = info["dt_next"]
                    its_l += info["solver_iterations"]
                    k += 1
                barrier()
                learned_runs[mode] = {"ms_per_step": sum(x.elapsed_time(y) for x, y in intervals) / a.steps,
                                      "solver_iterations_per_step": its_l / a.steps}
            except xc.XcoreError as e:
                learned_runs[mode] = {"error": str(e)}
    # ---- roofline of the dominant kernel (CUDA events on the library stream) ----------
    rk = st.bench_kernel(a.roofline_kernel, iters=20)
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    achieved = rk[1] / (rk[0] * 1e-3) / 1e9
    # DRAM bytes (read + write) per cell of one launch, measured by one ncu
    # capture of each kernel on this workload at 1024^2, scaled to this grid
    ncu_bytes_per_cell = {0: 25.23e6 / 1048576, 1: (235.73e6 + 18.77e6) / 1048576, 2: 33.64e6 / 1048576,
                          3: (185.02e6 + 11.52e6) / 1048576, 4: 8.43e6 / 1048576}
    traffic = ncu_bytes_per_cell[a.roofline_kernel] * rk[3] if a.roofline_kernel in ncu_bytes_per_cell else None
    ms_t = torch.tensor([ms, ms_e2e, ms_plain or 0.0], dtype=torch.float64, device="cuda")
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(ms_t, op=dist.ReduceOp.MAX)
    ms, ms_e2e, ms_plain_max = [float(v) for v in ms_t.cpu()]
    if rank != 0:
        barrier()
        return
    cpu = None
    gpu_at_cpu_grid = None
    if not a.no_cpu and world == 1:
        times = cpu_port_step_seconds(CPU_GRID, a.sweeps, steps=3)[1:]
        v = 1.0 / float(np.mean(times))
        cpu = {"value": v, "unit": "timesteps/s", "cores": 1, "kind": "port", "grid": f"{CPU_GRID}x{CPU_GRID}",
               "sample": f"2 timed {a.sweeps}-sweep time steps at {CPU_GRID}^2 after one warm-up step "
                         f"({np.mean(times):.2f} s each on this host; numpy + SciPy SuperLU, single-threaded); "
                         + cpu_note(CPU_GRID)}
        gpu_at_cpu_grid = gpu_steps_per_second(xc, CPU_GRID, a.sweeps, 10, sopt, weno_weights=a.weno_weights)
    names = {0: "advect_tile_kernel (WENO5, one field)", 1: "stokes_apply_kernel<double>",
             2: "vel_sweep2d_kernel<float,1> (finest-level FP32 velocity Jacobi sweep, one row per thread; operand "
                "copies exceed 2x L2)",
             5: "vel_sweep_rb_kernel<1> (finest-level FP32 velocity Jacobi sweep, four rows along z per thread; "
                "operand copies exceed 2x L2)",
             3: "vel_sweep2d_kernel<double,1> (finest-level velocity Jacobi sweep; operand copies exceed 2x L2)",
             4: "line_filter_kernel (FFT z pass)"}
    out = {
        "metric": METRIC,
        "value": world * 1e3 / ms,
        "unit": "timesteps/s",
        "n_gpus": world,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64+f32" if a.solver == "mixed" else "f64",
        "data": "synthetic: seeded lognormal crystal fraction and N(0,1) white-noise draws",
        "config": {
            "workload": f"xcore time step {N}x{N}: {a.sweeps} Picard sweeps (phsevo!, fluidmech!, noise!, "
                        f"update_phase_velocities!, update!), WENO5, BD2, etacntr 1e4, lognormal x",
            "grid": f"{N}x{N}", "sweeps": a.sweeps, "solver": a.solver, "stokes_rtol": a.rtol,
            "weno_weights": "common denominator, one division (within 1e-12)" if a.weno_weights
                            else "the reference's four-division form (bit for bit)",
            "solver_options": {k: v for k, v in sopt.items() if k not in ("solver", "rtol")},
            "solver_iterations_per_step": iters / a.steps, "worst_solver_rel_residual": resid,
            "e2e_solver_iterations_per_step": iters_e2e / a.steps,
            "timing": "value: sum of the K steps' device intervals, each step's draws uploaded before it; "
                      "e2e: one interval over the same K steps from the same saved state, draws copied in "
                      "and the crystal fraction copied out inside it",
            "plain_fp64_ms_per_step": ms_plain_max if ms_plain else None,
            "speedup_vs_plain_fp64": (ms_plain_max / ms) if ms_plain else None,
            "mixed_vs_plain_fp64_field_error": field_err,
            "field_error_note": f"max-norm relative deviation of W, U, P, x after {a.plain_steps} steps from the "
                                "same saved state: mixed solver vs the plain FP64 solver",
            "cpu_grid_gpu_timesteps_per_s": gpu_at_cpu_grid,
            "learned_preconditioner": dict(learned_info, other_modes=learned_runs),
            "cache": "working set (~2 GB of fields and solver vectors) exceeds L2 (129 MB); no flush needed",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
        },
        "e2e": {"value": world * 1e3 / ms_e2e, "unit": "timesteps/s", "h2d_bytes_per_step": 2 * 8 * N * N,
                "d2h_bytes_per_step": 8 * N * N},
        "roofline": {"kernel": names.get(a.roofline_kernel), "bound": "hbm", "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic,
                     "peak_source": "measured" if peaks else "fallback",
                     "ms_per_launch": rk[0], "algorithmic_bytes_per_launch": rk[1],
                     "algorithmic_flops_per_launch": rk[2], "units_per_launch": rk[3]},
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
    }
    print(json.dumps(out), flush=True)
    if world > 1:
        barrier()


if __name__ == "__main__":
    main()
