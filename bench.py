"""Throughput of the MPCD + active-colloid step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--precision fp64|fp32c]

Workload (the 64^3 single system): 64^3 cells, fluid density 10 (2,621,440
particles, Maxwell-Boltzmann at kT=1, zero net momentum), 500 colloids of radius
2 (diameter 4) with the displaced-fluid mass, WCA sigma=4 eps=1, v0=0.01,
Dr=0.001, SRD angle 90 deg, MPCD step 0.1 with 10 MD substeps.  Synthetic
initial state from the library's own keyed initialiser (seed 0 + rank).

One step = one MPCD step (rotation_mpcd, run, 10 substeps) over the whole system.
value = fluid particle-steps/s with the state resident in HBM (CUDA graph per
step, CUDA events on the library's stream).  e2e = the same metric through the
public API from pinned host buffers: upload of the state, setup, K steps each
followed by a device->host read of the step's diagnostics, download of the final
state.  roofline: the dominant kernel (the fluid streaming pass) timed per launch
with CUDA events over a second timed region, against its algorithmic bytes
(72 B per particle: read position and displacement, write position).

Multi-GPU: one independent replica per rank (different seed), no collective
in the data path ("scaling": "weak").

--impl reference: the reference's CPU step on the host cores, one single-threaded process
per core on a bounded sample: its own cpp/ routines (oracle/_ref/ref_harness) where they
were compiled from the reference sources, else the oracle's restatement of cpp/.
"""
import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L, DENSITY, NC, RADIUS = 64, 10, 500, 2.0
# Algorithmic bytes per particle.  The free-flight schedule (steps without a counting sort):
# the free-flight pass reads every particle's near flag (1 B) and moves a free particle
# through the step: FP64 reads x, w (48 B) and writes x and its next cell (28 B); FP32 reads
# the cell+offset record and the velocity (28 B) and writes the record and the cell (20 B).
FREE_BYTES = {"fp64": 76, "fp32c": 48}
# one MPCD step in that schedule, with a fraction f of near particles (density 10, per-cell
# data per particle):
#   FP64: rotation + classification 77 (rotcell 4, w 24 read and 24 written, x 24, flag 1)
#         + SRD map 9.6 + flight table 3.2; free pass 1 + 76 (1 - f); cell pass 13.6 and the
#         binning's cell sums 4; near passes 10 x 77 f (index 4, x and w 48, pending mark 1,
#         x written 24) + near binning 57 f + list 4 f
#   FP32: rotation + classification 45 (rotcell 4, v 12 read and 12 written, record 16, flag 1)
#         + map 4.8 + table 3.2; free pass 1 + 48 (1 - f); cell pass 8.8, cell sums 4; near
#         passes 10 x 48 f (index 4, record 16 read and written, velocity 12) + 4 f + list 4 f
#   (the near binning of the FP32 form is part of its last near pass)
#   (with n substeps the near passes count n times: b = 77 n - 15 and 48 (n - 1) + 8)
STEP_BYTES_FLIGHT = {"fp64": 184.4, "fp32c": 114.8}


def step_bytes(precision, near_frac, n_sub=10):
    b = 77.0 * n_sub - 15.0 if precision == "fp64" else 48.0 * (n_sub - 1) + 8.0
    return STEP_BYTES_FLIGHT[precision] + b * near_frac


def workload(seed=0):
    import numpy as np
    M = DENSITY * 4.0 / 3.0 * np.pi * RADIUS ** 3
    return dict(L=L, n_fluid=L ** 3 * DENSITY, n_colloid=NC,
                kw=dict(n_sub=10, ndt=0.1, kbt=1.0, kbt1=1.0, mass_fl=1.0, mass_colloid=M, sig_colloid=4.0,
                        eps=1.0, sigma=2 * RADIUS, I_colloid=0.4 * M * RADIUS ** 2, v0=0.01, theta_deg=90.0,
                        Dr=0.001, seed=seed, init_gap=0.5))


def config_dict(precision):
    return {"workload": "MPCD 64^3 cells, density 10 (2,621,440 fluid particles), 500 colloids r=2, "
                        "10 MD substeps per MPCD step",
            "box": [L, L, L], "n_fluid": L ** 3 * DENSITY, "n_colloid": NC, "n_sub": 10, "precision": precision,
            "l2": "state (>190 MB) larger than the 129 MB L2; no flush between steps",
            "init": "library keyed initialiser, Maxwell-Boltzmann, seed = rank"}


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self):
        self.p = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def stop(self, dev=0):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9 or f[0] != str(dev):
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic_per_particle(precision):
    """DRAM bytes per fluid particle of one free-flight launch from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(p) as f:
            return float(json.load(f)[f"k_free_flight_{precision}"]["dram_bytes_per_particle"])
    except (OSError, KeyError, ValueError):
        return None


# ---------------------------------------------------------------- CPU baseline

def synthetic_state(seed, n_fluid, L_=L, nc=NC, radius=RADIUS, gap=0.5, kbt=1.0, M=None):
    """Host-built initial state with the workload's shapes and distributions:
    colloids by random sequential addition (gap >= 0.5), fluid uniform outside the
    colloids, Maxwell-Boltzmann velocities with zero net momentum, isotropic
    orientations."""
    import numpy as np
    from scipy.spatial import cKDTree
    rng = np.random.default_rng(1000 + seed)
    M = DENSITY * 4.0 / 3.0 * np.pi * radius ** 3 if M is None else M
    X = np.empty((nc, 3))
    k = 0
    while k < nc:
        t = rng.uniform(0, L_, 3)
        d = X[:k] - t
        d -= L_ * np.round(d / L_)
        if k == 0 or np.min(np.einsum("ij,ij->i", d, d)) >= (2 * radius + gap) ** 2:
            X[k] = t
            k += 1
    tree = cKDTree(X, boxsize=L_)
    pos = np.empty((0, 3))
    while len(pos) < n_fluid:
        cand = rng.uniform(0, L_, (int((n_fluid - len(pos)) * 1.2) + 16, 3))
        dist, _ = tree.query(cand)
        pos = np.concatenate([pos, cand[dist >= radius]])
    pos = pos[:n_fluid]
    vel = rng.normal(0, np.sqrt(kbt), (n_fluid, 3))
    vel -= vel.mean(0)
    V = rng.normal(0, np.sqrt(kbt / M), (nc, 3))
    V -= V.mean(0)
    W = rng.normal(0, np.sqrt(kbt / (0.4 * M * radius ** 2)), (nc, 3))
    ra = rng.normal(size=(nc, 3))
    ra /= np.linalg.norm(ra, axis=1)[:, None]
    return dict(pos_fl=pos, vel_fl=vel, pos_colloid=X, vel_colloid=V, ang_vel_colloid=W, ra=ra)


def _cpu_worker(args):
    """Time `steps` oracle steps of the workload on one core (separate process)."""
    seed, steps, n_fluid_sample = args
    from oracle import oracle as O
    w = workload(seed)
    o = O.Oracle(L=w["L"], n_fluid=n_fluid_sample, n_colloid=w["n_colloid"], rng_mode=O.RNG_KEYED,
                 **{k: v for k, v in w["kw"].items() if k != "init_gap"})
    for k, v in synthetic_state(seed, n_fluid_sample).items():
        o.set(k, v)
    o.setup()
    o.step()  # warm
    t0 = time.perf_counter()
    o.run_steps(steps)
    dt = time.perf_counter() - t0
    o.close()
    return n_fluid_sample * steps / dt


HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def reference_available():
    """The reference's own cpp/ routines, compiled where the reference sources are (the
    oracle Makefile's `ref` target); absent where the sources are not."""
    return os.path.isfile(HARNESS) and os.access(HARNESS, os.X_OK)


def reference_baseline(processes, steps, n_fluid, tmp="/tmp"):
    """The stock reference step loop (oracle/_ref/ref_harness time mode): `processes`
    independent single-threaded runs at once, each `steps` MPCD steps of the workload from a
    synthetic state (seed = process), after the prologue and one untimed step."""
    import numpy as np
    w = workload(0)
    kw = w["kw"]
    procs = []
    for q in range(processes):
        st = synthetic_state(q, n_fluid)
        path = os.path.join(tmp, f"bgb_ref_state_{os.getpid()}_{q}.bin")
        with open(path, "wb") as f:
            for k in ("pos_fl", "vel_fl", "pos_colloid", "vel_colloid", "ang_vel_colloid"):
                np.ascontiguousarray(st[k], dtype=np.float64).tofile(f)
        args = [HARNESS, "time", str(w["L"]), str(n_fluid), str(w["n_colloid"]), str(kw["n_sub"]), repr(kw["ndt"]),
                repr(kw["kbt"]), repr(kw["kbt1"]), repr(kw["mass_fl"]), repr(kw["mass_colloid"]),
                repr(kw["sig_colloid"]), repr(kw["eps"]), repr(kw["sigma"]), repr(kw["I_colloid"]), repr(kw["v0"]),
                "77777", str(steps), path]
        procs.append((subprocess.Popen(args, stdout=subprocess.PIPE, text=True), path))
    rates = []
    for pr, path in procs:
        out, _ = pr.communicate()
        os.remove(path)
        if pr.returncode != 0:
            raise RuntimeError(f"ref_harness exited {pr.returncode}")
        rates.append(json.loads(out.strip().splitlines()[-1])["particle_steps_per_s"])
    return sum(rates), rates


def cpu_baseline(processes, steps, n_fluid):
    ctx = mp.get_context("spawn")
    with ctx.Pool(processes) as pool:
        rates = pool.map(_cpu_worker, [(s, steps, n_fluid) for s in range(processes)])
    return sum(rates), rates


# ---------------------------------------------------------------- our arm

def _barrier(dist):
    import torch
    if torch.cuda.is_available():
        torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()


def _max_over_ranks(x, dist):
    """The largest of the ranks' x (a time: the job's time is its slowest rank's)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(world, units_per_rank, steps, seconds):
    """Whole-job throughput: the units every rank processed (replicas: each rank runs its own
    system, so the work grows with the ranks) over the slowest rank's time."""
    return world * units_per_rank * steps / seconds


def make_sim(precision, rank):
    import torch

    import brownian_gb300 as bg
    w = workload(seed=rank)
    sim = bg.Simulation(w["L"], w["n_fluid"], w["n_colloid"],
                        precision=bg.FP64 if precision == "fp64" else bg.FP32C, **w["kw"])
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    sim.initialize(bg.INIT_PHYSICAL)
    sim.setup()
    return sim, stream


def measure_resident(sim, stream, precision, args, world, dist, with_clocks=True):
    """Timed region A (graph replay, state resident) and B (per-kernel CUDA events)."""
    import torch
    N = sim.N
    sim.step(args.warmup)  # also captures the step graphs
    _barrier(dist)
    clocks = Clocks()
    if with_clocks:
        clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = sim.launch_count
    e0.record(stream)
    sim.step(args.steps)
    e1.record(stream)
    _barrier(dist)
    clk = clocks.stop(int(os.environ.get("LOCAL_RANK", "0"))) if with_clocks else None
    ms = _max_over_ranks(e0.elapsed_time(e1), dist)
    gpu_launches = sim.launch_count - launches0
    value = aggregate_rate(world, N, args.steps, ms / 1e3)
    # B: the same steps, each kernel bracketed by CUDA events on the library's stream
    sim.profile(True)
    _barrier(dist)
    sim.step(args.steps)
    _barrier(dist)
    prof = sim.profile_read()
    sim.profile(False)
    near = sim.flight_near()
    f = near / N
    ff_launches, ff_ms = prof.get("k_free_flight", (0, 0.0))
    t_launch = ff_ms / max(ff_launches, 1) / 1e3
    alg = N * (1.0 + (1.0 - f) * FREE_BYTES[precision])
    achieved = alg / t_launch / 1e9 if ff_launches else None
    peak, peak_kind = measured_peak_hbm()
    tpp = ncu_traffic_per_particle(precision)
    total = sum(x[1] for x in prof.values())
    shares = {k: {"share": round(v[1] / total, 4), "launches": v[0], "us_per_launch": round(v[1] / v[0] * 1e3, 2)}
              for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])}
    roof = {"bound": "hbm",
            "kernel": "k_free_flight (the free particles' whole step: streaming and binning; the largest fluid pass, "
                      "run beside the substeps' latency-bound chain, which sets the step time)",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
            "traffic": (tpp * N) if tpp else None, "algorithmic_bytes": alg,
            "peak_source": f"{peak_kind} hbm_gbs (burst copy)", "launch_ms": t_launch * 1e3,
            "launches": ff_launches}
    sb = step_bytes(precision, f)
    return dict(value=value, ms=ms, gpu_launches=gpu_launches, clocks=clk, roofline=roof, shares=shares,
                step_frac=value / world * sb / (peak * 1e9), near=near, near_frac=f, step_bytes=sb)


def form_statistics(replicas, steps, lag=100, every=10):
    """Both precision forms on the 64^3 workload, `replicas` independent systems each (seeds
    100 + r, the same initial state for both forms), `steps` steps per system: per system the
    colloid MSD at `lag` steps (unwrapped positions in a device trajectory, a frame every
    `every` steps, averaged over colloids and time origins), the mean fluid temperature and
    the largest momentum change relative to sum |p|.  The forms are compared through the
    means over systems, with standard errors from the spread between systems (independent)."""
    import numpy as np

    import brownian_gb300 as bg
    per = {}
    for prec in ("fp64", "fp32c"):
        rows = []
        for r in range(replicas):
            w = workload(seed=100 + r)
            sim = bg.Simulation(w["L"], w["n_fluid"], w["n_colloid"],
                                precision=bg.FP64 if prec == "fp64" else bg.FP32C, **w["kw"])
            sim.initialize(bg.INIT_PHYSICAL)
            sim.setup()
            d0 = sim.diag()
            tr = bg.Trajectory(sim.Nc, steps // every + 1, L)
            tr.record(sim)
            temps, drift = [], 0.0
            for s in range(steps // every):
                sim.step(every)
                tr.record(sim)
                if (s + 1) % 10 == 0:
                    d = sim.diag()
                    temps.append(d["temperature_fluid"])
                    drift = max(drift, float(np.max(np.abs(np.array(d["momentum"]) - np.array(d0["momentum"])))))
            msd = float(tr.analyse(msd_lags=(lag // every,), vacf_lags=(0,), oacf_lags=(0,))["msd"][0])
            tr.close()
            scale = sim.N * np.sqrt(8.0 / np.pi)  # sum |p_i| of a thermal fluid (m = kT = 1)
            rows.append((msd, float(np.mean(temps)), drift / scale))
            sim.close()
        a = np.array(rows)
        n = len(a)
        per[prec] = {"msd": float(a[:, 0].mean()), "msd_stderr": float(a[:, 0].std(ddof=1) / np.sqrt(n)),
                     "temperature": float(a[:, 1].mean()), "temperature_stderr": float(a[:, 1].std(ddof=1) / np.sqrt(n)),
                     "momentum_drift_rel_mean": float(a[:, 2].mean()), "momentum_drift_rel_max": float(a[:, 2].max())}
    a, b = per["fp64"], per["fp32c"]
    return {"replicas": replicas, "steps": steps, "msd_lag_steps": lag, "frame_every": every,
            "workload": "64^3, 2,621,440 fluid particles, 500 colloids; replica r from the library initialiser, seed "
                        "100 + r, the same initial state for both forms",
            "fp64": a, "fp32c": b,
            "msd_rel_diff": (b["msd"] - a["msd"]) / a["msd"],
            "msd_rel_diff_stderr": float(np.hypot(a["msd_stderr"], b["msd_stderr"]) / a["msd"]),
            "temperature_diff": b["temperature"] - a["temperature"],
            "temperature_diff_stderr": float(np.hypot(a["temperature_stderr"], b["temperature_stderr"])),
            "momentum_drift_rel_fp64": a["momentum_drift_rel_max"],
            "momentum_drift_rel_fp32c": b["momentum_drift_rel_max"]}


def ensemble_params(nrep, seed=0):
    """The batched-ensemble workload: box sizes uniform over {16, 24, 32, 40, 48}^3, fluid
    density 10, colloid count uniform in [5, 200] capped at 10 % volume fraction, radius 2,
    v0 uniform in [0, 0.1], Dr = 0.001, distinct seeds, FP32-compensated form."""
    import numpy as np

    import brownian_gb300 as bg
    rng = np.random.default_rng(seed)
    out = []
    M = bg.displaced_mass(RADIUS, DENSITY)
    for i in range(nrep):
        Lr = int(rng.choice([16, 24, 32, 40, 48]))
        cap = int(0.1 * Lr ** 3 / (4.0 / 3.0 * np.pi * RADIUS ** 3))
        nc = int(min(rng.integers(5, 201), cap))
        out.append(bg.make_params(Lr, Lr ** 3 * DENSITY, nc, n_sub=10, mass_colloid=M, sig_colloid=2 * RADIUS,
                                  sigma=2 * RADIUS, I_colloid=0.4 * M * RADIUS ** 2, v0=float(rng.uniform(0, 0.1)),
                                  theta_deg=90.0, Dr=0.001, seed=1000 * (seed + 1) + i, precision=bg.FP32C))
    return out


def run_ensemble(nrep, steps, rank):
    """Replica-steps/s of the batched ensemble (autotuned launch shapes) against looping
    the single-system step over the same replicas."""
    import torch

    import brownian_gb300 as bg
    from brownian_gb300.tune import autotune
    P = ensemble_params(nrep, seed=rank)
    ens = bg.Ensemble(P)
    for s in ens:
        s.initialize(bg.INIT_PHYSICAL)
        s.setup()
    tuned = autotune(ens, steps=2)

    def batched(flight):
        ens.set_flight(flight)
        ens.step(2)
        t0 = time.perf_counter()
        ens.step(steps)
        return time.perf_counter() - t0

    # the batched step in the free-flight schedule (the default), then in the per-substep one
    batched_s = batched(True)
    l0 = ens.launch_count
    ens.step(1)
    launches_per_step = ens.launch_count - l0 - 1  # minus the error read-back
    batched_sub_s = batched(False)
    # the same replicas, each stepped by its own single-system call, one after the other:
    # each replica's step graph enqueued back to back on one stream, one synchronisation
    # per sweep over the replicas (a replica's next step needs its previous one only)
    # First with the batched kernels' schedule (every particle through every substep), so
    # that the ratio is the batching alone; then with the single-system free-flight schedule
    st = torch.cuda.Stream()

    def looped(flight):
        for s in ens:
            s.set_stream(st.cuda_stream)
            s.set_flight(flight)
            s.step(1)
        t0 = time.perf_counter()
        for _ in range(steps):
            for s in ens:
                s.step_async(1)
            ens[0].sync()
        for s in ens:
            s.sync()  # every replica's device checks
        return time.perf_counter() - t0

    looped_s = looped(False)
    looped_flight_s = looped(True)
    n_particles = sum(p.n_fluid for p in P)
    ens.close()
    return {"workload": "256 replicas" if nrep == 256 else f"{nrep} replicas",
            "replicas": nrep, "fluid_particles": n_particles, "steps": steps,
            "value": nrep * steps / batched_s, "unit": "replica-steps/s",
            "schedule": "free flight (mpcd_ensemble_set_flight(1), the default)",
            "particle_steps_per_s": n_particles * steps / batched_s,
            "per_substep": {"value": nrep * steps / batched_sub_s, "unit": "replica-steps/s",
                            "how": "the batched step with one pass over every particle per substep "
                                   "(mpcd_ensemble_set_flight(0))"},
            # against the faster of the two looped arms
            "speedup_vs_looped": min(looped_s, looped_flight_s) / batched_s,
            "looped": {"value": nrep * steps / looped_s, "unit": "replica-steps/s",
                       "how": "mpcd_step_async(1) of each replica in turn on one stream, one "
                              "synchronisation per sweep over the replicas; the single-system per-substep "
                              "schedule (mpcd_set_flight(0))"},
            "speedup_vs_looped_per_substep": looped_s / batched_s,
            "looped_free_flight": {"value": nrep * steps / looped_flight_s, "unit": "replica-steps/s",
                                   "how": "the same loop with the single-system free-flight schedule"},
            "speedup_vs_looped_free_flight": looped_flight_s / batched_s,
            "speedup_per_substep_schedules": looped_s / batched_sub_s,
            "launches_per_step": launches_per_step,
            "autotune": {"choice": tuned["choice"], "ms_per_step": tuned["ms_per_step"],
                         "trials": len(tuned["log"])},
            "timing": "wall clock around mpcd_ensemble_step(K) (it ends with a device synchronisation)"}


def run_large(steps, warmup=3):
    """The large single system: 128^3 cells, density 10 (20,971,520 fluid particles), 2,000
    colloids of radius 3 (mass of the displaced fluid, WCA sigma 6), v0 = 0.02, Dr = 0.0005,
    SRD angle 130 degrees, 20 MD substeps, FP32 form with the FP64 diagnostics.  Particle-steps/s
    from CUDA events around graph replays; per kernel its time per launch (profiled steps) and,
    for the fluid passes, the fraction of the measured copy bandwidth their algorithmic bytes
    reach."""
    import numpy as np
    import torch

    import brownian_gb300 as bg
    L3, NC3, R3, NSUB = 128, 2000, 3.0, 20
    M = DENSITY * 4.0 / 3.0 * np.pi * R3 ** 3
    N = L3 ** 3 * DENSITY
    sim = bg.Simulation(L3, N, NC3, precision=bg.FP32C, n_sub=NSUB, ndt=0.1, kbt=1.0, kbt1=1.0, mass_fl=1.0,
                        mass_colloid=M, sig_colloid=2 * R3, eps=1.0, sigma=2 * R3, I_colloid=0.4 * M * R3 ** 2,
                        v0=0.02, theta_deg=130.0, Dr=0.0005, seed=0, init_gap=0.5)
    st = torch.cuda.Stream()
    sim.set_stream(st.cuda_stream)
    sim.initialize(bg.INIT_PHYSICAL)
    sim.setup()
    sim.step(warmup)
    d0 = sim.diag()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    sim.step(steps)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    d1 = sim.diag()
    near_frac = sim.flight_near() / N
    sim.profile(True)
    sim.step(2)
    prof = sim.profile_read()
    sim.profile(False)
    peak = measured_peak_hbm()[0]
    # algorithmic bytes per fluid particle, FP32 form (the free-flight pass: the flag of every
    # particle and the free particles' record, velocity, record and cell; the cell pass: 88 B per
    # cell at density 10; a near pass: index, record read and written, velocity of the near
    # particles)
    per_particle = {"k_stream": 44, "k_rotate": 28, "k_rotate_sort": 64, "k_rotate_classify": 45,
                    "k_free_flight": 1.0 + (1.0 - near_frac) * FREE_BYTES["fp32c"], "k_cell_prep": 8.8,
                    "k_stream_near": 48.0 * near_frac}
    kernels = {}
    for k, (n, tms) in sorted(prof.items(), key=lambda kv: -kv[1][1]):
        us = tms / max(n, 1) * 1e3
        row = {"launches_per_step": n / 2, "us_per_launch": us, "share": tms / sum(v[1] for v in prof.values())}
        if k in per_particle:
            gbs = per_particle[k] * N / (us * 1e-6) / 1e9
            row.update({"algorithmic_bytes_per_particle": per_particle[k], "achieved_gbs": gbs,
                        "frac_of_measured_copy": gbs / peak})
        kernels[k] = row
    sim.close()
    b_step = step_bytes("fp32c", near_frac, NSUB)
    ps = N / (ms / 1e3)
    return {"workload": "128^3 cells, density 10 (20,971,520 fluid particles), 2000 colloids r=3 (WCA sigma 6), "
                        "v0 0.02, Dr 0.0005, SRD angle 130 deg, 20 substeps; FP32 form",
            "steps": steps, "warmup": warmup, "ms_per_step": ms, "value": ps, "unit": "particle-steps/s",
            "hbm_roofline_frac_step": b_step * ps / (peak * 1e9), "bytes_per_particle_step": b_step,
            "near_fraction": near_frac,
            "peak_gbs": peak, "kernels": kernels,
            "diag": {"temperature": d1["temperature_fluid"],
                     # total momentum change over the timed steps, relative to sum |p_i| of a thermal fluid
                     "momentum_drift_rel": float(np.max(np.abs(np.array(d1["momentum"]) - np.array(d0["momentum"])))
                                                 / (N * np.sqrt(8.0 / np.pi)))}}


def _speed_row(row, p, net, closure, bg, _t):
    """Time per MPCD step of full MPCD (FP64 and FP32 forms) and of the colloid-only step
    from the full run's colloid state, into row."""
    c0 = None
    for prec, name in ((bg.FP64, "full_fp64"), (bg.FP32C, "full_fp32c")):
        p.precision = prec
        full = closure._sim(p)
        full.initialize(bg.INIT_PHYSICAL)
        full.setup()
        full.step(3)
        t0 = _t.perf_counter()
        full.step(10)
        row[name + "_ms"] = (_t.perf_counter() - t0) / 10 * 1e3
        if c0 is None:
            c0 = full.get_colloids()
        full.close()
    sur = closure.Surrogate(p, net)
    sur.set_state(c0["pos_colloid"], c0["vel_colloid"], c0["ang_vel_colloid"], c0["ra"])
    sur.step(5)
    t0 = _t.perf_counter()
    sur.step(200)
    row["surrogate_ms"] = (_t.perf_counter() - t0) / 200 * 1e3
    sur.close()
    row["speedup_vs_fp64"] = row["full_fp64_ms"] / row["surrogate_ms"]
    row["speedup_vs_fp32c"] = row["full_fp32c_ms"] / row["surrogate_ms"]
    row["colloid_time_per_wall_s"] = {"surrogate": 0.1 / (row["surrogate_ms"] / 1e3),
                                      "full_fp64": 0.1 / (row["full_fp64_ms"] / 1e3),
                                      "full_fp32c": 0.1 / (row["full_fp32c_ms"] / 1e3)}


def run_closure(samples_steps, deploy_steps):
    """The learned closure: training samples from full MPCD of the 64^3 system with v0 swept
    over [0, 0.1] (500 colloids x 5 activities x samples_steps steps), GPU training, then
    colloid-only runs against full MPCD (the yardstick) on a 500-colloid system at volume
    fraction 0.1, and the time per MPCD step of both at 500 and 2000 colloids."""
    import time as _t

    import numpy as np

    import brownian_gb300 as bg
    from brownian_gb300 import closure
    M = bg.displaced_mass(RADIUS, DENSITY)

    def P(Lr, nc, v0, seed):
        return bg.make_params(Lr, Lr ** 3 * DENSITY, nc, n_sub=10, mass_colloid=M, sig_colloid=2 * RADIUS,
                              sigma=2 * RADIUS, I_colloid=0.4 * M * RADIUS ** 2, v0=v0, theta_deg=90.0, Dr=0.001,
                              seed=seed, precision=bg.FP32C)
    t0 = _t.perf_counter()
    X, Y = closure.generate_gpu([P(L, NC, v0, 500 + i) for i, v0 in enumerate((0.0, 0.025, 0.05, 0.075, 0.1))],
                                steps=samples_steps)
    t_data = _t.perf_counter() - t0
    rng = np.random.default_rng(0)
    perm = rng.permutation(X.shape[0])
    X, Y = X[perm], Y[perm]
    cut = int(0.95 * X.shape[0])
    net = closure.Network(max_batch=8192, seed=0)
    net.fit_normalisation(X[:cut], Y[:cut])
    t0 = _t.perf_counter()
    losses = closure.train(net, X[:cut], Y[:cut], epochs=12, batch=8192, lr=3e-4)
    t_train = _t.perf_counter() - t0
    held = closure.nll(net, X[cut:], Y[cut:])
    free = closure.free_nll(Y[:cut], Y[cut:])
    L500 = int(round((500 * 4.0 / 3.0 * np.pi * RADIUS ** 3 / 0.1) ** (1.0 / 3.0)))
    res = closure.compare(P(L500, 500, 0.05, 901), net, steps=deploy_steps)
    # colloid time per wall-second across the deployment range (500 and 2000 colloids,
    # volume fraction 0.05-0.2): full MPCD, the plain FP64 form and the FP32 form, against
    # the colloid-only step started from the full run's colloid state
    table = []
    for i, (nc, phi) in enumerate(((500, 0.1), (500, 0.05), (2000, 0.2), (2000, 0.1), (2000, 0.05))):
        Lr = int(round((nc * 4.0 / 3.0 * np.pi * RADIUS ** 3 / phi) ** (1.0 / 3.0)))
        row = {"colloids": nc, "volume_fraction": phi, "L": Lr, "fluid_particles": Lr ** 3 * DENSITY}
        try:
            _speed_row(row, P(Lr, nc, 0.05, 910 + i), net, closure, bg, _t)
        except Exception as e:  # a row that fails is reported, the others still run
            row["error"] = str(e)
        table.append(row)
    net.close()
    return {"workload": "closure trained on 64^3 / 500 colloids, v0 in {0, .025, .05, .075, .1}; deployed on "
                        f"{L500}^3 / 500 colloids (volume fraction 0.1, v0 = 0.05) against full MPCD",
            "samples": int(X.shape[0]), "data_s": t_data, "train_s": t_train, "epochs": len(losses),
            "train_loss_first_last": [losses[0], losses[-1]],
            "heldout_nll": held, "heldout_nll_without_network": free,
            "speed": table,
            "speedup_500_vs_fp32c_in_comparison_run": res["speedup"],
            "deploy_steps": deploy_steps, "blocks": res["blocks"], "lags": res["lags"],
            "rel_diff_vs_full": res["rel_diff_vs_full"], "rel_diff_stderr": res["rel_diff_stderr"],
            "fast_steps": res["fast_steps"],
            "stats": res["stats"],
            "timing": "wall clock around step calls (each ends with a synchronisation); full MPCD 10 steps after 3, "
                      "the colloid-only step 200 after 5"}


def run_ours(args, rank, world, dist):
    import torch

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    forms = [args.precision] + [p for p in ("fp64", "fp32c") if p != args.precision and args.both]
    res = {}
    for prec in forms:
        sim, stream = make_sim(prec, rank)
        res[prec] = measure_resident(sim, stream, prec, args, world, dist, with_clocks=(prec == args.precision))
        if prec == args.precision:
            head_sim = sim
        else:
            sim.close()
    sim = head_sim
    N = sim.N
    r = res[args.precision]

    # ---- timed region C: end to end through the public API from pinned host buffers
    host = sim.get_state()
    pinned = {k: torch.from_numpy(v).pin_memory().numpy() for k, v in host.items()}
    out = {k: torch.empty(v.shape, dtype=torch.float64).pin_memory().numpy() for k, v in host.items()}
    _barrier(dist)
    t0 = time.perf_counter()
    sim.set_state(pinned["pos_fl"], pinned["vel_fl"], pinned["pos_colloid"], pinned["vel_colloid"],
                  pinned["ang_vel_colloid"], pinned["ra"])
    sim.setup()
    for _ in range(args.steps):
        # the step enqueued, then its diagnostics read back: one round trip per step, which
        # also reports the step's device error bits (mpcd_diag checks them)
        sim.step_async(1)
        dd = sim.diag()
    sim.get_state(out=out)  # into the page-locked host buffers
    _barrier(dist)
    e2e_s = _max_over_ranks(time.perf_counter() - t0, dist)
    state_bytes = sum(v.nbytes for k, v in host.items() if k != "f")
    diag_bytes = 8 * 14
    e2e = {"value": aggregate_rate(world, N, args.steps, e2e_s), "unit": "particle-steps/s",
           "h2d_bytes_per_step": state_bytes / args.steps,
           "d2h_bytes_per_step": (state_bytes + host["f"].nbytes) / args.steps + diag_bytes,
           "timed": "set_state + setup + K x (mpcd_step_async + mpcd_diag, one round trip per step, the "
                    "step's error bits checked by the diag) + get_state, host pinned buffers"}
    d = sim.diag()
    sim.close()
    stats = (form_statistics(args.stat_replicas, args.stat_steps)
             if (args.both and args.stat_steps > 100 and args.stat_replicas > 1 and rank == 0) else None)
    ens = run_ensemble(args.ensemble, args.ensemble_steps, rank) if args.ensemble > 0 else None
    large = run_large(args.large_steps) if (args.large_steps > 0 and rank == 0) else None
    clo = run_closure(args.closure_steps, 2000) if (args.closure_steps > 0 and rank == 0) else None

    if rank != 0:
        return None
    line = {
        "metric": "MPCD fluid particle-steps/s", "value": r["value"], "unit": "particle-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic",
        "config": dict(config_dict(args.precision), parallelism=f"replicas x{world}"),
        "hbm_roofline_frac_step": r["step_frac"],
        "step_bytes_per_particle": r["step_bytes"],
        "near_fraction": r["near_frac"],
        "roofline": r["roofline"],
        "kernel_share": r["shares"],
        "e2e": e2e,
        "gpu_launches": r["gpu_launches"],
        "clocks": r["clocks"],
        "diag_end": {"temperature_fluid": d["temperature_fluid"], "momentum": d["momentum"],
                     "wall_events_per_substep": dd["events"] / 10.0, "run_candidates": dd["shell_records"]},
    }
    for prec in forms[1:]:
        o = res[prec]
        line[f"form_{prec}"] = {"value": o["value"], "unit": "particle-steps/s", "ms_per_step": o["ms"] / args.steps,
                                "speedup_vs_" + args.precision: o["value"] / r["value"],
                                "hbm_roofline_frac_step": o["step_frac"], "step_bytes_per_particle": o["step_bytes"],
                                "near_fraction": o["near_frac"], "roofline": o["roofline"],
                                "kernel_share": o["shares"], "gpu_launches": o["gpu_launches"]}
    if stats:
        line["fp32c_vs_fp64"] = stats
    if ens:
        line["ensemble"] = ens
    if clo:
        line["closure"] = clo
    if large is not None and rank == 0:
        line["large"] = large
    return line


def ensemble_demo(nrep, steps):
    """`nrep` replicas of the ensemble workload, `steps` batched free-flight steps with the
    default launch shapes (one graph per step; for launch lists)."""
    import brownian_gb300 as bg
    ens = bg.Ensemble(ensemble_params(nrep))
    for s in ens:
        s.initialize(bg.INIT_PHYSICAL)
        s.setup()
    ens.step(steps)
    print("ok", nrep, "replicas", steps, "steps", ens.launch_count, "launches")
    ens.close()


def trace_steps(warmup):
    """One traced step of each form on the headline workload, after `warmup` steps: every
    launch's start and end (us from the step's start) on the graph's own timeline, in order of
    start (a traced step runs 20-30 % slower than an untraced one; its shape is the step's)."""
    for precision in ("fp64", "fp32c"):
        sim, _ = make_sim(precision, 0)
        sim.step(max(warmup, 1))
        sim.trace_step()
        tr = sim.trace_step()
        print("== %s: %d launches, step %.1f us (traced)" % (precision, len(tr), max(t for _, _, t in tr) * 1e3))
        for name, a, b in sorted(tr, key=lambda x: x[1]):
            print("%-22s %8.1f %8.1f %7.1f" % (name, a * 1e3, b * 1e3, (b - a) * 1e3))
        sim.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32c"], help="form of the headline line")
    ap.add_argument("--both", type=int, default=1, help="also time the other precision form (sub-object)")
    ap.add_argument("--stat-steps", type=int, default=2000,
                    help="steps per system of the FP32c-vs-FP64 statistics (MSD at lag 100; <=100: skip)")
    ap.add_argument("--stat-replicas", type=int, default=24,
                    help="independent systems per form of the FP32c-vs-FP64 statistics (<2: skip)")
    ap.add_argument("--ensemble", type=int, default=256, help="replicas of the batched-ensemble sub-object (0: skip)")
    ap.add_argument("--ensemble-steps", type=int, default=50)
    ap.add_argument("--large-steps", type=int, default=5,
                    help="timed steps of the 128^3 / 2000-colloid FP32 system (0: skip)")
    ap.add_argument("--closure-steps", type=int, default=800,
                    help="steps per activity of the closure's training runs (500 colloids each; 0: skip)")
    ap.add_argument("--cpu-steps", type=int, default=3, help="oracle steps timed for cpu_baseline (0: skip)")
    ap.add_argument("--cpu-sample", type=int, default=0, help="fluid particles in the CPU sample (0: full 64^3 system)")
    ap.add_argument("--trace", action="store_true",
                    help="instead of the bench line: the timeline of one step of each form (mpcd_trace_step)")
    ap.add_argument("--ensemble-demo", type=int, default=0,
                    help="instead of the bench line: this many replicas of the ensemble workload stepped "
                         "--steps times with the default launch shapes (profiling)")
    args = ap.parse_args()
    if args.trace:
        trace_steps(args.warmup)
        return
    if args.ensemble_demo > 0:
        ensemble_demo(args.ensemble_demo, args.steps)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    n_full = L ** 3 * DENSITY
    sample_n = args.cpu_sample or n_full

    if args.impl == "reference":
        if rank != 0:
            return
        procs = os.cpu_count() or 1
        total = 0.0
        t0 = time.perf_counter()
        # each timed worker process does its own untimed warm-up step
        if reference_available():
            # the reference's own cpp/ routines (compiled from its sources where they are present)
            rate, rates = reference_baseline(procs, args.steps, sample_n)
            kind, what = "reference", "the reference's own cpp/ step loop (oracle/_ref/ref_harness)"
        else:
            # where the reference sources are absent: the oracle's restatement of cpp/, pinned bit
            # for bit to the reference's traces
            rate, rates = cpu_baseline(procs, args.steps, sample_n)
            kind, what = "port", "the oracle's restatement of cpp/ (the reference's sources are not on this machine)"
        wall = time.perf_counter() - t0
        line = {"impl": "reference", "metric": "MPCD fluid particle-steps/s", "value": rate,
                "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": dict(config_dict("fp64"), parallelism=f"{procs} CPU processes"),
                "cpu_baseline": {"value": rate, "unit": "particle-steps/s", "cores": procs, "kind": kind,
                                 "sample": f"{procs} independent single-threaded processes of {what}, each "
                                           f"{args.steps} MPCD steps of the 64^3 system with {sample_n} fluid "
                                           f"particles, after one untimed step; wall {wall:.1f} s"},
                "e2e": {"value": rate, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    # CPU baseline of our arm: start the oracle process before any GPU call (spawn)
    cpu = None
    if rank == 0 and args.cpu_steps > 0:
        t0 = time.perf_counter()
        rate, _ = cpu_baseline(1, args.cpu_steps, sample_n)
        cpu = {"value": rate, "unit": "particle-steps/s", "cores": 1, "kind": "port",
               "sample": f"one single-threaded oracle process (restatement of cpp/), {args.cpu_steps} MPCD steps of "
                         f"the 64^3 system with {sample_n} fluid particles after one warm-up step "
                         f"({time.perf_counter() - t0:.1f} s wall incl. set-up)"}
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    line = run_ours(args, rank, world, dist)
    if line is not None:
        line["cpu_baseline"] = cpu
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
