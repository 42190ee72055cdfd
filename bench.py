"""Benchmark: particle-steps/s of the Langevin step on one GB300.

Workload (the single large system): N = 2^20 particles at number density
0.8 in a cubic periodic box (an FCC lattice of 64^3 cells, a = (4/0.8)^(1/3),
L = 109.438), LennardJones plugin with ljNum 6, yukawaStrength 0 and
kT * wellDepth = epsilon = 1 at kT = 1.5, cutOff 2.5, Maxwell-Boltzmann
velocities at kT = 1.5, gamma = 1, dt = 0.002, cell grid 37^3 (the finest
with cellSize >= cutOff + the pair-list skin 0.4).  One step = forces -> push
-> nextSystem -> cell-list rebuild (system.cpp:187-206).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  `value` times the mixed-precision form (FP32 pairs,
Kahan sums, FP64 update) with state resident in HBM; `plain_fp64` times the
FP64 plain form on the same melted state; `force_rel_err` is the mixed form's
force error against FP64 on that state; `e2e` runs the reference-layout
drop-ins (cells_build -> force_evaluate -> nextSystem) on host buffers in
pinned memory, every copy inside the timed region.  `--impl reference` times
the CPU implementation of the path (oracle/_ref when present, else the
oracle's restatement) on the host cores.  Sub-objects of the line report the
other workloads on the same GPU: `batched` (512 AO replicas in one set of
launches), `differentiable` (the adjoint of a 2,000-step AO + Yukawa
trajectory, N = 32768), `gel` (2^23 aggregating AO colloids, with the
cell occupancy over time) and `c0` (the reference's own 4000-particle AO
case, with the CPU port beside it).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s, 1 GB300: FP32-mixed vs FP64 plain at \u22641e-5 rel force err"
UNIT = "particle-steps/s"
KT, WD, RC, LJN, DT, GAMMA = 1.5, 1.0 / 1.5, 2.5, 6, 0.002, 1.0
FLOPS_PER_PAIR_LJ = 30   # algorithmic FLOPs per in-range ordered pair (FMA = 2)
FLOPS_VGB = 60           # algorithmic FP64 FLOPs per particle of the vGB update
# algorithmic HBM bytes per particle-step of the whole mixed step, each unique state
# array read and written once: rebuild 84, force 28, vGB 180
BYTES_PER_PARTICLE_STEP = 292
# Verlet pair-list skin of the mixed form; the cell grid is the finest with
# cellSize >= rc + skin, so the list can be built from the 27-cell walk
SKIN = 0.4
# untimed steps run under the clock sampler before the timed ones (~1.5 s)
CLOCK_WINDOW_STEPS = 6000


def workload(cells=64, skin=SKIN):
    """The 2^20 LJ liquid (FCC start, rho = 0.8) on the finest grid of cells of
    at least cutOff + skin."""
    from proteinsim2015_gb300 import init
    a = (4.0 / 0.8) ** (1.0 / 3.0)
    box = cells * a
    pos = init.fcc(cells, a).reshape(-1)
    n = pos.size // 3
    scale = int(math.floor(box / (RC + max(skin, 0.0))))
    vel = init.maxwell(n, KT, seed=90210).reshape(-1)
    return dict(n=n, box=box, scale=scale, cell_size=box / scale, pos=pos, vel=vel,
                radius=np.full(n, 0.5), cells=cells)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# the dominant kernel of the mixed step and the ncu summary that gives its
# DRAM traffic per launch (a line "dram_bytes_per_launch: B") and its L1
# data-pipe load ("l1_data_pipe_wavefronts_per_launch: W",
# "l1_data_pipe_pct_of_peak: P")
FORCE_KERNEL = "force_list_kernel<MixedBody<LJPure<6>>, 1, 0, 0, 1>"
FORCE_PROFILE = os.path.join(ROOT, "profiles", "force_list_lj_rho0.8_n2e20.txt")


def profiled_value(path, key):
    """The number on the line "key: value" of a committed ncu summary, or None."""
    try:
        with open(path) as fh:
            for line in fh:
                if line.startswith(key + ":"):
                    return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def profiled_traffic(path):
    """DRAM bytes per launch (read + write) from a committed ncu summary, or None."""
    return profiled_value(path, "dram_bytes_per_launch")


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def cpu_steps(w, threads):
    """A stepping closure over the oracle restatement on the host cores:
    run(k) advances the workload k whole steps, with fresh counter-based
    Gaussians every step."""
    from oracle import port
    port.set_threads(threads)
    g = port.geom(w["n"], w["box"], w["cell_size"], w["scale"])
    f = port.make_force(port.LJ, RC, kT=KT, well_depth=WD, lj_num=LJN, yuk_str=0.0)
    c = port.vgb_coeffs(GAMMA, DT, KT)
    st = port.State(w["pos"], w["radius"], vel=w["vel"])
    cells = [None]

    def run(k):
        err, hi, cse, srt, _ = port.run(g, f, c, DT, st, k, None, vel_freq=1000,
                                        cells=cells[0])
        cells[0] = (hi, cse, srt)
        if err:
            msg = "oracle step %d failed with %d" % (st.step, err)
            try:
                from scipy.spatial import cKDTree
                p = np.mod(st.pos.reshape(-1, 3), w["box"])
                d, _ = cKDTree(p, boxsize=w["box"]).query(p, k=2)
                msg += "; min pair distance %.6g" % d[:, 1].min()
            except Exception:
                pass
            raise RuntimeError(msg)
    return run


def cpu_port_rate(w, budget_s, threads):
    """particle-steps/s of the oracle restatement on the same workload, over
    whole steps until about budget_s elapse (after one warm-up step)."""
    run = cpu_steps(w, threads)
    run(1)
    steps, t0 = 0, time.perf_counter()
    while True:
        run(1)
        steps += 1
        el = time.perf_counter() - t0
        if el >= budget_s or steps >= 1000:
            break
    return w["n"] * steps / el, steps, el


def cpu_baseline_child(budget_s):
    """Body of the child process that times the CPU baseline (it runs apart
    from the GPU process so neither disturbs the other)."""
    w = workload()
    cores = os.cpu_count() or 1
    try:
        v, steps, secs = cpu_port_rate(w, budget_s, cores)
        out = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "N=%d, %d whole steps (%.1f s) of the same workload" % (
                   w["n"], steps, secs)}
        v1, steps1, secs1 = cpu_port_rate(w, budget_s / 3.0, 1)
        out["one_thread"] = {"value": v1, "unit": UNIT, "cores": 1,
                             "sample": "N=%d, %d whole steps (%.1f s)" % (w["n"], steps1, secs1)}
    except Exception as e:
        out = {"value": None, "unit": UNIT, "cores": cores, "kind": "port", "error": str(e)}
    print(json.dumps(out))
    return 0


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    w = workload()
    # The reference cannot travel to the GPU machine (its tree is absent
    # there); its CPU path is the oracle restatement, pinned bit-exact to the
    # reference's own code by tests/test_oracle_golden.py.
    kind = "port"
    run = cpu_steps(w, threads)
    nw = max(1, min(args.warmup, 3))
    t_w = time.perf_counter()
    run(nw)
    per = (time.perf_counter() - t_w) / nw
    # one step of this arm is one whole step of the workload on the CPU; the
    # number of timed steps is bounded so the run ends within a few minutes
    k = max(1, min(args.steps, int(60.0 / max(per, 1e-3))))
    t0 = time.perf_counter()
    run(k)
    el = time.perf_counter() - t0
    v = w["n"] * k / el
    sample = ("N=%d LJ rho=0.8 from the FCC start, %d whole steps of %d requested "
              "(oracle restatement of the reference, %d threads)" % (w["n"], k, args.steps,
                                                                     threads))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws,
            "steps": k, "warmup": nw, "ms_per_step": 1e3 * el / k,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": "lj_rho0.8_N2^20", "n_particles": w["n"],
                                            "box": w["box"], "cell_scale": w["scale"]},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def cpu_baseline(budget_s=15.0):
    """The oracle restatement on the host cores over a bounded sample (about
    budget_s) of the same workload, timed in a child process."""
    p = subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-baseline-json",
                        str(budget_s)], capture_output=True, text=True, timeout=900)
    for line in reversed(p.stdout.splitlines()):
        if line.startswith("{"):
            return json.loads(line)
    return {"value": None, "unit": UNIT, "kind": "port",
            "error": "child failed rc=%d: %s" % (p.returncode, p.stderr[-500:])}


def pinned(n, dtype=None):
    import torch
    return torch.empty(n, dtype=dtype or torch.float64, pin_memory=True).numpy()


def e2e_dropin(psim, w, state, min_steps=30, min_seconds=1.0):
    """The reference's step loop on host arrays with the GPU drop-ins:
    force_evaluate -> nextSystem (with push) -> cells_build, for at least
    min_steps steps and min_seconds.  Returns (particle-steps/s, h2d
    bytes/step, d2h bytes/step, pair-list calls and builds, steps)."""
    n, box, scale = w["n"], w["box"], w["scale"]
    g = psim.geometry(n, box, box / scale, scale)
    p = psim.make_force("LJ", RC, kT=KT, well_depth=WD, lj_num=LJN, yukawa_strength=0.0)
    buf = {k: pinned(3 * n) for k in ("pos", "pos0", "vel", "frc", "frc0")}
    for k in buf:
        buf[k][:] = state[k]
    mass = pinned(n)
    mass[:] = 1.0
    rad = pinned(n)
    rad[:] = 0.5
    it = psim.Integrator(n, gamma=GAMMA, dt=DT, kT=KT, vel_freq=1000)
    import torch
    ncell = scale ** 3
    # the reference's arrays in pinned host memory, written in place each step
    cells = (pinned(2 * n, torch.int32), pinned(2 * ncell, torch.int32).view(np.uint32),
             pinned(4 * n))
    f = pinned(3 * n)
    hi, cse, srt = psim.cells_build(g, buf["pos"], rad, out=cells)
    t_cur = DT  # continue as a normal step
    # one system stepped through the drop-ins: keep the force pass's pair list
    # across calls (the library's default builds one per call)
    psim.set_force_list_skin(-1.0)
    calls0, builds0 = psim.force_list_stats()
    n_steps = 0
    t0 = time.perf_counter()
    while n_steps < min_steps or time.perf_counter() - t0 < min_seconds:
        psim.force_evaluate(p, g, srt, hi, cse, precision=psim.PRECISION_MIXED, out=f)
        it.next_system(t_cur, box, buf["pos"], buf["pos0"], buf["vel"], buf["frc"], buf["frc0"],
                       mass, particle_force=f)
        psim.cells_build(g, buf["pos"], rad, out=cells)
        t_cur += DT
        n_steps += 1
    el = time.perf_counter() - t0
    calls1, builds1 = psim.force_list_stats()
    # per step: force_evaluate (sorted, hash index, cell ranges in; force out),
    # next_system (positions, previous positions, the two forces, masses in;
    # positions, previous positions and the pushed forces out -- velocities
    # move only on the first and velocity steps), cells_build (positions,
    # radii in; hash index, cell ranges, sorted out)
    h2d = (32 * n + 8 * n + 8 * ncell) + (4 * 24 * n + 8 * n) + (24 * n + 8 * n)
    d2h = 24 * n + 4 * 24 * n + (8 * n + 8 * ncell + 32 * n)
    it.close()
    psim.set_force_list_skin(0.0)
    lists = {"calls": calls1 - calls0, "builds": builds1 - builds0}
    return n * n_steps / el, h2d, d2h, lists, n_steps


def mixed_vs_fp64(psim, g, p, w, state, seed, dev, steps=200, every=20):
    """The mixed form's error against the plain FP64 form in the quantities a
    run reports: from the same melted state and the same Philox noise, both
    forms step `steps` steps (velocities every step); every `every` steps the
    FP64 potential energy and virial per particle (psim_system_energy), the
    kinetic temperature (getTemperature) and g(r) (100 bins on [0.8, 2.9))
    are taken.  Reported: the relative differences of the run means and of
    the final values, and the largest relative g(r) bin difference."""
    runs = []
    for prec, skin in ((psim.PRECISION_MIXED, SKIN), (psim.PRECISION_FP64, 0.0)):
        s = psim.System(g, p, gamma=GAMMA, dt=DT, kT=KT, vel_freq=0, seed=seed + 1,
                        precision=prec, device=dev, skin=skin)
        s.upload(state["pos"], w["radius"], vel=state["vel"], pos0=state["pos0"],
                 frc=state["frc"], frc0=state["frc0"])
        u, vir, T, gr = [], [], [], []
        for _ in range(steps // every):
            s.step(every)
            e = s.energy()
            u.append(e[0])
            vir.append(e[1])
            T.append(s.temperature())
            gr.append(s.rdf(0.8, 2.9, 100))
        s.close()
        runs.append((np.array(u), np.array(vir), np.array(T), np.array(gr)))
    (um, wm, tm, gm), (u6, w6, t6, g6) = runs
    rel = lambda a, b: float(abs(a - b) / abs(b))
    gmean_m, gmean_6 = gm.mean(0), g6.mean(0)
    return {"steps": steps, "samples": steps // every, "n_particles": g.n_particles,
            "energy_per_particle": {"mixed": float(um.mean()), "fp64": float(u6.mean()),
                                    "rel_diff_mean": rel(um.mean(), u6.mean()),
                                    "rel_diff_final": rel(um[-1], u6[-1])},
            "virial_per_particle": {"mixed": float(wm.mean()), "fp64": float(w6.mean()),
                                    "rel_diff_mean": rel(wm.mean(), w6.mean()),
                                    "rel_diff_final": rel(wm[-1], w6[-1])},
            "temperature": {"mixed": float(tm.mean()), "fp64": float(t6.mean()),
                            "rel_diff_mean": rel(tm.mean(), t6.mean()),
                            "rel_diff_final": rel(tm[-1], t6[-1])},
            "gr": {"rel_l2_mean": float(np.linalg.norm(gmean_m - gmean_6) / np.linalg.norm(gmean_6)),
                   "max_bin_rel_diff_mean": float(np.max(np.abs(gmean_m - gmean_6) /
                                                         np.maximum(gmean_6, 1e-3))),
                   "bins": 100, "range": [0.8, 2.9]},
            "note": "same start and Philox noise; energy and virial are FP64 reductions "
                    "(pair energy u(r) integrated from the plugin's force law)"}


def run_batched(psim, dev, steps=2000, n_reps=512, tune=True, skin=0.3):
    """The batched-replica workload: 512 independent AO systems (N, phi,
    contact attraction and q drawn per replica), gamma = 1, dt = 1e-3, mixed
    form, every step one set of launches over all replicas.  `value`: with a
    pair list (skin 0.3; each replica's grid the finest with cellSize >= cutOff
    + skin).  `cell_walk`: the 27-cell walk every step, each replica's cell size
    chosen by the autotuner per size bucket."""
    from proteinsim2015_gb300 import batch
    draws = batch.c2_draws(n_reps)
    pos, vel = batch.states(draws)

    def timed(reps, sk):
        b = psim.Batch(reps, gamma=1.0, dt=0.001, kT=1.0, vel_freq=1000,
                       precision=psim.PRECISION_MIXED, device=dev, skin=sk)
        b.upload(pos, np.full(b.n, 0.5), vel=vel)
        b.step(3)
        lanes = None
        if sk > 0 and tune:   # threads per particle of the list pass, on the live batch
            lanes = batch.tune_lanes(b, steps=min(steps, 100))
        b0 = b.list_builds()
        ms = b.time_steps(steps)
        builds = b.list_builds() - b0
        prof = b.profile(5)
        out = {"value": b.n * steps / (ms * 1e-3), "ms_per_step": ms / steps,
               "phases_ms": {k: round(v, 5) for k, v in prof.items()},
               "launches": steps * b.launches_per_step() + builds * b.launches_per_rebuild()}
        if sk > 0:
            out["list_builds"] = builds
        if lanes:
            out["lanes_per_particle"] = {"chosen": lanes[0],
                                         "rates": {str(k): v for k, v in lanes[1].items()}}
        n = b.n
        b.close()
        return out, n

    listed, n = timed(batch.replicas(psim, draws, skin=skin), skin)
    t0 = time.time()
    factors, report = batch.autotune(psim, draws, device=dev) if tune else ([1.0] * n_reps, {})
    t_tune = time.time() - t0
    walk, _ = timed(batch.replicas(psim, draws, factors), 0.0)
    walk["autotune"] = {"seconds": round(t_tune, 1),
                        "buckets": {str(k): {"factor": v[0],
                                             "rates": {str(f): r for f, r in v[1].items()}}
                                    for k, v in report.items()}}
    out = {"workload": "c2_%d_ao_replicas" % n_reps, "unit": UNIT, "n_particles": int(n),
           "replicas": n_reps, "steps": steps, "skin": skin}
    out.update(listed)
    out["cell_walk"] = walk
    return out


def run_differentiable(psim, dev, steps=2000):
    """The differentiable-trajectory workload: N = 32768 colloids at phi = 0.15
    with AO attraction (q = 0.1, 3 kT) and Yukawa repulsion (A = 10 kT,
    kappa = 4, cutoff 3), 2,000 FP64 steps at dt = 1e-3 with fixed Philox noise;
    loss: the squared distance of the time-averaged smoothed g(r) (100 bins on
    [0.8, 3]) from the g(r) of perturbed parameters; gradients with respect to
    (AO strength, q, A, kappa) by the adjoint with a checkpoint every 100 steps."""
    from proteinsim2015_gb300 import adjoint as adj, init
    n, phi = 32768, 0.15
    box = (n * math.pi / 6.0 / phi) ** (1.0 / 3.0)
    scale = int(math.floor(box / 3.1))
    g = psim.geometry(n, box, box / scale, scale)
    pos = init.rsa_native(n, box, 1.0, seed=33).reshape(-1)
    vel = init.maxwell(n, 1.0, seed=34).reshape(-1)
    a = adj.Adjoint(g, steps, dt=0.001, seed=35, checkpoint_every=100, sample_every=10,
                    r_min=0.8, r_max=3.0, n_bins=100, device=dev)
    p, J = adj.plugin_params(3.0, 0.1, 10.0, 4.0)
    pt, _ = adj.plugin_params(3.3, 0.11, 9.0, 4.2)
    target = a.forward(pt, pos, vel)
    t0 = time.perf_counter()
    a.forward(p, pos, vel)
    t1 = time.perf_counter()
    loss, _, grad, _ = a.gradient(p, pos, target, vel)
    t2 = time.perf_counter()
    a.close()
    return {"workload": "c3_adjoint_N32768_phi0.15_2000steps", "n_particles": n, "steps": steps,
            "forward_s": t1 - t0, "gradient_s": t2 - t1, "adjoint_over_forward": (t2 - t1) / (t1 - t0),
            "forward_particle_steps_per_s": n * steps / (t1 - t0), "loss": loss,
            "grad_physical": dict(zip(("ao_strength", "q", "yukawa_A", "kappa"),
                                      (J.T @ grad).tolist())),
            "note": "q through the AO coefficients; the cutoff 1 + q is held fixed"}


def run_gel(psim, dev, steps=1000, skin=0.0, chunk=100, n=1 << 23):
    """The gel stress workload: N = 2^23 AO colloids at phi = 0.30 (q = 0.08,
    6 kT contact attraction, cutoff 1.08), seeded RSA start, gamma = 1,
    dt = 1e-3, mixed form.  skin 0: the cell list is rebuilt every step and
    the force pass walks the 27 cells (the workload as stated); skin > 0: a
    pair list rebuilt when a particle has moved skin/2.  Reports the maximum
    and mean particles per cell every `chunk` steps while the colloids
    aggregate, the clusters and the kinetic temperature at the end."""
    from proteinsim2015_gb300 import init, batch
    phi = 0.30
    box = (n * math.pi / 6.0 / phi) ** (1.0 / 3.0)
    f = batch.ao_params(psim, 6.0, 0.08)
    # cells of at least cutOff + skin and of the 1.2 contact distance the
    # cluster analysis walks (updateInteractions' radius)
    scale = int(math.floor(box / max(f.cutoff + skin, 1.2)))
    g = psim.geometry(n, box, box / scale, scale)
    t0 = time.time()
    pos = init.rsa_native(n, box, 1.0, seed=2023).reshape(-1)
    t_init = time.time() - t0
    vel = init.maxwell(n, 1.0, seed=5).reshape(-1)
    s = psim.System(g, f, gamma=1.0, dt=0.001, kT=1.0, vel_freq=1000, seed=11,
                    precision=psim.PRECISION_MIXED, device=dev, skin=skin)
    s.upload(pos, np.full(n, 0.5), vel=vel)
    s.step(3)
    occ, ms = [s.cell_occupancy()], 0.0
    for _ in range(max(1, steps // chunk)):
        ms += s.time_steps(chunk)
        occ.append(s.cell_occupancy())
    done = max(1, steps // chunk) * chunk
    prof = s.profile(5)
    _, groups, avg = s.clusters(1.2, 4)
    out = {"workload": "c4_gel_ao_phi0.30_N2^%d" % int(round(math.log2(n))), "n_particles": n,
           "box": box,
           "cell_scale": scale, "skin": skin, "steps": done,
           "value": n * done / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / done,
           "phases_ms": {k: round(v, 5) for k, v in prof.items()},
           "list_builds": s.list_builds(),
           "occupancy_max": [m for m, _ in occ], "occupancy_mean": occ[0][1],
           "occupancy_every_steps": chunk, "rsa_seconds": round(t_init, 2),
           "clusters_gt4": len(groups), "mean_cluster_size": avg,
           "temperature": s.temperature(),
           "temperature_note": "above kT while the colloids aggregate: the energy released "
                               "into the 6 kT wells outpaces the gamma = 1 friction; the "
                               "oracle reads the same at every dt tried, and a repulsive "
                               "control stays at kT"}
    s.close()
    return out


def run_c0(psim, dev, steps=10000, cpu_budget_s=3.0):
    """The reference's own CPU-runnable case: N = 4000 AO colloids (cutOff 1.1,
    wellDepth 0.25: -4 kT at contact) in the box the reference can represent,
    L = 21 with 7 cells a side (phi = 0.226), gamma = 1, dt = 1e-3, kT = 1,
    10,000 steps from a seeded RSA start with Maxwell-Boltzmann velocities: on
    the GPU in the mixed form with a pair list and in the plain FP64 form, and
    the oracle port (the CPU baseline) on all host cores over a few seconds."""
    from proteinsim2015_gb300 import init
    n, L, scale = 4000, 21.0, 7
    g = psim.geometry(n, L, L / scale, scale)
    f = psim.make_force("AO", 1.1, kT=1.0, well_depth=0.25)
    pos = init.rsa_native(n, L, 1.0, seed=90210).reshape(-1)
    vel = init.maxwell(n, 1.0, seed=90211).reshape(-1)
    out = {"workload": "c0_ao_N4000_L21", "n_particles": n, "steps": steps, "unit": UNIT}
    for name, prec, skin in (("mixed_list", psim.PRECISION_MIXED, psim.auto_skin(g, f)),
                             ("plain_fp64", psim.PRECISION_FP64, 0.0)):
        s = psim.System(g, f, gamma=1.0, dt=0.001, kT=1.0, vel_freq=1000, seed=7, precision=prec,
                        device=dev, skin=skin)
        s.upload(pos, np.full(n, 0.5), vel=vel)
        s.step(3)
        ms = s.time_steps(steps)
        out[name] = {"value": n * steps / (ms * 1e-3), "ms_per_step": ms / steps, "skin": skin}
        s.close()
    from oracle import port
    cores = os.cpu_count() or 1
    port.set_threads(cores)
    pg = port.geom(n, L, L / scale, scale)
    pf = port.make_force(port.AO, 1.1, kT=1.0, well_depth=0.25)
    c = port.vgb_coeffs(1.0, 0.001, 1.0)
    st = port.State(pos, np.full(n, 0.5), vel=vel)
    cells = None
    done, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < cpu_budget_s:
        err, hi, cse, srt, _ = port.run(pg, pf, c, 0.001, st, 50, None, vel_freq=1000,
                                        cells=cells)
        cells = (hi, cse, srt)
        if err:
            break
        done += 50
    el = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": n * done / el if done else None, "unit": UNIT, "cores": cores,
                           "kind": "port",
                           "sample": "N=4000, %d whole steps (%.1f s) of the same workload" % (
                               done, el)}
    return out


def profile_workload(args):
    """A short run of one workload for a profiler capture; prints one JSON line."""
    import proteinsim2015_gb300 as psim
    dev = 0
    if args.profile_workload == "batched":
        # 64 of the 512 replicas: the same kernels on ~0.7 M particles, so a
        # profiler's save and restore of device memory between passes stays small
        out = run_batched(psim, dev, steps=args.steps, n_reps=64, tune=False)
    elif args.profile_workload == "adjoint":
        out = run_differentiable(psim, dev, steps=args.steps)
    elif args.profile_workload == "gel":
        # the gel's kernels (27-cell walk, cell list rebuilt every step) on a
        # quarter of its particles at the same volume fraction, so a
        # profiler's save and restore of device memory stays small
        out = run_gel(psim, dev, steps=args.steps, chunk=args.steps, n=1 << 21)
    else:   # the 2^20 liquid in the plain FP64 form, or the mixed form's 27-cell walk
        w = workload()
        n, box, scale = w["n"], w["box"], w["scale"]
        g = psim.geometry(n, box, box / scale, scale)
        p = psim.make_force("LJ", RC, kT=KT, well_depth=WD, lj_num=LJN, yukawa_strength=0.0)
        fp64 = args.profile_workload == "fp64"
        s = psim.System(g, p, gamma=GAMMA, dt=DT, kT=KT, vel_freq=1000, seed=90210,
                        precision=psim.PRECISION_FP64 if fp64 else psim.PRECISION_MIXED,
                        device=dev)
        s.upload(w["pos"], w["radius"], vel=w["vel"])
        s.step(max(args.warmup, 1))
        ms = s.time_steps(args.steps)
        out = {"workload": "lj_rho0.8_N2^20_" + ("fp64" if fp64 else "mixed_walk"),
               "value": n * args.steps / (ms * 1e-3), "ms_per_step": ms / args.steps,
               "phases_ms": s.profile(2)}
        s.close()
    out["profile_only"] = True
    print(json.dumps(out))
    return 0


def run_gpu(args):
    import proteinsim2015_gb300 as psim
    if args.profile_only and args.profile_workload != "mixed":
        return profile_workload(args)
    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    dev = local
    if psim.device_count() <= dev:
        raise SystemExit("no CUDA device %d" % dev)
    w = workload(skin=args.skin)
    n, box, scale = w["n"], w["box"], w["scale"]
    g = psim.geometry(n, box, box / scale, scale)
    p = psim.make_force("LJ", RC, kT=KT, well_depth=WD, lj_num=LJN, yukawa_strength=0.0)
    seed = 90210 + 7919 * rank   # independent replicas per rank
    s = psim.System(g, p, gamma=GAMMA, dt=DT, kT=KT, vel_freq=1000, seed=seed,
                    precision=psim.PRECISION_MIXED, device=dev, skin=args.skin)
    s.upload(w["pos"], w["radius"], vel=w["vel"])
    s.step(max(args.warmup, 3))          # W >= 3 untimed warm-up steps (melting the lattice)
    if dist:
        dist.barrier()
    # clocks are sampled every 100 ms over ~1.5 s of untimed steps of the same
    # workload and then over the timed steps, so the record covers the load
    # the timed steps run under
    # threads per particle of the list force pass, tuned on the live system
    # (untimed steps, part of the warm-up); a profile-only run stays short:
    # one lane, no clock window
    from proteinsim2015_gb300 import batch as _batch
    tune = args.skin > 0 and not args.profile_only
    lanes, lane_rates = _batch.tune_lanes(s, steps=200) if tune else (1, {})
    with ClockSampler(dev) as clk:
        if not args.profile_only:
            s.time_steps(CLOCK_WINDOW_STEPS)
        builds0 = s.list_builds()
        ms = s.time_steps(args.steps)
        builds_timed = s.list_builds() - builds0
    if dist:
        import torch
        t = torch.tensor([ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * n * args.steps / (ms * 1e-3)
    if rank != 0:
        dist.barrier()
        return 0
    # ---- per-phase device times on the mixed form (roofline of the force pass)
    prof = s.profile(20)
    pairs = s.pair_count(RC)
    builds, steps_run = s.list_builds(), s.get_step()[0]
    if args.profile_only:
        print(json.dumps({"profile_only": True, "value": value, "unit": UNIT,
                          "ms_per_step": ms / args.steps, "phases_ms": prof,
                          "pairs_per_particle": pairs, "skin": args.skin,
                          "cell_scale": scale, "list_builds": s.list_builds()}))
        s.close()
        return 0
    state = s.download()
    # ---- plain FP64 form on the same melted state
    s64 = psim.System(g, p, gamma=GAMMA, dt=DT, kT=KT, vel_freq=1000, seed=seed,
                      precision=psim.PRECISION_FP64, device=dev)
    s64.upload(state["pos"], w["radius"], vel=state["vel"], pos0=state["pos0"],
               frc=state["frc"], frc0=state["frc0"])
    s64.step(2)
    k64 = max(5, min(args.steps // 20, 50))
    ms64 = s64.time_steps(k64)
    prof64 = s64.profile(3)
    plain = n * k64 / (ms64 * 1e-3)
    # ---- the mixed form without a pair list (the 27-cell walk, the cell
    # list rebuilt every step) on the same state and grid: the precision gain
    # apart from the Verlet-list gain
    s0 = psim.System(g, p, gamma=GAMMA, dt=DT, kT=KT, vel_freq=1000, seed=seed,
                     precision=psim.PRECISION_MIXED, device=dev, skin=0.0)
    s0.upload(state["pos"], w["radius"], vel=state["vel"], pos0=state["pos0"],
              frc=state["frc"], frc0=state["frc0"])
    s0.step(3)
    k0 = max(10, min(args.steps, 200))
    ms0 = s0.time_steps(k0)
    prof0 = s0.profile(3)
    s0.close()
    mixed_skin0 = {"value": n * k0 / (ms0 * 1e-3), "unit": UNIT, "steps": k0,
                   "ms_per_step": ms0 / k0, "force_ms": prof0["force_ms"], "skin": 0.0,
                   "speedup_vs_fp64": (n * k0 / (ms0 * 1e-3)) / plain}
    precision_errors = mixed_vs_fp64(psim, g, p, w, state, seed, dev)
    # ---- force error of the mixed form (the pair-list pass the timed steps
    # ran) against the plain FP64 pass, on the melted state
    hi, cse, srt = s.download_cells()
    f64 = psim.force_evaluate(p, g, srt, hi, cse, precision=psim.PRECISION_FP64)
    f32 = s.forces()
    ferr = float(np.linalg.norm(f32 - f64) / np.linalg.norm(f64))
    rms = float(np.sqrt(np.mean(np.sum(f64.reshape(-1, 3) ** 2, axis=1))))
    fmax = float(np.max(np.abs(f32 - f64).reshape(-1, 3).max(1)) / rms)
    s64.close()
    # ---- end to end through the reference-layout drop-ins on pinned host buffers
    e2e_v, h2d, d2h, e2e_lists, e2e_steps = e2e_dropin(psim, w, state)
    # the host link the drop-ins' traffic crosses: its measured rates
    link = psim.measure_host_link(dev)
    e2e_ms = n / e2e_v * 1e3
    link_gbs = (h2d + d2h) / (e2e_ms * 1e-3) / 1e9
    # ---- roofline of the dominant kernel (the force pass)
    fp32_peak = psim.measure_fp32_peak(dev)
    f_ms = prof["force_ms"]
    flops_launch = n * pairs * FLOPS_PER_PAIR_LJ
    achieved = flops_launch / (f_ms * 1e-3) / 1e12
    peaks = measured_peaks()
    # ---- CPU baseline: the oracle restatement on the host cores, bounded sample
    cpu = cpu_baseline(15.0)
    # ---- batched replicas (512 AO systems), against this single large system
    batched = None
    if args.batched_steps > 0 and ws == 1:
        batched = run_batched(psim, dev, args.batched_steps)
        batched["vs_single_system"] = batched["value"] / value
    differentiable = run_differentiable(psim, dev) if args.batched_steps > 0 and ws == 1 else None
    gel = None
    if args.gel_steps > 0 and ws == 1:
        gel = run_gel(psim, dev, args.gel_steps, skin=0.0)
        gl = run_gel(psim, dev, args.gel_steps, skin=0.3)
        gel["pair_list"] = {k: gl[k] for k in ("skin", "value", "ms_per_step", "phases_ms",
                                               "list_builds", "cell_scale", "temperature",
                                               "clusters_gt4")}
    c0 = run_c0(psim, dev) if args.gel_steps > 0 and ws == 1 else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32-pair/f64-update",
        "data": "synthetic FCC-melt start, seeded Maxwell-Boltzmann velocities",
        "config": {"workload": "lj_rho0.8_N2^20", "n_particles": n, "box": box,
                   "cell_scale": scale, "cell_size": box / scale, "potential": "LJ 12-6 rc=2.5",
                   "kT": KT, "gamma": GAMMA, "dt": DT, "precision": "mixed",
                   "noise": "philox", "parallelism": "replicas" if ws > 1 else "single",
                   "skin": args.skin, "pair_list": args.skin > 0, "list_lanes": lanes,
                   "l2": "inputs larger than L2 (FP64 SoA state ~300 MB, sorted copies 32 MB)"},
        "plain_fp64": {"value": plain, "unit": UNIT, "steps": k64, "ms_per_step": ms64 / k64,
                       "force_ms": prof64["force_ms"]},
        "speedup_vs_fp64": value / plain,
        "mixed_skin0": mixed_skin0,
        "precision_errors": precision_errors,
        "force_rel_err": ferr, "force_abs_err_max_over_rms_force": fmax,
        "phases_ms": {k: round(v, 5) for k, v in prof.items()},
        "pairs_per_particle": pairs,
        "list_lanes_rates": {str(k): v for k, v in lane_rates.items()},
        "pair_list": {"skin": args.skin, "rebuilds": builds, "steps": steps_run,
                      "rebuild_every": (steps_run / builds) if builds else None},
        "e2e": {"value": e2e_v, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": e2e_steps, "force_lists": e2e_lists,
                "ms_per_step": e2e_ms,
                "link_roofline": {"bound": "host link", "achieved": link_gbs,
                                  "peak": link["both"], "unit": "GB/s",
                                  "frac": link_gbs / link["both"],
                                  "read_gbs": link["read"], "write_gbs": link["write"],
                                  "peak_source": "measured: SM loads and stores on pinned "
                                                 "host memory, both directions at once"},
                "path": "force_evaluate -> next_system -> cells_build on pinned host arrays, read and written in place by the GPU over NVLink-C2C (copies where the device has no pageable host access)"},
        "gpu_launches": args.steps * s.launches_per_step() + builds_timed * s.launches_per_rebuild(),
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak,
                     "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                     "traffic": profiled_traffic(FORCE_PROFILE),
                     "kernel": FORCE_KERNEL,
                     "algorithmic": "%d FLOP/pair x %.2f pairs/particle x N per launch" % (
                         FLOPS_PER_PAIR_LJ, pairs),
                     "peak_source": "measured FP32 FMA probe (MEASURED_PEAKS.json has no FP32 figure)",
                     "hbm_peak_gbs": peaks.get("hbm_gbs"),
                     # the bound the pass meets: the L1 data pipe (one
                     # wavefront per cycle per SM) serving the record gathers
                     "l1_data_pipe": {
                         "wavefronts_per_launch": profiled_value(
                             FORCE_PROFILE, "l1_data_pipe_wavefronts_per_launch"),
                         "frac": (profiled_value(FORCE_PROFILE, "l1_data_pipe_pct_of_peak") or 0.0)
                         / 100.0 or None,
                         "source": "ncu summary " + os.path.relpath(FORCE_PROFILE, ROOT)}},
        "step_roofline": {
            "flops_per_particle_step": pairs * FLOPS_PER_PAIR_LJ + FLOPS_VGB,
            "bytes_per_particle_step": BYTES_PER_PARTICLE_STEP,
            "achieved_tflops": value * (pairs * FLOPS_PER_PAIR_LJ + FLOPS_VGB) / 1e12,
            "achieved_gbs": value * BYTES_PER_PARTICLE_STEP / 1e9,
            "frac": max(value * (pairs * FLOPS_PER_PAIR_LJ + FLOPS_VGB) / 1e12 / fp32_peak,
                        value * BYTES_PER_PARTICLE_STEP / 1e9 / peaks["hbm_gbs"])
            if peaks.get("hbm_gbs") else None,
            "note": "whole step: max(FLOP/s over the FP32 peak, algorithmic bytes/s over "
                    "the measured HBM copy rate)"},
        "cpu_baseline": cpu,
        "batched": batched,
        "differentiable": differentiable,
        "gel": gel,
        "c0": c0,
        "clocks": clk.summary(),
    }
    print(json.dumps(line))
    if dist:
        dist.barrier()
    s.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-baseline-json", type=float, default=None,
                    help=argparse.SUPPRESS)
    ap.add_argument("--batched-steps", type=int, default=2000,
                    help="steps of the batched-replica run (0: skip it)")
    ap.add_argument("--gel-steps", type=int, default=1000,
                    help="steps of the 2^23 AO gel run (0: skip it)")
    ap.add_argument("--skin", type=float, default=SKIN,
                    help="pair-list skin of the mixed form (0: walk the 27 cells every step)")
    ap.add_argument("--profile-only", action="store_true",
                    help="time the mixed form and its phases only (short runs under ncu)")
    ap.add_argument("--profile-workload", default="mixed",
                    choices=["mixed", "fp64", "walk", "batched", "adjoint", "gel"],
                    help="with --profile-only: the workload to run for --steps steps: the "
                         "2^20 liquid in the mixed form, in the plain FP64 form, or in the "
                         "mixed form without a skin (the 27-cell walk), the 512 AO replicas "
                         "with a pair list, the differentiable trajectory, or the gel at "
                         "2^21 particles")
    args = ap.parse_args()
    if args.cpu_baseline_json is not None:
        return cpu_baseline_child(args.cpu_baseline_json)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
