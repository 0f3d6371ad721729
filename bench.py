"""Benchmark of the DEM pair-force + integration path on GB300.

Workload (default): one seeded random-sequential-attachment aggregate of 32768 monomers
(r = 14 nm, rho = 1700 kg/m^3), Luding frictional contact plus limited-range Hamaker attraction
(A = 1e-19 J, h0 = 0.4 nm, surface-gap cutoff 2r = centre distance 4r), no bonds, Verlet list of
radius 4.5r (cutoff + 0.5r skin) rebuilt every 20 steps with spring history carried across
rebuilds, velocity-Verlet with dt = 0.01 sqrt(m/k_n), velocities uniform in +-0.1 m/s. One bench
step = 20 velocity-Verlet steps (one rebuild period) over all 32768 particles; the metric is
particle-steps/s. The headline value is the mixed-precision path (FP32 pair arithmetic, FP64
separation/overlap/springs/sums/integration); the plain FP64 path is timed in the same run.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
Under torchrun (N > 1) every rank runs an independent replica (the single aggregate does not
shard without a halo exchange); value = all ranks' particle-steps / max rank time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_PART = 32768
VV_PER_STEP = 20
SEED = (1 << 32) + 0
METRIC = "particle-steps/s batched FP32/FP64 vs plain FP64 GPU at <=1e-6 rel err; p99 latency"


def workload_desc(precision):
    from libgran_gb300 import _abi as A
    from libgran_gb300 import configs as K
    mat = K.Material()
    d = K.make_desc(N_PART, A.LG_BINARY_CONTACT, A.LG_HAMAKER_LIMITED, contact=mat.contact(), hamaker=mat.hamaker(),
                    pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r, precision=precision, max_neighbors=96)
    return mat, d


def workload_state(generator=None):
    """The seeded aggregate and velocities; `generator` is a module with generate_aggregate and
    generate_velocities (the engine's by default; the reference arm passes the oracle's, which gives
    the same bits without loading the engine library)."""
    from libgran_gb300 import configs as K
    if generator is None:
        from libgran_gb300 import system as generator
    mat = K.Material()
    x0 = generator.generate_aggregate(SEED, N_PART, mat.r)
    v0 = generator.generate_velocities(SEED, N_PART, 0.1)
    return x0, v0


def repo_native_libraries():
    """Shared libraries of this repository mapped into the process (from /proc/self/maps)."""
    libs = set()
    try:
        for line in open("/proc/self/maps"):
            path = line.split()[-1] if len(line.split()) >= 6 else ""
            if path.endswith(".so") and path.startswith(ROOT + os.sep):
                libs.add(os.path.relpath(path, ROOT))
    except OSError:
        return None
    return sorted(libs)


# ------------------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append(parts)
            except Exception:
                pass
        os.unlink(self.path)
        if not rows:
            return out
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        out.update(sm_mhz=statistics.median(sm) if sm else None, sm_max_mhz=max(mx) if mx else None,
                   reasons=sorted(reasons), samples=len(rows))
        return out


def read_profile_traffic(kernel_tag):
    """DRAM bytes per launch from the committed ncu summary of this kernel (profiles/*.md)."""
    import glob
    for p in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        for line in open(p):
            if line.startswith("traffic_per_launch_bytes[%s]:" % kernel_tag):
                try:
                    return float(line.split(":", 1)[1].split()[0])
                except ValueError:
                    return None
    return None


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


# ------------------------------------------------------------------------------------------------
def cpu_reference_rate(x0, v0, target_s=12.0, threads=None):
    """The oracle (CPU restatement of libgran's path, FP64, OpenMP over all host cores) on a bounded
    sample of the same workload: the same aggregate and parameters, timed over whole
    20-step rebuild periods."""
    from libgran_gb300 import _abi as A
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    mat, d = workload_desc(A.LG_PRECISION_FP64)
    o = O.OracleSystem(d, x0, v0, threads=threads)
    t = time.perf_counter()
    o.step(mat.dt, VV_PER_STEP, VV_PER_STEP)
    probe = time.perf_counter() - t
    periods = max(1, int(target_s / max(probe, 1e-6)))
    t = time.perf_counter()
    o.step(mat.dt, VV_PER_STEP * periods, VV_PER_STEP)
    el = time.perf_counter() - t
    steps = VV_PER_STEP * periods
    return {"value": N_PART * steps / el, "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "sample": "%d particles x %d velocity-Verlet steps (%d rebuild periods) of the same aggregate, %.1f s"
                      % (N_PART, steps, periods, el)}


def run_reference_arm(args, rank, world):
    """The reference's CPU path: the oracle (libgran's functors and loop restated in C, OpenMP over
    all host cores) on the same workload. Inputs come from the oracle's own generator, so this arm
    loads no library of the engine."""
    if rank != 0:
        return
    from libgran_gb300 import _abi as A
    from oracle import oracle as O
    x0, v0 = workload_state(O)
    threads = os.cpu_count() or 1
    mat, d = workload_desc(A.LG_PRECISION_FP64)
    o = O.OracleSystem(d, x0, v0, threads=threads)
    # a bounded sample per bench step keeps the whole run within a few minutes
    probe_t = time.perf_counter()
    o.step(mat.dt, 2, VV_PER_STEP)
    per_vv = (time.perf_counter() - probe_t) / 2
    vv_per_sample = max(2, min(VV_PER_STEP, int(4.0 / max(per_vv, 1e-6))))
    for _ in range(args.warmup):
        o.step(mat.dt, vv_per_sample, VV_PER_STEP)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        o.step(mat.dt, vv_per_sample, VV_PER_STEP)
        times.append(time.perf_counter() - t)
    total = sum(times)
    value = N_PART * vv_per_sample * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "rsa_aggregate_32768_contact_hamaker_verlet", "n_part": N_PART,
                   "vv_steps_per_sample": vv_per_sample, "precision": "fp64", "threads": threads},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                         "sample": "%d particles x %d velocity-Verlet steps per bench step (oracle port of libgran's "
                                   "functors and loop; libgran's own build needs its absent submodules)"
                                   % (N_PART, vv_per_sample)},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "native_libraries": repo_native_libraries(),
    }
    print(json.dumps(line), flush=True)


def accuracy_run(x0, v0, total=None, every=1000):
    """Config 1's accuracy run: total (10^4) velocity-Verlet steps of the 32768 aggregate in FP64
    and in mixed precision, side by side. Every `every` steps:
      * forces and torques of both paths at an identical state: fresh FP64 and mixed handles are
        built from the FP64 run's state (positions, velocities, orientations, spins; springs start
        from zero in both), and their construction force evaluations are compared (normwise
        relative error over the system);
      * one rebuild period (20 steps) of both fresh handles from that state: normwise relative
        difference of the displacements (float-float integration inside a run of steps, springs);
      * energy (kinetic + spring + Hamaker potential) of both long runs.
    Energy drift is reported relative to the initial total energy and to the initial kinetic
    energy (the Hamaker potential of the contacts is three orders of magnitude larger than the
    kinetic energy)."""
    from libgran_gb300 import _abi as A
    from libgran_gb300.system import System
    total = total or int(os.environ.get("LG_ACCURACY_STEPS", "10000"))
    mat, d64 = workload_desc(A.LG_PRECISION_FP64)
    _, dmx = workload_desc(A.LG_PRECISION_MIXED)
    run = {"fp64": System(d64, x0, v0), "mixed": System(dmx, x0, v0)}
    energy = {k: [] for k in run}
    ke0 = None
    checkpoints = []
    done = 0
    t0 = time.perf_counter()
    while True:
        for k, s in run.items():
            o = s.observables()
            energy[k].append(o["ke_total"] + o["potential_energy"])
            if ke0 is None:
                ke0 = o["ke_total"]
        st = run["fp64"].get_state()
        a = System(d64, *st)
        b = System(dmx, *st)
        fa, fb = a.get(A.LG_FIELD_A), b.get(A.LG_FIELD_A)
        ta, tb = a.get(A.LG_FIELD_ALPHA), b.get(A.LG_FIELD_ALPHA)
        cp = {"step": done, "force_rel_err": float(np.abs(fa - fb).max() / np.abs(fa).max()),
              "torque_rel_err": float(np.abs(ta - tb).max() / max(np.abs(ta).max(), 1e-300)),
              "live_contact_slots": int(a.pair_stats()["live_contact_slots"])}
        a.step(mat.dt, VV_PER_STEP, VV_PER_STEP)
        b.step(mat.dt, VV_PER_STEP, VV_PER_STEP)
        da, db = a.get(A.LG_FIELD_X) - st[0], b.get(A.LG_FIELD_X) - st[0]
        cp["period_displacement_rel_diff"] = float(np.abs(da - db).max() / np.abs(da).max())
        a.close()
        b.close()
        checkpoints.append(cp)
        if done >= total:
            break
        for s in run.values():
            s.step(mat.dt, every, VV_PER_STEP)
        done += every
    xa, xb = run["fp64"].get(A.LG_FIELD_X), run["mixed"].get(A.LG_FIELD_X)
    disp = np.abs(xa - x0).max()
    errs = {k: s.device_errors() for k, s in run.items()}
    for s in run.values():
        s.close()
    e = {k: np.array(v) for k, v in energy.items()}
    out = {
        "vv_steps": total, "checkpoint_every": every,
        "force_rel_err_max": max(c["force_rel_err"] for c in checkpoints),
        "torque_rel_err_max": max(c["torque_rel_err"] for c in checkpoints),
        "period_displacement_rel_diff_max": max(c["period_displacement_rel_diff"] for c in checkpoints),
        "energy_drift_rel_fp64": float(np.abs(e["fp64"] - e["fp64"][0]).max() / abs(e["fp64"][0])),
        "energy_drift_rel_mixed": float(np.abs(e["mixed"] - e["mixed"][0]).max() / abs(e["mixed"][0])),
        "energy_drift_over_ke0_fp64": float(np.abs(e["fp64"] - e["fp64"][0]).max() / ke0),
        "energy_drift_over_ke0_mixed": float(np.abs(e["mixed"] - e["mixed"][0]).max() / ke0),
        "energy_mixed_minus_fp64_over_ke0_max": float(np.abs(e["mixed"] - e["fp64"]).max() / ke0),
        "final_position_diff_over_max_displacement": float(np.abs(xa - xb).max() / disp),
        "device_errors": errs,
        "checkpoints": checkpoints,
        "energy_fp64": e["fp64"].tolist(), "energy_mixed": e["mixed"].tolist(), "ke0": ke0,
        "wall_s": time.perf_counter() - t0,
        "basis": "identical states: fresh FP64 and mixed handles built from the FP64 run's state every %d steps "
                 "(springs from zero in both); energies from the two independent %d-step runs" % (every, total),
    }
    return out


def time_path(precision, x0, v0, args, l2_flush, tune=False, kernel=None):
    """Device-timed K bench steps (each 20 VV steps, replayed as one CUDA graph) with CUDA events on
    the handle's stream; L2 is flushed before every timed bench step (the flush is outside the
    timed region). The force kernel's own duration is then measured on 2 further bench steps with
    events around every launch (no graphs), so the roofline uses the kernel time alone."""
    from libgran_gb300 import _abi as A
    from libgran_gb300.system import System
    mat, d = workload_desc(precision)
    if kernel is not None:
        d.force_kernel = kernel
    s = System(d, x0, v0)
    tuning = None
    if tune:  # the project autotuner picks the kernel family and shape on the live system
        s.autotune(mat.dt, probe_steps=VV_PER_STEP, rebuild_every=VV_PER_STEP, use_cache=False)
        tuning = s.tuning()
    for _ in range(args.warmup):
        s.step(mat.dt, VV_PER_STEP, VV_PER_STEP)
    l0 = s.launch_count()
    total_ms = 0.0
    for _ in range(args.steps):
        l2_flush()
        total_ms += s.step_timed(mat.dt, VV_PER_STEP, VV_PER_STEP)
    launches = s.launch_count() - l0
    s.enable_kernel_timing(True)
    s.force_kernel_time()
    for _ in range(2):
        l2_flush()
        s.step(mat.dt, VV_PER_STEP, VV_PER_STEP)
    kms, kcount = s.force_kernel_time()
    s.enable_kernel_timing(False)
    stats = s.pair_stats()
    errs = s.device_errors()
    return s, mat, {"ms": total_ms, "launches": launches, "kernel_ms": kms, "kernel_launches": kcount,
                    "pair_stats": stats, "device_errors": errs, "tuning": tuning}


def c0_section(steps=10000):
    """Config 0 as configured: 256 monomers (seed 0), sintered bonds + contact + full Hamaker, all
    pairs, velocities +-0.1 m/s, 10^4 velocity-Verlet steps -- on the GPU in FP64 (the automatic
    choice: pair-parallel kernel, bit-identical to the oracle) and in mixed precision, and on the
    host cores with the oracle (the full run). Reports particle-steps/s of each and whether the FP64
    end state equals the oracle's bit for bit."""
    from libgran_gb300 import _abi as A
    from libgran_gb300 import configs as K
    from libgran_gb300.system import System
    from oracle import oracle as O
    from libgran_gb300.system import generate_aggregate, generate_velocities
    mat = K.Material()
    n = 256
    # the GPU runs take the library's generator; the oracle run takes the oracle's own, which gives
    # the same bits
    x0, v0 = generate_aggregate(0, n, mat.r), generate_velocities(0, n, 0.1)
    out = {"n_part": n, "vv_steps": steps}
    xs = {}
    for name, prec in (("fp64", A.LG_PRECISION_FP64), ("mixed", A.LG_PRECISION_MIXED)):
        d = K.make_desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_FULL, contact=mat.contact(), sinter=mat.sinter(),
                        hamaker=mat.hamaker(), precision=prec)
        s = System(d, x0, v0)
        s.step(mat.dt, 100)  # graphs captured
        s2 = System(d, x0, v0)
        ms = s2.step_timed(mat.dt, steps)
        xs[name] = s2.get(A.LG_FIELD_X)
        out[name] = {"particle_steps_per_s": n * steps / (ms / 1e3), "us_per_step": 1e3 * ms / steps}
        s.close()
        s2.close()
    d = K.make_desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_FULL, contact=mat.contact(), sinter=mat.sinter(),
                    hamaker=mat.hamaker())
    threads = os.cpu_count() or 1
    o = O.OracleSystem(d, O.generate_aggregate(0, n, mat.r), O.generate_velocities(0, n, 0.1), threads=threads)
    t = time.perf_counter()
    o.step(mat.dt, steps)
    el = time.perf_counter() - t
    out["cpu_oracle"] = {"particle_steps_per_s": n * steps / el, "cores": threads, "s": el}
    out["fp64_end_state_equals_oracle"] = bool(np.array_equal(xs["fp64"], o.get(A.LG_FIELD_X)))
    xo = o.get(A.LG_FIELD_X)
    out["mixed_end_position_rel_diff"] = float(np.abs(xs["mixed"] - xo).max() / np.abs(xo - x0).max())
    return out


def kernel_name(t):
    from libgran_gb300 import _abi as A
    if t and t["force_kernel"] == A.LG_FORCE_KERNEL_PERSISTENT:
        return "forces_step_mixed (one persistent launch per step)"
    return "forces_mixed (contacts || hamaker -> finish)"


def tuning_desc(t):
    """The autotuner's pick as names (kernel family and shape)."""
    from libgran_gb300 import _abi as A
    if not t:
        return None
    names = {A.LG_FORCE_KERNEL_COMPACT: "compact", A.LG_FORCE_KERNEL_ROWGROUP: "rowgroup",
             A.LG_FORCE_KERNEL_PAIRS: "pairs", A.LG_FORCE_KERNEL_PERSISTENT: "persistent"}
    out = {"kernel": names.get(t["force_kernel"], str(t["force_kernel"])), "probe_ms_per_step": t["ms_per_step"]}
    if t["force_kernel"] == A.LG_FORCE_KERNEL_ROWGROUP:
        out["threads_per_row"] = t["threads_per_row"]
    if t["force_kernel"] == A.LG_FORCE_KERNEL_COMPACT:
        out["contact_lanes_per_row"] = t["threads_per_row"]
    if t["force_kernel"] == A.LG_FORCE_KERNEL_PERSISTENT:
        out.update(min_blocks_per_sm=t["step_min_blocks"], hamaker_slices=t["step_slices"],
                   items={0: "pulled", 1: "round robin", 2: "two launches side by side"}.get(t["step_assign"]))
    return out


def batched_section(args, l2_flush):
    """Batched workload: 4096 independent aggregates (log-normal sizes, median 256, clipped to
    32..2048, about 1 % clipped per side), sintered bonds + limited Hamaker + frictional contact for
    non-bonded pairs, velocity Verlet, one handle, 20-step rebuild periods replayed as CUDA graphs,
    force kernel chosen by the autotuner. Compared with launching a sample of the same aggregates
    one by one (one handle each)."""
    from libgran_gb300 import _abi as A
    from libgran_gb300 import configs as K
    from libgran_gb300.system import System
    mat = K.Material()
    count = int(os.environ.get("LG_BATCH_COUNT", "4096"))
    sizes = K.lognormal_sizes(count, 256, 32, 2048, seed=2)
    t0 = time.perf_counter()
    x0, v0 = K.seeded_aggregates(sizes, 2, mat.r)
    out = {"systems": count, "particles": int(sizes.sum()), "median_size": float(np.median(sizes)),
           "max_size": int(sizes.max())}

    def desc(n, prec):
        return K.make_desc(n, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, contact=mat.contact(), sinter=mat.sinter(),
                           hamaker=mat.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r, precision=prec)
    res = {}
    for name, prec in (("mixed", A.LG_PRECISION_MIXED), ("fp64", A.LG_PRECISION_FP64)):
        s = System(desc(int(sizes.sum()), prec), x0, v0, sizes=sizes)
        kern, T = s.autotune(mat.dt, probe_steps=VV_PER_STEP, rebuild_every=VV_PER_STEP)
        tuned = s.tuning()
        for _ in range(args.warmup):
            s.step(mat.dt, VV_PER_STEP, VV_PER_STEP)
        ms = 0.0
        steps = max(2, args.steps // (1 if name == "mixed" else 2))
        for _ in range(steps):
            l2_flush()
            ms += s.step_timed(mat.dt, VV_PER_STEP, VV_PER_STEP)
        res[name] = {"value": sizes.sum() * VV_PER_STEP * steps / (ms / 1e3), "ms_per_step": ms / steps,
                     "tuning": tuning_desc(tuned), "device_errors": s.device_errors()}
        s.close()
    # one by one: a sample of the aggregates, each its own handle, launched in turn
    sample = min(64, count)
    handles = [System(desc(int(sizes[a]), A.LG_PRECISION_MIXED),
                      x0[int(sizes[:a].sum()):int(sizes[:a + 1].sum())],
                      v0[int(sizes[:a].sum()):int(sizes[:a + 1].sum())]) for a in range(sample)]
    for _ in range(3):  # both list parities replayed once, so the graphs are captured before timing
        for h in handles:
            h.step(mat.dt, VV_PER_STEP, VV_PER_STEP)
    import torch
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(2):
        for h in handles:
            h.step(mat.dt, VV_PER_STEP, VV_PER_STEP)
    for h in handles:
        h.device_errors()  # synchronises each handle's stream
    el = time.perf_counter() - t
    res["one_by_one_mixed"] = {"value": sizes[:sample].sum() * VV_PER_STEP * 2 / el, "sample_systems": sample}
    for h in handles:
        h.close()
    out.update(res)
    out["batched_over_one_by_one"] = res["mixed"]["value"] / res["one_by_one_mixed"]["value"]
    out["setup_s"] = time.perf_counter() - t0
    return out


def e2e_path(s, mat, args, x0, v0):
    """Same metric through the public API with host buffers: every bench step uploads the state
    (x, v, theta, omega) from pinned host memory, runs 20 VV steps and reads back the state and
    its observables (kinetic energies, momenta, centre of mass, radius of gyration: the quantities
    libgran's compute_energy / mass_distribution helpers report); host<->device copies are inside
    the timed region."""
    import torch
    from libgran_gb300 import _abi as A
    fields = (A.LG_FIELD_X, A.LG_FIELD_V, A.LG_FIELD_THETA, A.LG_FIELD_OMEGA)
    host = {f: torch.from_numpy(np.ascontiguousarray(s.get(f))).pin_memory() for f in fields}
    views = tuple(host[f].numpy() for f in fields)  # numpy views of the pinned buffers, made once
    times = []
    for k in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        s.set_state(*views)
        s.step(mat.dt, VV_PER_STEP, VV_PER_STEP)
        s.get_state(out=views)
        obs = s.observables(A.LG_OBS_STATE)
        t = time.perf_counter() - t
        if k >= args.warmup:
            times.append(t)
    h2d = 4 * N_PART * 3 * 8
    d2h = 4 * N_PART * 3 * 8 + 8 * 19
    return {"value": N_PART * VV_PER_STEP * len(times) / sum(times), "unit": "particle-steps/s",
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}, obs


def run_gb300(args, rank, world):
    import torch
    from libgran_gb300 import _abi as A
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    x0, v0 = workload_state()
    flush_buf = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def l2_flush():
        flush_buf.fill_(1.0)
        torch.cuda.synchronize()

    # plain FP64 first (its number is reported beside the headline)
    s64, mat, t64 = time_path(A.LG_PRECISION_FP64, x0, v0, args, l2_flush)
    s64.close()
    # the FP64 kernel with reciprocals instead of repeated divisions (within 1e-12, opt-in)
    s64f, _, t64f = time_path(A.LG_PRECISION_FP64, x0, v0, args, l2_flush, kernel=A.LG_FORCE_KERNEL_FP64_FAST)
    s64f.close()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    sm, mat, tm = time_path(A.LG_PRECISION_MIXED, x0, v0, args, l2_flush, tune=True)
    clk = clocks.stop()
    torch.cuda.synchronize()
    def amax(v):
        t = torch.tensor([v], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t[0])
    if dist:
        dist.barrier()
    units = N_PART * VV_PER_STEP * args.steps
    value, tm["ms"] = combine_ranks(tm["ms"], units, world, amax if dist else None)
    value64, t64["ms"] = combine_ranks(t64["ms"], units, world, amax if dist else None)
    value64f, t64f["ms"] = combine_ranks(t64f["ms"], units, world, amax if dist else None)
    e2e, obs = e2e_path(sm, mat, args, x0, v0)
    e2e["value"] *= world
    sm.close()
    if rank != 0:
        return
    acc = accuracy_run(x0, v0) if os.environ.get("LG_BENCH_ACCURACY", "1") != "0" else None
    # roofline of the dominant kernel (mixed force kernel)
    ps = tm["pair_stats"]
    z_list = ps["mean_row_length"]
    z_act = (ps["live_contact_slots"] + ps["bonded_slots"]) / N_PART
    bytes_per_particle = 168.0 + 4.0 * z_list + 144.0 * z_act
    # duration of one force evaluation in the steady state: the graph-replayed timed region per
    # velocity-Verlet step (an upper bound: it also holds the amortised list rebuild and the
    # period's first half kick); the eager per-launch time (events around every launch, no graphs)
    # is reported beside it
    per_launch_ms = tm["ms"] / (args.steps * VV_PER_STEP)
    eager_eval_ms = tm["kernel_ms"] / max(tm["kernel_launches"], 1)
    achieved = bytes_per_particle * N_PART / (per_launch_ms / 1e3) / 1e9
    peaks = measured_peaks()
    peak = peaks.get("hbm_gbs", 6800.0)
    traffic = read_profile_traffic("forces_mixed_c1")
    cpu = cpu_reference_rate(x0, v0, target_s=float(os.environ.get("LG_CPU_SAMPLE_S", "12")))
    c0 = c0_section() if os.environ.get("LG_BENCH_C0", "1") != "0" else None
    batched = None
    if os.environ.get("LG_BENCH_BATCHED", "1") != "0":
        batched = batched_section(args, l2_flush)
    restruct = None
    if os.environ.get("LG_BENCH_RESTRUCT", "1") != "0":
        restruct = restructuring_section(args, l2_flush)
    serving = None
    if os.environ.get("LG_BENCH_SERVING", "1") != "0":
        lams = [float(v) for v in os.environ.get("LG_SERVE_LAMBDAS", "8,32,64,128").split(",")]
        dur = float(os.environ.get("LG_SERVE_SECONDS", "8"))
        per = int(os.environ.get("LG_SERVE_SLOTS_PER_CLASS", "24")) or None
        serving = {"sweep": [serving_section(lam, dur, slots_per_class=per) for lam in lams],
                   "accuracy": serving_force_error()}
    line = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": tm["ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": "rsa_aggregate_32768_contact_hamaker_verlet", "n_part": N_PART,
                   "vv_steps_per_step": VV_PER_STEP, "rebuild_every": VV_PER_STEP, "r_verlet": "4.5r",
                   "hamaker_cutoff": "centre distance 4r (surface gap 2r)", "precision": "mixed",
                   "l2": "flushed (512 MiB write) before every timed step", "parallelism": "replicas" if world > 1
                   else "single GPU"},
        "plain_fp64": {"value": value64, "unit": "particle-steps/s", "ms_per_step": t64["ms"] / args.steps,
                       "force_kernel_ms_per_launch": t64["kernel_ms"] / max(t64["kernel_launches"], 1)},
        "plain_fp64_fast": {"value": value64f, "unit": "particle-steps/s", "ms_per_step": t64f["ms"] / args.steps,
                            "force_kernel_ms_per_launch": t64f["kernel_ms"] / max(t64f["kernel_launches"], 1),
                            "kernel": "LG_FORCE_KERNEL_FP64_FAST (per-step forces within 1e-12 of the reference's)"},
        "mixed_over_fp64": value / value64,
        "mixed_over_fp64_fast": value / value64f,
        "accuracy": acc,
        "e2e": e2e,
        "gpu_launches": tm["launches"],
        "tuning": tuning_desc(tm["tuning"]),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": kernel_name(tm["tuning"]), "bytes_per_particle": bytes_per_particle,
                     "per_launch_ms": per_launch_ms, "per_launch_basis": "graph-replayed timed region per VV step",
                     "eager_eval_ms": eager_eval_ms, "peak_source": "measured" if peaks else "fallback"},
        "cpu_baseline": cpu,
        "clocks": {"sm_mhz": clk["sm_mhz"], "sm_max_mhz": clk["sm_max_mhz"], "reasons": clk["reasons"]},
        "device_errors": tm["device_errors"],
        "c0": c0,
        "batched": batched,
        "restructuring": restruct,
        "serving": serving,
    }
    print(json.dumps(line), flush=True)


def restructuring_section(args, l2_flush, steps=None, count=None):
    """Batched restructuring: aggregates of log-uniform 128..4096 monomers, sintered bonds that break
    above 10 nN (each bond its own strength), frictional contact for non-bonded pairs, limited
    Hamaker, each pushed by a rigid plane wall moving at 1 m/s (surface contact k_n = 1e4 N/m). Runs
    the batch in mixed precision and in FP64 (the FP64 path is bit-identical to the FP64 oracle)
    and reports the broken-bond fraction and final radius of gyration of both, their relative
    difference, and particle-steps/s."""
    from libgran_gb300 import _abi as A
    from libgran_gb300 import configs as K
    from libgran_gb300.system import System
    mat = K.Material()
    count = count or int(os.environ.get("LG_RESTRUCT_COUNT", "1024"))
    steps = steps or int(os.environ.get("LG_RESTRUCT_STEPS", "2000"))
    sizes = K.loguniform_sizes(count, 128, 4096, seed=3)
    x0, v0 = K.seeded_aggregates(sizes, 3, mat.r)
    x0 = K.rest_on_wall(x0, sizes, mat.r)
    wall = K.wall_facet(mat, extent=50 * mat.r)
    out = {"systems": count, "particles": int(sizes.sum()), "vv_steps": steps}
    res = {}
    for name, prec in (("mixed", A.LG_PRECISION_MIXED), ("fp64", A.LG_PRECISION_FP64)):
        d = K.make_desc(int(sizes.sum()), A.LG_BINARY_BREAKING_SINTER, A.LG_HAMAKER_LIMITED, contact=mat.contact(),
                        sinter=mat.sinter(), hamaker=mat.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r,
                        precision=prec, n_facets=1, facet_auto_move=1, force_kernel=A.LG_FORCE_KERNEL_COMPACT)
        probe = System(d, x0, v0, facets=[wall], sizes=sizes)
        nb = len(probe.bonds()) // 2
        probe.close()
        s = System(d, x0, v0, facets=[wall], neck=np.full(nb, 1e-8), sizes=sizes)
        b0 = len(s.bonds())
        l2_flush()
        ms = s.step_timed(mat.dt, steps, VV_PER_STEP)
        obs = s.batch_observables()
        b1 = len(s.bonds())
        res[name] = {"particle_steps_per_s": sizes.sum() * steps / (ms / 1e3),
                     "broken_fraction": (b0 - b1) / max(b0, 1),
                     "rg_mean": float(np.mean([o["radius_of_gyration"] for o in obs])),
                     "rg": np.array([o["radius_of_gyration"] for o in obs]), "device_errors": s.device_errors()}
        s.close()
    rg_rel = float(np.max(np.abs(res["mixed"]["rg"] - res["fp64"]["rg"]) / res["fp64"]["rg"]))
    for k in res:
        res[k].pop("rg")
    out.update(res)
    out["rg_max_rel_diff_mixed_vs_fp64"] = rg_rel
    bf = res["fp64"]["broken_fraction"]
    out["broken_fraction_rel_diff"] = abs(res["mixed"]["broken_fraction"] - bf) / bf if bf > 0 else None
    return out


SLOT_CLASSES = (128, 256, 512, 1024, 2048, 4096, 8192)


def serving_section(lam, duration_s, seed=4, budget_bytes=150 * 10 ** 9, slots_per_class=None):
    """Serving workload: Poisson arrivals at rate lam (requests/s) for duration_s seconds; each
    request an aggregate of log-uniform 64..8192 monomers with its own seed and a step budget drawn
    uniformly from 2e3..2e4 (multiples of 20), mixed precision, sintered bonds + contact + limited
    Hamaker; a 150 GB device-memory budget. Resident requests occupy slots of one batch (the
    default size classes) and advance in the same launches. Reports request latency percentiles,
    the sustained particle-steps/s of the whole run (submission of the first request to retirement
    of the last), mean slot occupancy and resident particles."""
    from libgran_gb300 import _abi as A
    from libgran_gb300 import configs as K
    from libgran_gb300.serving import Server
    from libgran_gb300.system import generate_aggregate, generate_velocities
    mat = K.Material()
    d = serving_template(A.LG_PRECISION_MIXED)
    rng = np.random.default_rng(seed)
    t, arrivals = 0.0, []
    while True:
        t += rng.exponential(1.0 / lam)
        if t > duration_s:
            break
        n = int(K.loguniform_sizes(1, 64, 8192, seed=int(rng.integers(1 << 31)))[0])
        steps = int(rng.integers(100, 1001)) * 20
        arrivals.append((t, n, steps, len(arrivals)))
    # inputs are generated before the clock starts (a client would send them)
    inputs = [(generate_aggregate((4 << 32) + k, n, mat.r), generate_velocities((4 << 32) + k, n, 0.1))
              for (_, n, _, k) in arrivals]
    srv = Server(d, budget_bytes=budget_bytes, dt=mat.dt)
    if slots_per_class:
        srv.set_slots([c for c in SLOT_CLASSES for _ in range(int(slots_per_class))])
    t0 = time.perf_counter()
    nxt = 0
    busy, resident = [], []
    while True:
        now = time.perf_counter() - t0
        while nxt < len(arrivals) and arrivals[nxt][0] <= now:
            _, n, steps, k = arrivals[nxt]
            srv.submit(inputs[k][0], inputs[k][1], steps)
            nxt += 1
        a, q, _ = srv.tick()
        st = srv.stats()
        busy.append(st["slots_busy"])
        resident.append(st["resident_particles"])
        if nxt >= len(arrivals) and a == 0 and q == 0:
            break
        if a == 0 and q == 0 and nxt < len(arrivals):
            time.sleep(max(0.0, min(0.01, arrivals[nxt][0] - (time.perf_counter() - t0))))
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    return {"lambda_per_s": lam, "requests": len(arrivals), "completed": st["completed"], "failed": st["failed"],
            "p50_latency_ms": st["p50_latency_ms"], "p99_latency_ms": st["p99_latency_ms"],
            "max_latency_ms": st["max_latency_ms"], "particle_steps_per_s": st["particle_steps"] / wall,
            "offered_particle_steps_per_s": sum(n * steps for (_, n, steps, _) in arrivals) / duration_s,
            "wall_s": wall, "peak_bytes": st["peak_bytes"], "budget_bytes": budget_bytes, "slots": st["slots"],
            "slot_particles": st["slot_particles"], "mean_slots_busy": float(np.mean(busy)) if busy else 0.0,
            "mean_resident_particles": float(np.mean(resident)) if resident else 0.0,
            "gpu_busy_frac": st["device_ms"] / 1e3 / wall, "periods": st["periods"],
            "resident_particle_steps_per_device_s": st["particle_steps"] / max(st["device_ms"] / 1e3, 1e-9)}


def serving_template(precision):
    from libgran_gb300 import _abi as A
    from libgran_gb300 import configs as K
    mat = K.Material()
    return K.make_desc(1, A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, contact=mat.contact(), sinter=mat.sinter(),
                       hamaker=mat.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r, precision=precision,
                       max_neighbors=96)


def serving_force_error():
    """Mixed against FP64 forces and torques of serving requests at identical states: requests of
    64, 1024 and 8192 monomers (the size range) as submitted, both precisions' construction force
    evaluations (normwise relative error over the request)."""
    from libgran_gb300 import _abi as A
    from libgran_gb300 import configs as K
    from libgran_gb300.system import System, generate_aggregate, generate_velocities
    mat = K.Material()
    out = {"force_rel_err_max": 0.0, "torque_rel_err_max": 0.0, "sizes": [64, 1024, 8192]}
    for k, n in enumerate(out["sizes"]):
        x0, v0 = generate_aggregate((4 << 32) + 10 ** 6 + k, n, mat.r), generate_velocities((4 << 32) + 10 ** 6 + k, n, 0.1)
        res = []
        for prec in (A.LG_PRECISION_FP64, A.LG_PRECISION_MIXED):
            d = serving_template(prec)
            d.n_part = n
            s = System(d, x0, v0)
            res.append((s.get(A.LG_FIELD_A), s.get(A.LG_FIELD_ALPHA)))
            s.close()
        (fa, ta), (fb, tb) = res
        out["force_rel_err_max"] = max(out["force_rel_err_max"], float(np.abs(fa - fb).max() / np.abs(fa).max()))
        out["torque_rel_err_max"] = max(out["torque_rel_err_max"],
                                        float(np.abs(ta - tb).max() / max(np.abs(ta).max(), 1e-300)))
    return out


def combine_ranks(ms, units_per_rank, world, all_reduce_max=None):
    """Whole-job throughput of `world` replicas: every rank processed units_per_rank units; the job
    time is the slowest rank's (max over ranks)."""
    if world > 1 and all_reduce_max is not None:
        ms = all_reduce_max(ms)
    return world * units_per_rank / (ms / 1e3), ms


def run_profile(args):
    """Profiling driver (no timing output): build the workload and run --warmup + --steps bench
    steps of one path, so that ncu can capture its kernels."""
    import torch
    from libgran_gb300 import _abi as A
    from libgran_gb300.system import System
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    prec = A.LG_PRECISION_MIXED if args.profile in ("mixed", "c0-mixed") else A.LG_PRECISION_FP64
    if args.profile.startswith("c0"):
        # the 256-monomer all-pairs aggregate (sintered bonds + contact + full Hamaker), 100 steps a
        # bench step, no list
        from libgran_gb300 import configs as K
        from libgran_gb300.system import generate_aggregate, generate_velocities
        mat = K.Material()
        x0, v0 = generate_aggregate(0, 256, mat.r), generate_velocities(0, 256, 0.1)
        d = K.make_desc(256, A.LG_BINARY_SINTER, A.LG_HAMAKER_FULL, contact=mat.contact(), sinter=mat.sinter(),
                        hamaker=mat.hamaker(), precision=prec)
        s = System(d, x0, v0)
        s.step(mat.dt, 100 * (args.warmup + args.steps))
        print(json.dumps({"profile": args.profile, "vv_steps": 100 * (args.warmup + args.steps),
                          "device_errors": s.device_errors(), "launches": s.launch_count()}))
        return
    if args.profile == "batched-mixed":
        # the batched workload: 4096 aggregates (LG_BATCH_COUNT; median 256 monomers), sintered bonds
        # + limited Hamaker + contact, mixed precision, the compacted kernels
        from libgran_gb300 import configs as K
        mat = K.Material()
        sizes = K.lognormal_sizes(int(os.environ.get("LG_BATCH_COUNT", "4096")), 256, 32, 2048, seed=2)
        x0, v0 = K.seeded_aggregates(sizes, 2, mat.r)
        d = K.make_desc(int(sizes.sum()), A.LG_BINARY_SINTER, A.LG_HAMAKER_LIMITED, contact=mat.contact(),
                        sinter=mat.sinter(), hamaker=mat.hamaker(), pairs=A.LG_PAIRS_VERLET, r_verlet=4.5 * mat.r,
                        precision=A.LG_PRECISION_MIXED)
        s = System(d, x0, v0, sizes=sizes)
        s.step(mat.dt, VV_PER_STEP * (args.warmup + args.steps), VV_PER_STEP)
        print(json.dumps({"profile": args.profile, "vv_steps": VV_PER_STEP * (args.warmup + args.steps),
                          "device_errors": s.device_errors(), "launches": s.launch_count()}))
        return
    x0, v0 = workload_state()
    mat, d = workload_desc(prec)
    if args.kernel is not None:
        d.force_kernel = {"compact": A.LG_FORCE_KERNEL_COMPACT, "persistent": A.LG_FORCE_KERNEL_PERSISTENT,
                          "fp64fast": A.LG_FORCE_KERNEL_FP64_FAST}[args.kernel]
    s = System(d, x0, v0)
    if args.shape:
        s.set_step_shape(*[int(v) for v in args.shape.split(",")])
    s.step(mat.dt, VV_PER_STEP * (args.warmup + args.steps), VV_PER_STEP)
    print(json.dumps({"profile": args.profile, "vv_steps": VV_PER_STEP * (args.warmup + args.steps),
                      "device_errors": s.device_errors(), "launches": s.launch_count()}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--profile", default=None, choices=[None, "mixed", "fp64", "c0-fp64", "c0-mixed", "batched-mixed"],
                    help="profiling driver: run one path without timing (c0-*: the 256-monomer all-pairs case)")
    ap.add_argument("--kernel", default=None, choices=[None, "compact", "persistent", "fp64fast"],
                    help="profiling driver: force kernel (compact / persistent: mixed; fp64fast: FP64)")
    ap.add_argument("--shape", default=None,
                    help="profiling driver, persistent kernel: min_blocks,slices,assign")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    if args.profile:
        run_profile(args)
        return
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
        return
    run_gb300(args, rank, world)


if __name__ == "__main__":
    main()
