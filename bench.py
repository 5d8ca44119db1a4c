"""Benchmark: particle-steps/s of the DEM step on one GB300.

Workload (default): the granular column collapse -- 50,000 convex hull grains
(semi-axes U[0.5, 1.5] cm, Avalanche law, linked-cell neighbour list) in a
random packing (bulk solid fraction ~0.52, coordination ~5) that fills a
0.5 x 0.5 m column about 1.1 m high on a rigid floor.  The packing is built
on the CPU by the seeded packer (rockable_gb300/host/rk_pack.cpp, through
scenes.column_collapse); its grains touch but carry no load.  Before any
timing the pile settles by gravity between four walls with the scene's laws,
stiffnesses and time step (`--load-steps` DEM steps with numerical damping,
scenes.loaded), then the walls are removed: every form
starts from that settled, contact-rich column at release, contact history
included.  The reference arm (`--impl reference`), which
must not load the GPU library, times the CPU path on the packing at t = 0;
the `cpu_baseline` leg times it on the same state, and
config.cpu_on_settled_state on the settled one the GPU forms run on.

One bench step is one segment of `--segment` DEM steps (100: the fixed
schedule's interVerlet), each DEM step one pass of the velocity-Verlet step
loop (drift, narrow phase + force law, ordered resultants, accelerations,
half-kick), so every timed bench step of a fixed-schedule form holds exactly
one neighbour-list rebuild; the learned-skin forms rebuild when they decide
to, inside the same DEM steps.  `value` counts free bodies x DEM steps.

Legs of one run (rank 0 prints one JSON line):
  value       : device-timed throughput of the headline form over K bench
                steps, state resident in HBM (CUDA events on the engine's
                stream); every form is in `forms`;
  e2e         : the same metric through the C ABI with host-owned state:
                every bench step uploads the bodies' kinematics from pinned
                host memory, runs rk_step(segment) and downloads the result;
  roofline    : the headline form's dominant kernel (narrow phase or
                resultants), algorithmic bytes over its event-timed launch
                duration against the measured HBM copy bandwidth, with the
                ncu DRAM traffic and FP64 rate from profiles/;
  cpu_baseline: the oracle (CPU restatement of the reference path, OpenMP on
                the host's cores) on a bounded sample of the same segment;
  iso         : the 200k-grain isotropic compression (six servo walls at
                100 kPa), plain FP64 and the headline form, with its own CPU
                sample (the >= 50x target);
  rockfall    : the breakable bonded rockfall (40 blocks x 500 grains,
                Weibull vertex bonds made by the C++ host at load, 30 degree
                slope, 10 m/s), plain FP64 and mixed, with their broken sets;
  batched     : many independent slope scenes in one context.
`--impl reference` times the CPU path alone on the column workload and never
loads the GPU library.
"""
import argparse
import json
import os
import platform
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s @1 GB300: plain FP64 vs mixed+learned-skin, <=1e-4 rel force err"
TUNE_STEPS = 10  # untimed block-size tuning steps (rk_set_autotune, 2 rounds of 5 sizes)
PROFILE = os.path.join(ROOT, "profiles", "step_kernels_column_30k_headline.md")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20, help="timed bench steps (segments)")
    ap.add_argument("--warmup", type=int, default=5, help="untimed bench steps before them")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--segment", type=int, default=100, help="DEM steps per bench step")
    ap.add_argument("--n", type=int, default=50000, help="grains of the column")
    ap.add_argument("--load-steps", type=int, default=50000,
                    help="damped DEM steps (2 x dt: 0.1 s) that settle the column between walls before the release")
    ap.add_argument("--iso-load-steps", type=int, default=40000,
                    help="damped DEM steps (0.02 s) of servo compression before the box is timed")
    ap.add_argument("--forms", default="plain_fp64,mixed,mixed_learned_skin_exact",
                    help="comma list of the forms to time (the last one is the headline)")
    ap.add_argument("--iso-n", type=int, default=200000, help="grains of the compression box (0: skip)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="budget of each CPU sample")
    ap.add_argument("--ref-seconds", type=float, default=150.0, help="budget of the reference arm's timed steps")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--ncu-window", default="",
                    help="form whose extra window (a rebuild and one segment, after its timed steps) is bracketed "
                         "by cuProfilerStart/Stop, for ncu --profile-from-start off")
    ap.add_argument("--rock-clusters", type=int, default=40,
                    help="500-grain bonded blocks of the rockfall workload (0: skip)")
    ap.add_argument("--batch-scenes", type=int, default=256, help="scenes of the batched slope workload (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=100)
    ap.add_argument("--batch-settle", type=int, default=3000)
    return ap.parse_args()


# ------------------------------------------------------------------ host --
def guarded(fn, *args):
    """A secondary workload of the bench line: its failure is reported in
    its own object (with the error) instead of losing the headline line."""
    try:
        return fn(*args)
    except Exception as ex:  # the engine's RkError, a memory limit, ...
        import traceback
        traceback.print_exc()
        return {"error": "%s: %s" % (type(ex).__name__, ex)}


def cu_profiler(on):
    """cuProfilerStart / cuProfilerStop (CUDA driver API) on the current
    context: the window a profiler started with --profile-from-start off
    records."""
    import ctypes
    lib = ctypes.CDLL("libcuda.so.1")
    rc = (lib.cuProfilerStart if on else lib.cuProfilerStop)()
    if rc != 0:
        raise RuntimeError("cuProfiler%s failed: %d" % ("Start" if on else "Stop", rc))


def cpu_info():
    """Model and logical cores of this host (lscpu when present)."""
    model = platform.processor() or platform.machine()
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() in ("Model name", "Model"):
                v = line.split(":", 1)[1].strip()
                if v and not v.isdigit():
                    model = v
                    break
    except Exception:
        pass
    return {"model": model, "logical_cores": os.cpu_count(), "machine": platform.machine()}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_constants():
    """Per-unit figures of the headline kernels from the committed ncu
    summary: lines `bench: <key> = <value>` (DRAM bytes and FP64 operations
    per entry / per body, with the capture they come from)."""
    out = {}
    try:
        for line in open(PROFILE):
            if line.startswith("bench:") and "=" in line:
                k, v = line[len("bench:"):].split("=", 1)
                out[k.strip()] = float(v.split()[0])
    except Exception:
        pass
    return out


def fp64_peak():
    """Measured FP64 peak of this GPU: a cuBLAS DGEMM burst (4096^3, best of
    5), the FP64 counterpart of the driver's bf16 GEMM peak."""
    try:
        import torch
        a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
        b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
        torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 1e30
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a, b
        return 2.0 * 4096 ** 3 / (best / 1e3) / 1e12
    except Exception:
        return None


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.proc = None
        self.out = None

    def start(self):
        try:
            self.out = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]],
                stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        self.out.flush()
        rows = [l.split(",") for l in open(self.out.name).read().strip().split("\n") if l.strip()]
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) >= 9:
                for k, nm in enumerate(names):
                    if "Active" in r[5 + k] and "Not" not in r[5 + k]:
                        reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def dist_setup():
    """One process per GPU under torchrun (RANK / LOCAL_RANK / WORLD_SIZE /
    MASTER_* from the environment): NCCL with a GPU, gloo without one (the
    CPU tests of the multi-rank path).  Returns (rank, world size, module)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    backend = "gloo"
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
        backend = "nccl"
    dist.init_process_group(backend)
    return rank, ws, dist


def rank_max(x, dist):
    """The largest x over the ranks (the slowest replica's time sets the job's)."""
    if not dist:
        return float(x)
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(ws, units_per_rank, steps, ms):
    """Whole-job throughput: every rank's units over the slowest rank's time
    (replicas: each rank runs the full workload on its own GPU)."""
    return ws * units_per_rank * steps / (ms / 1000.0)


def pinned(shape):
    """Pinned host buffer (page-locked through torch when available)."""
    try:
        import torch
        return torch.empty(int(np.prod(shape)), dtype=torch.float64, pin_memory=True).numpy().reshape(shape)
    except Exception:
        return np.zeros(shape)


# ------------------------------------------------------------- CPU path --
def cpu_segments(scene, segment, count, budget_s, warm=0):
    """The oracle (OpenMP over the host's cores) on `count` bench steps of
    the scene from its initial state: each a full neighbour-list rebuild, timed,
    and a sample of s DEM steps, timed; the segment's time is the rebuild plus
    segment / s times the sample (linear extrapolation of the steps; s is
    chosen from a first measurement so that all of it fits the budget).
    `warm` untimed bench steps (one DEM step each) come first.  Returns the
    segment times (s), s, the rebuild and step times, and the oracle."""
    from oracle import oracle
    from rockable_gb300 import scenes
    oracle.build()
    d = tempfile.mkdtemp(prefix="rk_cpu_")
    conf = scenes.write_conf(scene, d)
    drv = os.path.join(d, "drivingSystem.txt")
    o = oracle.Oracle(conf, driving=drv if os.path.exists(drv) else None)
    t0 = time.perf_counter()
    o.update_nl()
    t_rb = time.perf_counter() - t0
    t0 = time.perf_counter()
    o.run(1)
    t_st = time.perf_counter() - t0
    per = budget_s / max(1, count)
    s = int(max(1, min(segment, (per - t_rb) / max(t_st, 1e-9))))
    o.run(warm)  # the untimed bench steps: one DEM step each (they only warm the caches)
    segs, rbs, sts = [], [], []
    for k in range(count):
        t0 = time.perf_counter()
        o.update_nl()
        rb = time.perf_counter() - t0
        t0 = time.perf_counter()
        o.run(s)
        st = (time.perf_counter() - t0) / s
        segs.append(rb + segment * st)
        rbs.append(rb)
        sts.append(st)
    return segs, s, float(np.mean(rbs)), float(np.mean(sts)), o


def cpu_threads():
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def cpu_baseline(scene, segment, budget_s, label):
    """Bounded CPU sample of one bench step of the workload (reported only)."""
    nfree = len(scene["bodies"]["mass"]) - scene["n_driven"]
    segs, s, rb, st, o = cpu_segments(scene, segment, 1, budget_s)
    v = nfree * segment / float(np.mean(segs))
    return {"value": v, "unit": "particle-steps/s", "cores": cpu_threads(), "kind": "port", "cpu": cpu_info(),
            "sample": ("%s: one neighbour-list rebuild (%.2f s) and %d DEM steps (%.4f s each) of the "
                       "%d-body scene; the %d-step segment's time is the rebuild plus %d x the step time "
                       "(linear extrapolation)" % (label, rb, s, st, o.n, segment, segment))}


def run_reference(a, rank):
    """The reference's CPU path (the oracle: restatement of the reference
    step loop, OpenMP over all host threads) on the column workload from its
    initial state; W untimed bench steps, then exactly K timed ones, each a
    sampled segment (cpu_segments).  Never loads the GPU library."""
    if rank != 0:
        return
    from rockable_gb300 import scenes
    # the GPU arm's packing before its gravity load (which runs on the GPU):
    # the same grains, walls already removed
    scene = scenes.column_collapse(n=a.n)
    nfree = len(scene["bodies"]["mass"]) - scene["n_driven"]
    segs, s, rb, st, o = cpu_segments(scene, a.segment, a.steps, a.ref_seconds, warm=a.warmup)
    T = float(np.sum(segs))
    value = nfree * a.segment * a.steps / T
    threads = cpu_threads()
    sample = ("every bench step: one full neighbour-list rebuild (mean %.2f s) and %d DEM steps (mean %.4f s each) "
              "of the %d-body column from t = 0, the %d-step segment's time being the rebuild plus %d x the step "
              "time (linear extrapolation); %d untimed bench steps (one DEM step each) first" % (
                  rb, s, st, o.n, a.segment, a.segment, a.warmup))
    out = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": a.gpus, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": 1000.0 * T / max(1, a.steps), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
           "impl": "reference",
           "config": {"workload": scene["name"], "law": scene["law"], "bodies": int(o.n), "free_bodies": int(nfree),
                      "dem_steps_per_step": a.segment,
                      "state": ("the packed column at t = 0, before the gravity load that the GPU arm runs on the "
                                "GPU (this arm does not load the GPU library); the GPU arm's cpu_baseline times the "
                                "same CPU path on the loaded state"),
                      "cpu": cpu_info()},
           "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------- GPU path --
SKIN = {"plain_fp64": None, "mixed": None, "mixed_learned_skin": "ref", "mixed_learned_skin_exact": "exact",
        "plain_fp64_learned_skin_exact": "exact"}


def engine(scene, form, dev, skin=None):
    """A context holding the scene at its initial state, ready to step."""
    from rockable_gb300 import scenes
    from rockable_gb300.abi import GpuScene, RK_FORM_FP64, RK_FORM_MIXED
    e = GpuScene(device=dev, form=RK_FORM_FP64 if form.startswith("plain") else RK_FORM_MIXED)
    e.upload_shapes(scene["shape_tables"])
    e.upload_bodies(scene["bodies"], scene["n_driven"])
    if scene.get("scene_of") is not None:
        e.set_scenes(scene["scene_of"])
    scenes.set_scene_params(e, scene)
    if scene.get("entries") is not None:  # a loaded state: its contacts and their history
        e.upload_entries(scene["entries"])
    if skin:
        d = scene["dVerlet"]
        # the interval stays within 3x the fixed schedule's, so that the
        # network (which proposes it) sees a window every few hundred steps
        e.set_skin(use_mlp=True, skin_min=0.1 * d, skin_max=4.0 * d, dverlet_ratio=2.0, interval_min=2,
                   interval_max=3 * int(round(scene["interVerlet"] / scene["dt"])), seed=3,
                   exact_contacts=(skin == "exact"))
    elif scene.get("entries") is None:
        e.update_nl()
    e.set_graphs(True)
    return e


def time_form(scene, label, a, dev, dist, ws, steps, warmup):
    """One form: tuning steps and `warmup` untimed bench steps from the
    scene's initial state, then exactly `steps` timed bench steps (one
    rk_step call, CUDA events on the context stream, barrier and sync on both
    sides), then one profiled segment.  Returns the context and the record."""
    nfree = len(scene["bodies"]["mass"]) - scene["n_driven"]
    e = engine(scene, label, dev, SKIN[label])
    e.autotune(2)
    e.step(TUNE_STEPS)
    if warmup:
        e.step(warmup * a.segment)
    clocks = Clocks()
    if dist:
        dist.barrier()
    e.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    rep = e.step(steps * a.segment)
    wall = time.perf_counter() - t0
    ms, launches = e.last_step_timing()
    ck = clocks.stop()
    ms = rank_max(ms, dist)
    st = e.stats()
    e.set_profiling(True)
    e.step(a.segment)
    prof = e.profile()
    e.set_profiling(False)
    if a.ncu_window == label:  # the launch list of one rebuild and one segment, for ncu
        e.synchronize()
        cu_profiler(True)
        e.update_nl()
        e.step(a.segment)
        e.synchronize()
        cu_profiler(False)
    rec = {"value": job_rate(ws, nfree, steps * a.segment, ms), "ms": ms, "ms_per_step": ms / steps,
           "ms_per_dem_step": ms / (steps * a.segment), "wall_s": wall, "gpu_launches": int(launches),
           "nl_rebuilds_in_timed": int(rep["nl_updates"]), "entries": int(st["n_entries"]),
           "active": int(st["n_active"]), "active_per_free": st["n_active"] / max(1, nfree), "clocks": ck,
           "skin": e.skin_stats() if SKIN[label] else None, "block_sizes": e.block_sizes(),
           "phases_ms_per_dem_step": {q: w[0] / a.segment for q, w in prof.items()},
           "phases_launches": {q: w[1] for q, w in prof.items()}, "profiled_steps": a.segment, "t_end": rep["t"]}
    return e, rec


def roofline(rec, scene, consts, fp64):
    """The dominant kernel of a form (narrow phase or resultants, by device
    time per DEM step): algorithmic bytes per launch (140 B per entry: 12 B key
    + the history read and written; 352 B per body: 200 B of state read and
    152 B written) over its event-timed launch duration, against the measured
    HBM copy bandwidth; DRAM traffic and FP64 operations per unit from the
    committed ncu summary."""
    ph = rec["phases_ms_per_dem_step"]
    la = rec["phases_launches"]
    hbm, src = peaks()
    nb = len(scene["bodies"]["mass"])
    dom = "narrow_force" if ph["narrow_force"] >= ph["gather_accel"] else "gather_accel"
    if dom == "narrow_force":
        unit_bytes, units, unit_name, key = 140.0, rec["entries"], "entries", "narrow"
    else:
        unit_bytes, units, unit_name, key = 352.0, nb, "bodies", "gather"
    # the phase's kernels per DEM step (one launch of k_narrow_force; the
    # resultant kernel plus, when a body has many entries, its block sums),
    # event-timed in the profiled segment
    per_step_ms = ph[dom]
    launches_per_step = la[dom] / max(1, rec["profiled_steps"])
    achieved = unit_bytes * units / (per_step_ms / 1e3) / 1e9 if per_step_ms > 0 else None
    per_launch_ms = per_step_ms / launches_per_step if launches_per_step else None
    out = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
           "frac": (achieved / hbm) if achieved else None, "peak_source": src,
           "algorithmic_bytes_per_unit": unit_bytes, "units": int(units), "unit_name": unit_name,
           "ms_per_dem_step": per_step_ms, "launches_per_dem_step": launches_per_step,
           "ms_per_launch": per_launch_ms, "phase_ms_per_dem_step": {k: ph[k] for k in ("narrow_force", "gather_accel")}}
    tb = consts.get(key + "_dram_bytes_per_unit")
    out["traffic"] = tb * units if tb is not None else None
    out["traffic_note"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum per %s of this kernel (%s) x this "
                           "form's %s" % (unit_name[:-1], os.path.relpath(PROFILE, ROOT), unit_name)
                           if tb is not None else "no ncu capture of this kernel on this workload")
    fl = consts.get(key + "_fp64_ops_per_unit")
    if fl is not None and per_step_ms > 0:
        ach = fl * units / (per_step_ms / 1e3) / 1e12
        out["fp64"] = {"achieved_tflops": ach, "peak_tflops": fp64, "frac": (ach / fp64) if fp64 else None,
                       "peak_source": "measured: cuBLAS DGEMM 4096^3 burst on this GPU",
                       "ops_per_unit": fl, "ops_source": "ncu dadd + dmul + 2 dfma thread instructions (%s)" %
                       os.path.relpath(PROFILE, ROOT)}
    return out


def e2e_leg(scene, label, a, dev, dist, ws, steps):
    """The headline form through the C ABI with host-owned state, from the
    same state and after the same tuning and warm-up steps as the timed leg
    (a context of its own): every bench step uploads the kinematics (pos,
    vel, acc, Q, vrot, arot: 152 B per body) from one pinned buffer, runs
    rk_step(segment) and downloads them back (rk_upload/download_kinematics_
    packed)."""
    N = len(scene["bodies"]["mass"])
    nfree = N - scene["n_driven"]
    g = engine(scene, label, dev, SKIN[label])
    g.autotune(2)
    g.step(TUNE_STEPS)
    if a.warmup:
        g.step(a.warmup * a.segment)
    hb = pinned((19 * N,))
    g.download_kinematics_packed(hb)
    g.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    rebuilds = 0
    for _ in range(steps):
        g.upload_kinematics_packed(hb)
        rebuilds += int(g.step(a.segment)["nl_updates"])
        g.download_kinematics_packed(hb)
    el = rank_max(time.perf_counter() - t0, dist)
    g.close()
    return {"value": job_rate(ws, nfree, steps * a.segment, 1000.0 * el), "unit": "particle-steps/s",
            "h2d_bytes_per_step": int(N * 19 * 8), "d2h_bytes_per_step": int(N * 19 * 8), "steps": steps,
            "nl_rebuilds": rebuilds,
            "note": "every bench step: the kinematics (pos, vel, acc, Q, vrot, arot) of every body H2D from one "
                    "pinned packed buffer, rk_step(%d), the same fields D2H back" % a.segment}


def rockfall_workload(a, dev):
    """The breakable bonded rockfall (scenes.rockfall_bonded: 40 blocks of
    500 grains, vertex bonds with Weibull strengths, 30 degree slope,
    10 m/s), loaded through the C++ host from its conf file: the host makes
    the bonds at load (stickVerticesInClusters, setVariableStickParams) and
    drives the engine context that is timed here.  Plain FP64 and mixed
    forms from the same conf; after the timed steps, the broken interfaces
    of the two forms are compared."""
    from rockable_gb300 import scenes
    from rockable_gb300.abi import HostScene, RK_FORM_MIXED
    t0 = time.perf_counter()
    sc = scenes.rockfall_bonded(nclusters=a.rock_clusters)
    t_gen = time.perf_counter() - t0
    conf = scenes.write_conf(sc, tempfile.mkdtemp(prefix="rk_rock_"))
    nfree = len(sc["bodies"]["mass"]) - sc["n_driven"]
    steps = max(2, a.steps // 4)
    forms, broken, t_open = {}, {}, {}
    for label in ["plain_fp64", "mixed"]:
        t0 = time.perf_counter()
        hs = HostScene(conf)
        t_open[label] = time.perf_counter() - t0
        g = hs.gpu
        if label == "mixed":
            g.set_form(RK_FORM_MIXED)
        g.update_nl()
        _, _, b0 = g.interfaces()
        g.set_graphs(True)
        g.autotune(2)
        g.step(TUNE_STEPS)
        g.synchronize()
        clocks = Clocks()
        clocks.start()
        rep = g.step(steps * a.segment)
        ms, launches = g.last_step_timing()
        ck = clocks.stop()
        st = g.stats()
        _, _, bf = g.interfaces()
        broken[label] = bf.copy()
        e = g.entries()
        forms[label] = {"value": nfree * steps * a.segment / (ms / 1e3), "ms": ms,
                        "ms_per_dem_step": ms / (steps * a.segment), "gpu_launches": int(launches),
                        "nl_rebuilds_in_timed": int(rep["nl_updates"]), "entries": int(st["n_entries"]),
                        "active": int(st["n_active"]), "interfaces": int(len(bf)),
                        "interfaces_broken_at_start": int(b0.sum()), "interfaces_broken": int(bf.sum()),
                        "bonds_intact": int(np.sum(e["bond"] >= 0)), "clocks": ck}
        hs.close()
    same = bool(np.array_equal(broken["plain_fp64"], broken["mixed"]))
    return {"workload": sc["name"], "bodies": len(sc["bodies"]["mass"]), "free_bodies": nfree, "law": sc["law"],
            "clusters": sc["pack"]["clusters"], "per_cluster": sc["pack"]["per_cluster"],
            "bond_eps": sc["bond_eps"], "slope_deg": 30.0, "v0": 10.0, "dem_steps_per_step": a.segment,
            "steps": steps, "tune_steps": TUNE_STEPS, "forms": forms,
            "mixed_vs_plain": forms["mixed"]["value"] / forms["plain_fp64"]["value"],
            "broken_sets_equal_at_end": same,
            "broken_set_difference": int(np.sum(broken["plain_fp64"] != broken["mixed"])),
            "setup_s": {"generate": t_gen, "host_open": t_open}}


def batched_workload(a, dev):
    """Many independent slope scenes (N ~ U{200..5000} grains each, slopes
    25-45 degrees, Default law) in ONE engine context: every launch covers all
    scenes, each step's launches replay as one CUDA graph.  For the plain
    FP64 form and the headline form (mixed + learned skin), the aggregate
    particle-steps/s and each scene's own step time when it runs alone in a
    context of its own (the spread, and the sum that batching replaces).
    The replayed graph's step time against the sum of its kernels' event
    times (launch by launch) measures what a persistent kernel could still
    remove: the gaps between launches."""
    from rockable_gb300 import scenes
    t0 = time.perf_counter()
    bt = scenes.slope_batch(nscenes=a.batch_scenes)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    g = scenes.settle(bt, steps=a.batch_settle, device=dev, rebuild_every=10, relax_steps=a.batch_settle // 3)
    src = scenes.scene_from_gpu(bt, g)
    g.close()
    t_settle = time.perf_counter() - t0
    nfree = int(sum(bt["free_per_scene"]))
    out = {"workload": bt["name"], "scenes": int(a.batch_scenes), "free_bodies": nfree,
           "bodies": int(len(bt["scene_of"])), "law": "Default", "steps": a.batch_steps, "unit": "particle-steps/s",
           "forms": {}, "setup_s": {"generate": t_gen, "settle": t_settle}}
    for label in ["plain_fp64", "mixed_learned_skin_exact"]:
        e = engine(src, label, dev, SKIN[label])
        e.autotune(2)
        e.step(TUNE_STEPS)
        e.step(max(3, a.warmup) * 10)
        clocks = Clocks()
        e.synchronize()
        clocks.start()
        rep = e.step(a.batch_steps)
        ms, launches = e.last_step_timing()
        ck = clocks.stop()
        st = e.stats()
        gst = e.graph_stats()
        bsz = e.block_sizes()
        e.set_profiling(True)
        e.step(a.batch_steps)
        prof = e.profile()
        sk = e.skin_stats() if SKIN[label] else None
        e.close()
        kernels_ms = sum(w[0] for q, w in prof.items()) / a.batch_steps
        solo = []
        for k in range(len(bt["free_per_scene"])):
            p = engine(scenes.part_of(src, k), label, dev, SKIN[label])
            p.step(3)
            p.step(a.batch_steps)
            pms, _ = p.last_step_timing()
            solo.append(pms / a.batch_steps)
            p.close()
        solo = np.array(solo)
        out["forms"][label] = {
            "value": nfree * a.batch_steps / (ms / 1000.0), "ms_per_step": ms / a.batch_steps,
            "gpu_launches": int(launches), "graph": gst, "block_sizes": bsz, "entries": int(st["n_entries"]),
            "active": int(st["n_active"]), "nl_rebuilds_in_timed": int(rep["nl_updates"]), "clocks": ck,
            "skin": sk,
            "solo_ms_per_step": {"min": float(solo.min()), "median": float(np.median(solo)),
                                 "p90": float(np.percentile(solo, 90)), "max": float(solo.max()),
                                 "sum": float(solo.sum())},
            "batched_vs_solo_sum": float(solo.sum() / (ms / a.batch_steps)),
            "phases_ms_per_step": {q: w[0] / a.batch_steps for q, w in prof.items()},
            "step_kernels_ms_per_step": kernels_ms}
    head = out["forms"]["mixed_learned_skin_exact"]
    out["value"] = head["value"]
    out["headline_vs_plain"] = head["value"] / out["forms"]["plain_fp64"]["value"]
    pl = out["forms"]["plain_fp64"]
    out["persistent_kernel_bound"] = (
        "plain FP64: graph replay %.4f ms per step; the same kernels event-timed one phase at a time (launch by "
        "launch, the same number of steps and rebuilds) %.4f ms per step: a persistent kernel could remove at "
        "most the launch gaps left in the replay, max(0, %.4f) ms per step" % (
            pl["ms_per_step"], pl["step_kernels_ms_per_step"], pl["ms_per_step"] - pl["step_kernels_ms_per_step"]))
    return out


def iso_workload(a, dev, dist, ws, order):
    """Config 4: the compression box, plain FP64 and the headline form, and
    a CPU sample of the same segment (reported against the >= 50x target)."""
    from rockable_gb300 import scenes
    t0 = time.perf_counter()
    packed = scenes.iso_compression(n=a.iso_n)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    sc = scenes.loaded(packed, a.iso_load_steps, device=dev)
    t_load = time.perf_counter() - t0
    nfree = len(sc["bodies"]["mass"]) - sc["n_driven"]
    steps = max(2, a.steps // 4)
    forms = {}
    for label in ["plain_fp64", order[-1]]:
        e, rec = time_form(sc, label, a, dev, dist, ws, steps, 1)
        e.close()
        forms[label] = rec
    head = forms[order[-1]]
    out = {"workload": sc["name"], "bodies": len(sc["bodies"]["mass"]), "free_bodies": nfree,
           "law": sc["law"], "servo": "tritriIsostaticCompression at %g Pa, no gravity" % sc["servo"]["pressure"],
           "pack": sc["pack"], "load": sc["load"],
           "state": ("the packed box after %d DEM steps of servo compression with numerical damping 0.5 "
                     "(scenes.loaded)" % a.iso_load_steps),
           "dem_steps_per_step": a.segment, "steps": steps, "warmup": 1,
           "forms": forms, "headline_form": order[-1],
           "headline_vs_plain": head["value"] / forms["plain_fp64"]["value"],
           "setup_s": {"generate": t_gen, "load": t_load}}
    if not a.no_cpu:
        cb = cpu_baseline(sc, a.segment, 2.0 * a.cpu_seconds, "the compressed box")
        out["cpu_baseline"] = cb
        out["vs_cpu"] = {k: v["value"] / cb["value"] for k, v in forms.items()}
        out["target_50x_at_200k"] = ("met" if min(out["vs_cpu"].values()) >= 50.0 else "not met")
    return out


def main():
    a = parse()
    if a.impl == "reference":
        # the reference's CPU path runs once, on rank 0; under torchrun the
        # other ranks exit without work (no process group: nothing to join)
        run_reference(a, int(os.environ.get("RANK", "0")))
        return
    rank, ws, dist = dist_setup()
    from rockable_gb300 import build_ext
    if rank == 0:
        build_ext.build()
    if dist:
        dist.barrier()
    from rockable_gb300 import scenes
    dev = int(os.environ.get("LOCAL_RANK", "0")) if ws > 1 else 0
    t0 = time.perf_counter()
    packed = scenes.column_collapse(n=a.n, walls=True)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    scene = scenes.loaded(packed, a.load_steps, device=dev, dt_factor=2.0)
    t_load = time.perf_counter() - t0
    N = len(scene["bodies"]["mass"])
    nfree = N - scene["n_driven"]
    order = [f.strip() for f in a.forms.split(",") if f.strip()]
    forms = {}
    for label in order:
        e, rec = time_form(scene, label, a, dev, dist, ws, a.steps, a.warmup)
        forms[label] = rec
        e.close()
    head = forms[order[-1]]
    consts = profile_constants()
    fp64 = fp64_peak() if rank == 0 else None
    roof = roofline(head, scene, consts, fp64)
    e2e = None if a.no_e2e else e2e_leg(scene, order[-1], a, dev, dist, ws, a.steps)
    iso = guarded(iso_workload, a, dev, dist, ws, order) if (a.iso_n > 0 and rank == 0) else None
    rockfall = guarded(rockfall_workload, a, dev) if (rank == 0 and a.rock_clusters > 0) else None
    batched = guarded(batched_workload, a, dev) if (rank == 0 and a.batch_scenes > 0) else None
    cpu = cpu_settled = None
    if rank == 0 and not a.no_cpu:
        # the reference arm's state (the packed column at t = 0, no walls),
        # and the settled state the GPU forms are timed on
        cpu = cpu_baseline(scenes.drop_bodies(packed, packed["walls"]), a.segment, a.cpu_seconds,
                           "the packed column at t = 0 (the reference arm's state)")
        cpu_settled = cpu_baseline(scene, a.segment, a.cpu_seconds, "the settled column at release (the GPU "
                                   "forms' state)")
    if rank == 0:
        out = {"metric": METRIC, "value": head["value"], "unit": "particle-steps/s", "n_gpus": ws, "steps": a.steps,
               "warmup": a.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64+f32 (mixed form; the plain form is f64)",
               "data": "synthetic (seeded generator and CPU packer, rockable_gb300.scenes)",
               "form": "mixed precision + learned skin with exact contact detection (headline); plain FP64 and "
                       "mixed alongside",
               "forms": forms, "headline_form": order[-1],
               "headline_vs_plain": (head["value"] / forms["plain_fp64"]["value"]) if "plain_fp64" in forms else None,
               "config": {"workload": scene["name"], "law": scene["law"], "bodies": N, "free_bodies": nfree,
                          "dem_steps_per_step": a.segment, "entries": head["entries"], "active": head["active"],
                          "active_per_free": head["active_per_free"],
                          "nl_rebuilds_in_timed": head["nl_rebuilds_in_timed"], "dt": scene["dt"],
                          "interVerlet_steps": int(round(scene["interVerlet"] / scene["dt"])),
                          "pack": scene["pack"], "load": scene["load"], "cpu_on_settled_state": cpu_settled,
                          "state": ("the packed column settled by gravity between four walls (%d DEM steps of "
                                    "2 x dt with numerical damping 0.5, scenes.loaded), walls removed, then %d tuning and %d "
                                    "warm-up DEM steps of each form before its timed ones" % (
                                        a.load_steps, TUNE_STEPS, a.warmup * a.segment)),
                          "l2": "inputs larger than L2 (entries + bodies > 129 MB)" if head["entries"] * 240 + N * 600 >
                          129e6 else "working set below L2 size (no flush between steps: consecutive DEM steps reuse it)",
                          "parallelism": "replicas" if ws > 1 else "single GPU",
                          "setup_s": {"generate": t_gen, "load": t_load}},
               "gpu_launches": head["gpu_launches"], "wall_s": head["wall_s"], "clocks": head["clocks"],
               "roofline": roof, "e2e": e2e, "cpu_baseline": cpu, "iso": iso, "rockfall": rockfall,
               "batched": batched}
        print(json.dumps(out), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
