"""Benchmark: particle-steps/s of the DEM step on one GB300.

Workload (default): the granular column collapse -- 50,000 convex hull grains
(Avalanche law, linked-cell neighbour list) falling onto a rigid floor --
generated with a fixed seed by rockable_gb300.scenes.  One "step" is one pass
of the velocity-Verlet step loop (drift, narrow phase + force law, ordered
resultants, accelerations, half-kick, plus the NL rebuild every interVerlet).

Legs of one run:
  value      : device-timed throughput of K steps, state resident in HBM
               (CUDA events on the engine's stream);
  e2e        : the same metric through the C ABI with host-owned state: every
               step uploads the bodies' kinematics from pinned host memory and
               downloads the stepped state;
  roofline   : the narrow-phase kernel's algorithmic bytes (140 B per
               neighbour-list entry) over its event-timed duration, against
               the measured HBM copy bandwidth;
  cpu_baseline: the oracle (CPU restatement of the reference path, OpenMP) on
               a bounded sample of the same scene, on this host's cores.
`--impl reference` times the CPU path alone, on this workload.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s @1 GB300: plain FP64 vs mixed+learned-skin, <=1e-4 rel force err"
TUNE_STEPS = 10  # untimed block-size tuning steps before the warm-up (rk_set_autotune, 2 rounds of 5 sizes)
NCU_NARROW_MIXED_BYTES_PER_ENTRY = 22.877e6 / 183166  # ncu, 50k-grain column, mixed form (124.9 B)
NCU_GATHER_BYTES_PER_BODY = 11.54432e6 / 50001  # ncu --set full, 50k-grain column, exact learned skin (230.9 B)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scene", default="column", choices=["column", "cubes"])
    ap.add_argument("--n", type=int, default=50000)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--collapse-steps", type=int, default=50000,
                    help="untimed steps of the collapse before the timed forms (the middle of a 100k-step run)")
    ap.add_argument("--forms", default="plain_fp64,mixed,mixed_learned_skin,mixed_learned_skin_exact",
                    help="comma list of the forms to time (the last one is the headline)")
    ap.add_argument("--batch-scenes", type=int, default=256,
                    help="scenes of the batched slope workload (0: skip it)")
    ap.add_argument("--batch-steps", type=int, default=100)
    ap.add_argument("--batch-settle", type=int, default=3000)
    return ap.parse_args()


def make_scene(a):
    from rockable_gb300 import scenes
    if a.scene == "cubes":
        return scenes.sphero_cube_box()
    return scenes.column_collapse(n=a.n)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


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


def cpu_baseline(scene, budget_s):
    """Oracle (CPU restatement, OpenMP) on a bounded sample of the workload."""
    from oracle import oracle
    from rockable_gb300 import scenes
    oracle.build()
    d = tempfile.mkdtemp(prefix="rk_cpu_")
    conf = scenes.write_conf(scene, d)
    o = oracle.Oracle(conf)
    o.update_nl()
    nfree = o.n - o.n_driven
    o.run(1)  # warm-up: first-touch of the entry arrays
    # chunks of steps until the budget is spent (the first steps' time is no
    # guide to the rest: contacts and list updates come later)
    t0 = time.perf_counter()
    o.run(2)
    t1 = (time.perf_counter() - t0) / 2.0
    chunk = max(1, min(200, int(0.1 * budget_s / max(t1, 1e-6))))
    steps = 0
    t0 = time.perf_counter()
    while steps < 2000 and (steps == 0 or time.perf_counter() - t0 < budget_s):
        o.run(chunk)
        steps += chunk
    el = time.perf_counter() - t0
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": nfree * steps / el, "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "sample": "%d steps of the %d-body scene (after load and the initial NL update), %.1f s" % (
                steps, o.n, el)}


def _nvtx():
    try:
        import torch
        return torch.cuda.nvtx
    except Exception:
        return None


def batched_workload(a, dev):
    """Many independent slope scenes (N ~ U{200..5000} grains each, slopes
    25-45 degrees, Default law) in ONE engine context: every launch covers all
    scenes, each step's launches replay as one CUDA graph.  Reports the
    aggregate particle-steps/s, and each scene's own step time when it runs
    alone in a context of its own (the spread, and the sum that batching
    replaces)."""
    from rockable_gb300 import scenes
    from rockable_gb300.abi import GpuScene
    t0 = time.perf_counter()
    bt = scenes.slope_batch(nscenes=a.batch_scenes)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    g = scenes.settle(bt, steps=a.batch_settle, device=dev, rebuild_every=10, relax_steps=a.batch_settle // 3)
    src = scenes.scene_from_gpu(bt, g)
    g.close()
    t_settle = time.perf_counter() - t0
    nfree = int(sum(bt["free_per_scene"]))

    def engine(sc, entries=None):
        e = GpuScene(device=dev)
        e.upload_shapes(sc["shape_tables"])
        e.upload_bodies(sc["bodies"], sc["n_driven"])
        if sc.get("scene_of") is not None:
            e.set_scenes(sc["scene_of"])
        scenes.set_scene_params(e, sc)
        if entries is not None:
            e.upload_entries(entries)
        else:
            e.update_nl()
        e.set_graphs(True)
        return e

    e = engine(src, src["entries"])
    e.autotune(2)
    e.step(TUNE_STEPS)
    e.step(max(3, a.warmup))
    clocks = Clocks()
    e.synchronize()
    clocks.start()
    nvtx = _nvtx()
    if nvtx:
        nvtx.range_push("timed_batch")
    rep = e.step(a.batch_steps)
    if nvtx:
        nvtx.range_pop()
    ms, launches = e.last_step_timing()
    ck = clocks.stop()
    st = e.stats()
    gst = e.graph_stats()
    bsz = e.block_sizes()
    e.set_profiling(True)
    e.step(a.batch_steps)
    prof = e.profile()
    e.close()
    solo = []
    for k in range(len(bt["free_per_scene"])):
        part = scenes.part_of(src, k)
        p = engine(part)
        p.step(3)
        p.step(a.batch_steps)
        pms, _ = p.last_step_timing()
        solo.append(pms / a.batch_steps)
        p.close()
    solo = np.array(solo)
    return {"workload": bt["name"], "scenes": len(solo), "free_bodies": nfree, "bodies": int(len(bt["scene_of"])),
            "law": "Default", "form": "plain FP64, step graphs", "steps": a.batch_steps,
            "value": nfree * a.batch_steps / (ms / 1000.0), "unit": "particle-steps/s",
            "ms_per_step": ms / a.batch_steps, "gpu_launches": int(launches), "graph": gst,
            "block_sizes": bsz,
            "entries": int(st["n_entries"]), "active": int(st["n_active"]), "nl_rebuilds_in_timed": int(rep["nl_updates"]),
            "clocks": ck,
            "solo_ms_per_step": {"min": float(solo.min()), "median": float(np.median(solo)),
                                 "p90": float(np.percentile(solo, 90)), "max": float(solo.max()),
                                 "sum": float(solo.sum())},
            "batched_vs_solo_sum": float(solo.sum() / (ms / a.batch_steps)),
            "phases_ms_per_step": {q: w[0] / a.batch_steps for q, w in prof.items()},
            "setup_s": {"generate": t_gen, "settle": t_settle}}


def prepare_column(a, dev=0, report=None):
    """The column-collapse state every timed run starts from: the seeded
    loose deposit (t = 0, the column released onto the floor) advanced by
    --collapse-steps steps at the benchmark parameters (mixed form, not
    timed), i.e. a slice from the middle of the workload's 100k-step run."""
    from rockable_gb300 import scenes
    from rockable_gb300.abi import GpuScene, RK_FORM_MIXED
    scene = scenes.column_collapse(n=a.n)
    e = GpuScene(device=dev, form=RK_FORM_MIXED)
    e.upload_shapes(scene["shape_tables"])
    e.upload_bodies(scene["bodies"], scene["n_driven"])
    scenes.set_scene_params(e, scene)
    e.update_nl()
    e.set_graphs(True)
    done = 0
    while done < a.collapse_steps:
        k = min(10000, a.collapse_steps - done)
        e.step(k)
        done += k
        if report is not None:
            st = e.stats()
            report.append((done, st["n_entries"], st["n_active"], st["e_trans"]))
    src = scenes.scene_from_gpu(scene, e)
    e.close()
    return src


def reference_input(a):
    """The benchmark's input state for the CPU arm: the same seeded scene,
    settled the same way when a GPU is present (input preparation only,
    outside the timed region), else the freshly deposited pile."""
    from rockable_gb300 import scenes
    scene = make_scene(a)
    if a.scene != "column":
        return scene, "lattice as generated"
    try:
        import torch
        have_gpu = torch.cuda.is_available()
    except Exception:
        have_gpu = False
    if not have_gpu:
        return scene, "deposited pile (no GPU to settle it)"
    return prepare_column(a), ("the benchmark state: the seeded loose column after %d collapse steps, "
                               "prepared on the GPU, not timed" % a.collapse_steps)


def run_reference(a, rank):
    """The reference's CPU path (the oracle: restatement of the reference
    step loop, OpenMP over all host threads) on the same workload: W warm-up
    steps, then exactly K timed steps."""
    if rank != 0:
        return
    from oracle import oracle
    from rockable_gb300 import scenes
    src, how = reference_input(a)
    oracle.build()
    d = tempfile.mkdtemp(prefix="rk_ref_")
    o = oracle.Oracle(scenes.write_conf(src, d))
    o.update_nl()
    nfree = o.n - o.n_driven
    o.run(max(0, a.warmup))
    t0 = time.perf_counter()
    o.run(a.steps)
    el = time.perf_counter() - t0
    value = nfree * a.steps / el
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    sample = "%d timed steps after %d warm-up steps of the %d-body scene (%s), %.1f s" % (
        a.steps, a.warmup, o.n, how, el)
    out = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": a.gpus, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": 1000.0 * el / max(1, a.steps), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
           "impl": "reference",
           "config": {"workload": src["name"], "law": src["law"], "bodies": int(o.n), "free_bodies": int(nfree)},
           "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


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
    from rockable_gb300.abi import GpuScene, RK_LAW
    dev = int(os.environ.get("LOCAL_RANK", "0")) if ws > 1 else 0
    settle_log = []
    t_settle = time.perf_counter()
    if a.scene == "column":
        src = prepare_column(a, dev, settle_log)  # the state S every form starts from
        scene = src
    else:
        scene = make_scene(a)
        src = None
    t_settle = time.perf_counter() - t_settle
    b = scene["bodies"]
    N = len(b["mass"])
    nfree = N - scene["n_driven"]
    from rockable_gb300.abi import RK_FORM_FP64, RK_FORM_MIXED

    def engine(form):
        e = GpuScene(device=dev, form=form)
        e.upload_shapes(scene["shape_tables"])
        e.upload_bodies(src["bodies"] if src else b, scene["n_driven"])
        scenes.set_scene_params(e, scene)
        if src:
            e.upload_entries(src["entries"])
        e.set_graphs(True)
        return e

    def timed(e, steps, label):
        clocks = Clocks()
        if dist:
            dist.barrier()
        e.synchronize()
        clocks.start()
        nvtx = None
        try:
            import torch
            nvtx = torch.cuda.nvtx
            nvtx.range_push("timed_" + label)
        except Exception:
            nvtx = None
        t0 = time.perf_counter()
        rep = e.step(steps)
        wall = time.perf_counter() - t0
        if nvtx:
            nvtx.range_pop()
        ms, launches = e.last_step_timing()
        ck = clocks.stop()
        ms = rank_max(ms, dist)
        return {"ms": ms, "launches": launches, "wall": wall, "rep": rep, "clocks": ck,
                "value": job_rate(ws, nfree, steps, ms)}

    def profile(e, n):
        e.set_profiling(True)
        e.step(n)
        p = e.profile()
        e.set_profiling(False)
        return p

    forms = {}
    dmin = scene["dVerlet"]
    # skin: None (fixed interVerlet), "ref" (learned skin, Rockable's NEAR tests), "exact" (distance-only)
    known = {"plain_fp64": (RK_FORM_FP64, None), "mixed": (RK_FORM_MIXED, None),
             "mixed_learned_skin": (RK_FORM_MIXED, "ref"), "mixed_learned_skin_exact": (RK_FORM_MIXED, "exact")}
    order = [f.strip() for f in a.forms.split(",") if f.strip()]
    for label in order:
        form, skin = known[label]
        e = engine(form)
        if skin:
            e.set_skin(use_mlp=True, skin_min=0.1 * dmin, skin_max=4.0 * dmin, dverlet_ratio=2.0, interval_min=2,
                       interval_max=1000, seed=3, exact_contacts=(skin == "exact"))
        else:
            e.update_nl()
        e.autotune(2)
        e.step(TUNE_STEPS)
        e.step(a.warmup)
        r = timed(e, a.steps, label)
        st = e.stats()
        nprof = max(1, min(a.steps, 120))
        prof = profile(e, nprof)
        r.update({"entries": st["n_entries"], "active": st["n_active"], "prof": prof, "nprof": nprof,
                  "skin": e.skin_stats() if skin else None, "block_sizes": e.block_sizes()})
        forms[label] = r
        if label != order[-1]:
            e.close()
        else:
            g = e
    head = forms[order[-1]]
    ms, launches, wall, rep, ck, value = (head["ms"], head["launches"], head["wall"], head["rep"], head["clocks"],
                                          head["value"])
    prof, nprof = head["prof"], head["nprof"]
    # roofline of the headline form's dominant kernel: the narrow phase (140
    # algorithmic bytes per entry: 12 B key + history read and written) or the
    # resultant / integration kernel (352 B per body: 200 B of state read, 152 B
    # written), whichever takes more device time per step
    C = head["entries"]
    hbm, src_peak = peaks()
    per_step = {k: prof[k][0] / max(nprof, 1) for k in ("narrow_force", "gather_accel")}
    dominant = max(per_step, key=per_step.get)
    if dominant == "narrow_force":
        unit_bytes, units, unit_name = 140.0, C, "entries"
        t_launch = prof["narrow_force"][0] / max(prof["narrow_force"][1], 1)  # ms per launch
        traffic = NCU_NARROW_MIXED_BYTES_PER_ENTRY * C
        tnote = "ncu DRAM bytes per entry of k_narrow_force_mixed (column, mixed form) x this form's entries"
    else:
        unit_bytes, units, unit_name = 352.0, N, "bodies"
        t_launch = per_step["gather_accel"]  # ms per step (k_gather_accel, plus k_gather_heavy when used)
        traffic = NCU_GATHER_BYTES_PER_BODY * N if NCU_GATHER_BYTES_PER_BODY else None
        tnote = ("ncu DRAM bytes per body of k_gather_accel (column, learned-skin form) x bodies"
                 if NCU_GATHER_BYTES_PER_BODY else "not captured for this kernel")
    achieved = unit_bytes * units / (t_launch / 1000.0) / 1e9 if t_launch > 0 else None
    st = {"n_entries": C, "n_active": head["active"]}
    # ---- e2e through the C ABI with host-owned state (headline form)
    e2e = None
    if not a.no_e2e:
        hb = pinned((19 * N,))  # packed pos | vel | acc | Q | vrot | arot
        g.download_kinematics_packed(hb)
        k_e2e = max(5, min(a.steps, 50))
        g.synchronize()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(k_e2e):
            g.upload_kinematics_packed(hb)
            g.step(1)
            g.download_kinematics_packed(hb)
        el = rank_max(time.perf_counter() - t0, dist)
        e2e = {"value": job_rate(ws, nfree, k_e2e, 1000.0 * el), "unit": "particle-steps/s",
               "h2d_bytes_per_step": int(N * 19 * 8), "d2h_bytes_per_step": int(N * 19 * 8),
               "steps": k_e2e, "note": "every step: the kinematics (pos, vel, acc, Q, vrot, arot) of every body "
                                       "H2D from one pinned packed buffer, rk_step(1), the same fields D2H back "
                                       "(rk_upload/download_kinematics_packed)"}
    batched = None
    if rank == 0 and a.batch_scenes > 0:
        batched = batched_workload(a, dev)
    cpu = None
    if rank == 0 and not a.no_cpu:
        cpu = cpu_baseline(src if src else scene, a.cpu_seconds)
    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": ws, "steps": a.steps,
               "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64+f32 (mixed form; plain form is f64)",
               "data": "synthetic (seeded generator, rockable_gb300.scenes)",
               "form": ("mixed precision + learned skin with exact contact detection (headline); plain FP64, "
                        "mixed, and the learned skin with Rockable's NEAR tests alongside"),
               "forms": {k: {"value": v["value"], "ms_per_step": v["ms"] / a.steps, "entries": v["entries"],
                             "active": v["active"], "nl_rebuilds_in_timed": v["rep"]["nl_updates"],
                             "gpu_launches": v["launches"], "skin": v["skin"], "block_sizes": v["block_sizes"],
                             "phases_ms_per_step": {q: w[0] / v["nprof"] for q, w in v["prof"].items()}}
                         for k, v in forms.items()},
               "headline_form": order[-1],
               "headline_vs_plain": (head["value"] / forms["plain_fp64"]["value"]) if "plain_fp64" in forms else None,
               "config": {"workload": scene["name"], "law": scene["law"], "bodies": N, "free_bodies": nfree,
                          "entries": int(C), "active": int(st["n_active"]),
                          "nl_rebuilds_in_timed": int(rep["nl_updates"]), "dt": scene["dt"],
                          "interVerlet_steps": int(round(scene["interVerlet"] / scene["dt"])),
                          "l2": "inputs larger than L2 (entries + bodies > 129 MB)" if C * 240 + N * 600 > 129e6 else
                          "working set below L2 size (no flush between steps: consecutive DEM steps reuse it)",
                          "parallelism": "replicas" if ws > 1 else "single GPU",
                          "setup_before_warmup": "%d untimed block-size tuning steps; step graphs on" % TUNE_STEPS,
                          "state": ("loose column (ballistic deposit) released onto the floor, %d collapse steps "
                                    "before the tuning and warm-up" % a.collapse_steps)
                          if a.scene == "column" else "lattice as generated"},
               "gpu_launches": int(launches), "wall_s": wall, "clocks": ck,
               "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": hbm,
                            "unit": "GB/s", "frac": (achieved / hbm) if achieved else None, "traffic": traffic,
                            "traffic_note": tnote,
                            "limiter": "FP64 pipe (ncu: 73% busy in the narrow phase and the resultants, "
                                       "81% in the global vertices)",
                            "peak_source": src_peak, "algorithmic_bytes_per_unit": unit_bytes,
                            "units": int(units), "unit_name": unit_name, "ms_per_launch": t_launch,
                            "phase_ms_per_step": per_step},
               "setup": {"settle_s": t_settle, "settle_log": settle_log},
               "phases_ms_per_step": {k: v[0] / nprof for k, v in prof.items()},
               "phases_launches": {k: v[1] for k, v in prof.items()},
               "e2e": e2e, "cpu_baseline": cpu, "batched": batched}
        print(json.dumps(out), flush=True)
    g.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
