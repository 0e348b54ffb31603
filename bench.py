"""Benchmark: particle-substeps/s of the MPM substep on one GB300.

Workload (default): the 1M-particle three-box scene on a sparse 4^3-block grid
over a 256^3 domain (fixed-corotated, snow and Drucker-Prager sand boxes,
dt = 5e-5), synthetic and seeded.  A "step" is one substep over all particles.

  value        particle-substeps/s with the state resident in HBM (CUDA events
               around K substeps on the library's stream; the K-substep
               region is repeated until the repeats cover --min-seconds and
               the median repeat is reported)
  e2e          the same metric through the C ABI with host buffers: per e2e step
               sv_create (host->device upload of the state), one frame of
               substeps (1/24 s of simulated time), sv_download (device->host)
  roofline     the dominant kernel's algorithmic bytes per launch / its average
               duration, against the measured HBM copy bandwidth; for the fused
               particle pass the duration is the kernels' own device-timer
               reading over every launch of the timed region (graph replays
               included), cross-checked by CUDA events around the kernel in K
               direct-launch substeps after it (event_check)
  cpu_baseline the CPU oracle (the reference substep restated in C++, fp32,
               all host threads) on a bounded sample of the same scene
  adaptive     (--adaptive) sv_step_adaptive over the simulated time of K
               substeps, the scene's dt as the largest step
  error_vs_fp64  --error-substeps substeps (default 3) from the initial state
               on the GPU and on the fp64 CPU oracle: relative errors of x, v,
               C and F
  secondary    the 8M-particle dam break (--secondary), measured the same way:
               its own value, roofline, e2e and error against fp64

--impl reference runs only the CPU restatement of the reference substep (the
reference itself is Rust and cannot be built here) on the same scene.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-substeps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scene", default="three_boxes_1m")
    ap.add_argument("--sort-interval", type=int, default=0,
                    help="substeps between binning sorts (0 adaptive, 1 every substep like the reference)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip sv_autotune (by default the binning interval x CTAs/SM candidates are timed first "
                         "and the fastest is kept; the handle's defaults win unless beaten by more than 2 %%)")
    ap.add_argument("--no-graphs", action="store_true", help="launch every kernel directly (no CUDA graphs)")
    ap.add_argument("--deterministic", action="store_true",
                    help="the deterministic P2G mode (fixed summation order, fp32 positions, no graphs)")
    ap.add_argument("--closure", default="plain", choices=["plain", "learned"],
                    help="snow/sand constitutive update: SVD + return map, or the learned closure (trained first)")
    ap.add_argument("--closure-source", default="batched_64,self",
                    help="comma-separated workloads whose plain runs give the closure's training pairs (their snow "
                         "and sand particles); 'self' is the measured scene's own first substeps")
    ap.add_argument("--closure-pairs", type=int, default=50_000_000, help="training pairs to harvest")
    ap.add_argument("--closure-iters", type=int, default=20000, help="Adam steps of 65536 pairs")
    ap.add_argument("--closure-augment", type=float, default=0.1,
                    help="half of the harvested pairs are widened by F (I + a R), R symmetric with entries in [-1, 1)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="bound on the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--adaptive", action="store_true",
                    help="also time sv_step_adaptive over the same span of simulated time (max step = the scene's dt)")
    ap.add_argument("--bake", type=int, default=0,
                    help="also time this many whole frames with a frame-cache store after each, against the same "
                         "frames without stores")
    ap.add_argument("--error-substeps", type=int, default=3,
                    help="also run this many substeps from the initial state on the GPU and on the fp64 CPU oracle "
                         "and report the relative errors of x, v, C, F (0: off)")
    ap.add_argument("--secondary", default="dam_break_8m,batched_64",
                    help="comma-separated further workloads measured the same way: the first is reported under "
                         "'secondary', the others under 'additional' ('' for none)")
    ap.add_argument("--closure-workload", default="snow_sand_2m",
                    help="also measure this workload with the learned closure against the return maps, reported "
                         "under 'closure_check' ('' for none; --closure learned measures the headline instead)")
    ap.add_argument("--min-seconds", type=float, default=0.5,
                    help="repeat the K-substep timed region until the repeats cover this long; the median is reported")
    ap.add_argument("--max-repeats", type=int, default=2000)
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(scene, seconds_budget: float):
    """Times the CPU oracle (fp32, all host threads) on the full scene for as
    many substeps as fit the time budget (at least one)."""
    import oracle

    threads = os.cpu_count() or 1
    o = oracle.OracleState(scene.io_state.particles, scene.consts, scene.extras, fp64=False, threads=threads)
    n = scene.io_state.particles.n
    done = 0
    t0 = time.perf_counter()
    while True:
        o.step(1, scene.dt, scene.gravity)
        done += 1
        if time.perf_counter() - t0 > seconds_budget or done >= scene.substeps:
            break
    dt = time.perf_counter() - t0
    o.close()
    return {
        "value": n * done / dt,
        "unit": METRIC,
        "cores": threads,
        "kind": "port",
        "sample": f"{done} substeps of the full {n}-particle scene (first substeps from the initial state), "
                  f"{dt:.1f} s, fp32 C++ restatement of the reference CPU substep",
    }


def error_vs_fp64(scene, substeps: int):
    """Relative L2 error of the GPU state against the fp64 oracle after
    `substeps` substeps from the same initial state (live particles)."""
    import oracle
    from squishy_volumes_gb300 import CudaState

    gpu = CudaState.from_io_state(scene.io_state, scene.consts, scene.extras)
    gpu.step(substeps, scene.dt, scene.gravity)
    out = gpu.download()
    gpu.close()
    ref = oracle.OracleState(scene.io_state.particles, scene.consts, scene.extras, fp64=True,
                             threads=os.cpu_count() or 1)
    ref.step(substeps, scene.dt, scene.gravity)
    exp = ref.download()
    ref.close()
    live = (exp.flags & 32) == 0
    res = {"substeps": substeps, "particles_compared": int(live.sum())}
    vnorm = np.linalg.norm(exp.velocities[live].astype(np.float64))
    for k in ("positions", "velocities", "velocity_gradients", "position_gradients"):
        a = getattr(out, k)[live].astype(np.float64)
        b = getattr(exp, k)[live].astype(np.float64)
        d = np.abs(a - b)
        # C vanishes in rigid motion; its natural scale is |v| / dx
        scale = max(np.linalg.norm(b), vnorm / scene.consts.grid_node_size) if k == "velocity_gradients" \
            else np.linalg.norm(b)
        res[k] = {"rel_l2": float(np.linalg.norm(a - b) / max(scale, 1e-300)), "max_abs": float(d.max()) if d.size else 0.0}
    res["flags_equal"] = bool(np.array_equal(out.flags, exp.flags))
    return res


def bake_frames(scene, make_gpu, frames: int):
    """Whole frames of the workload, the reference's compute-thread loop
    (compute_thread.rs:136-169): step to the frame's end, then hand the state
    (with the grid) to the frame cache, whose writer thread restores the
    particle order and writes the file while the next frame computes.  The
    same frames without stores give the compute-only rate."""
    import shutil
    import tempfile

    from squishy_volumes_gb300 import CudaState
    from squishy_volumes_gb300.frames import FrameCache

    fps = scene.consts.frames_per_second
    frame_substeps = int(math.ceil((1.0 / fps) / scene.dt))
    res = {"frames": frames, "substeps_per_frame": frame_substeps, "store_grid": True}
    for store in (False, True):
        st_ = make_gpu()
        if not isinstance(st_, CudaState):
            st_.close()
            return None
        st_.step(frame_substeps, scene.dt, scene.gravity)  # warm-up frame: graphs captured
        directory = tempfile.mkdtemp(prefix="sv_bake_")
        cache = None
        if store:
            # two warm-up stores give both in-flight slots their pinned buffers
            cache = FrameCache(directory, scene.io_state.particles)
            cache.store(st_, store_grid=True)
            cache.store(st_, store_grid=True)
            cache.flush()
        calls = []
        t0 = time.perf_counter()
        for _ in range(frames):
            st_.step(frame_substeps, scene.dt, scene.gravity)
            if cache is not None:
                c0 = time.perf_counter()
                cache.store(st_, store_grid=True)
                calls.append(time.perf_counter() - c0)
        t_compute = time.perf_counter()
        if cache is not None:
            cache.flush()
        t1 = time.perf_counter()
        if cache is None:
            res["frames_per_s_without_store"] = frames / (t1 - t0)
        else:
            written, nbytes = cache.info()
            cache.close()
            res["frames_per_s"] = frames / (t1 - t0)
            res["frames_per_s_until_last_store_queued"] = frames / (t_compute - t0)
            res["store_call_ms_median"] = float(np.median(calls) * 1e3)
            res["bytes_per_frame"] = nbytes // max(written, 1)
        st_.close()
        shutil.rmtree(directory, ignore_errors=True)
    return res


def algorithmic_bytes(kernel: str, live: int, grid_nodes: int, cell_form: bool):
    """Algorithmic HBM bytes per launch: per particle-substep the particle
    state is read (x 12, v 12, C 36, F 36, material/flags 4 = 100 B) and
    written (96 B), +12 B each way in the int32-cell form; per active grid
    node the scatter writes m + p (16 B) and the gather reads v (12 B)."""
    x = 12 + (12 if cell_form else 0)
    if kernel == "g2p2g":
        # one full particle-substep: read x, v, C, F, material/flags, write
        # x, v, C, F; grid: scatter writes m + p, gather reads v per node
        return live * ((x + 12 + 36 + 36 + 4) + (x + 12 + 36 + 36)) + grid_nodes * (16 + 12)
    if kernel == "p2g":
        # read x, v, C, F, material/flags; write grid m + p per active node
        return live * (x + 12 + 36 + 36 + 4) + grid_nodes * 16
    if kernel == "g2p":
        # read x, F, material/flags and grid v; write x, v, C, F
        return live * (x + 36 + 4) + grid_nodes * 12 + live * (x + 12 + 36 + 36)
    if kernel == "grid_update":
        return grid_nodes * (16 + 12)
    if kernel == "radix_sort":
        return live * 16  # key + index written and read once
    return None


def _barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def _max_over_ranks(x, world, dev):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measure_scene(args, name, rank, world, local, dev, primary):
    """One workload: the timed region, the per-kernel roofline, the e2e run
    through the C ABI with host buffers and the error against the fp64
    oracle.  Returns the fields of the bench line for it."""
    import torch

    from squishy_volumes_gb300 import CudaState, FrameInput, Harness, RunParameters, scenes

    made = scenes.SCENES[name]()
    if isinstance(made, list):
        # batched configuration: every scene in one handle; the CPU baseline
        # and the fp64 error report use the largest scene alone
        from squishy_volumes_gb300.state import BatchedCudaState

        batch = made
        scene = max(batch, key=lambda s: s.io_state.particles.n)
        n = sum(s.io_state.particles.n for s in batch)
        scene.extras.sort_interval = args.sort_interval
        make_gpu = lambda: BatchedCudaState.from_scenes([s.io_state for s in batch], [s.consts for s in batch],
                                                       scene.extras)
        h2d_particles = [s.io_state.particles for s in batch]
    else:
        batch = None
        scene = made
        n = scene.io_state.particles.n
        scene.extras.sort_interval = args.sort_interval
        if args.deterministic and primary:
            scene.extras.deterministic_p2g, scene.extras.position_form = 1, 0
        make_gpu = lambda: CudaState.from_io_state(scene.io_state, scene.consts, scene.extras)
        h2d_particles = [scene.io_state.particles]
    gpu = make_gpu()
    # All work, warm-up included, is queued on a torch stream handed to the
    # library (the CUDA graphs of the binning periods are captured on it).
    stream = torch.cuda.Stream(device=dev)
    gpu.set_stream(stream.cuda_stream)
    closure_info = None
    if primary and args.closure == "learned":
        closure_info = train_closure(gpu, scene, args)
    tuned = None
    if not args.no_autotune:
        st0 = gpu.stats()
        t0 = time.perf_counter()
        tuned = gpu.autotune(scene.dt, scene.gravity, 48)
        tuned["default"] = {"sort_interval": "adaptive, at most 8", "cta_per_sm": st0["cta_per_sm"]}
        tuned["seconds"] = round(time.perf_counter() - t0, 2)
    gpu.set_graphs(not args.no_graphs)
    status, done = gpu.step(args.warmup, scene.dt, scene.gravity)
    if status:
        raise RuntimeError(f"warm-up status {status:#x}")
    torch.cuda.synchronize()

    # Timed region: K substeps bracketed by CUDA events recorded on the
    # library's stream, with a barrier and a synchronize on both sides.  It
    # is repeated until the repeats cover at least --min-seconds (so that the
    # clock sampler sees the GPU under load), and the median repeat is
    # reported; the state keeps evolving from repeat to repeat.
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    reps = []
    stats0 = gpu.stats()
    with ClockSampler(local) as clocks:
        while True:
            _barrier(world)
            torch.cuda.synchronize()
            ev0.record(stream)
            status, done = gpu.step(args.steps, scene.dt, scene.gravity)
            ev1.record(stream)
            torch.cuda.synchronize()
            _barrier(world)
            if status or done != args.steps:
                raise RuntimeError(f"timed run status {status:#x}, done {done}")
            reps.append(_max_over_ranks(ev0.elapsed_time(ev1) * 1e-3, world, dev))
            if (sum(reps) >= args.min_seconds and len(reps) >= 3) or len(reps) >= args.max_repeats:
                break
    stats1 = gpu.stats()
    elapsed = float(np.median(reps))
    live = stats1["live_particles"]
    value = live * args.steps * world / elapsed
    launches = (stats1["kernel_launches"] - stats0["kernel_launches"]) / len(reps)
    if closure_info is not None:
        closure_info.update(compare_closure(gpu, scene, args, stream, value, live, world, stats0, stats1,
                                            args.steps * len(reps)))

    # The fused particle pass timed inside the timed region: the library's
    # kernels read the GPU's global nanosecond timer at the pass's first CTA
    # and at the end of its fp64 pass's last CTA, every launch, graph
    # replays included (sv_stats pass_ns / pass_count).
    pass_count = stats1["pass_count"] - stats0["pass_count"]
    pass_ns = stats1["pass_ns"] - stats0["pass_ns"]
    timed_pass_ms = pass_ns * 1e-6 / pass_count if pass_count else None
    timed_pass_share = pass_ns * 1e-9 / max(sum(reps), 1e-12) if pass_count else None

    # per-kernel durations of every kernel group: K more substeps right
    # after the timed region, with CUDA events around each group on the
    # library's stream (direct launches: events cannot sit inside a
    # replayed graph) -- the breakdown, and a cross-check of the pass above
    gpu.set_profiling(True)
    gpu.step(args.steps, scene.dt, scene.gravity)
    prof = json.loads(gpu.profile_report())
    gpu.set_profiling(False)
    st = gpu.stats()
    grid_nodes = st["grid_blocks"] * 64
    total_ms = sum(v["ms"] for v in prof.values())
    dom = max(prof.items(), key=lambda kv: kv[1]["ms"])[0]
    hbm, peak_kind = measured_peaks()
    cell_form = scene.extras.position_form == 1
    alg = algorithmic_bytes(dom, live, grid_nodes, cell_form)
    event_ms = prof[dom]["ms"] / prof[dom]["launches"]
    avg_ms = timed_pass_ms if (dom == "g2p2g" and timed_pass_ms) else event_ms
    achieved = alg / (avg_ms * 1e-3) / 1e9 if alg else None
    traffic = None
    tfile = ROOT / "profiles" / "traffic.json"
    if tfile.exists():
        try:
            traffic = json.loads(tfile.read_text()).get(name, {}).get(dom)
        except Exception:
            traffic = None
    roofline = {
        "kernel": dom,
        "bound": "hbm",
        "achieved": round(achieved, 1) if achieved else None,
        "peak": hbm,
        "peak_kind": peak_kind,
        "unit": "GB/s",
        "frac": round(achieved / hbm, 4) if achieved else None,
        "traffic": traffic,
        "bytes_per_launch": int(alg) if alg else None,
        "share": round(timed_pass_share, 4) if (dom == "g2p2g" and timed_pass_share) else round(prof[dom]["ms"] / total_ms, 4),
        "ms_per_launch": round(avg_ms, 5),
        "timer": ("device global timer over the timed region: the fused pass from its first CTA's start to its fp64 "
                  f"pass's end, {pass_count} launches (graph replays included)")
        if (dom == "g2p2g" and timed_pass_ms) else "CUDA events around each launch, K substeps after the timed region",
        "event_check": {"ms_per_launch": round(event_ms, 5), "share": round(prof[dom]["ms"] / total_ms, 4),
                        "how": "CUDA events around each kernel group, K direct-launch substeps after the timed region"},
        "kernels_ms_per_substep": {k: round(v["ms"] / args.steps, 5) for k, v in prof.items()},
    }
    # whole-substep roofline: 212 B per particle-substep of state and binning
    # (+24 B in the int32-cell form) plus 56 B per active grid node
    rho = grid_nodes / max(live, 1)
    bps = 212 + (24 if cell_form else 0) + 56 * rho
    sub_achieved = bps * live * args.steps / elapsed / 1e9 * world
    roofline["substep"] = {
        "bytes_per_particle_substep": round(bps, 1),
        "achieved": round(sub_achieved, 1),
        "frac": round(sub_achieved / hbm, 4),
    }

    # adaptive time steps (sv_step_adaptive) over the time K fixed substeps
    # span, from the state reached, the scene's dt as the largest step
    adaptive = None
    if primary and args.adaptive and batch is None:
        gpu.step_adaptive(gpu.time + args.warmup * scene.dt * (1 - 1e-6), scene.dt, scene.gravity)
        sa0 = gpu.stats()
        torch.cuda.synchronize()
        ev0.record(stream)
        status_a, done_a, _ = gpu.step_adaptive(gpu.time + args.steps * scene.dt * (1 - 1e-6), scene.dt, scene.gravity)
        ev1.record(stream)
        torch.cuda.synchronize()
        sa1 = gpu.stats()
        el_a = ev0.elapsed_time(ev1) * 1e-3
        adaptive = {
            "value": sa1["live_particles"] * done_a / el_a,
            "unit": METRIC,
            "substeps": done_a,
            "status": status_a,
            "ms_per_substep": el_a * 1e3 / max(done_a, 1),
            "speculation_misses": sa1["adaptive_misses"] - sa0["adaptive_misses"],
            "split_substeps": sa1["adaptive_split"] - sa0["adaptive_split"],
            "graph_replays": sa1["graph_replays"] - sa0["graph_replays"],
            "max_time_step": scene.dt,
        }
    gpu.close()

    # end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        fps = scene.consts.frames_per_second
        frame_substeps = int(math.ceil((1.0 / fps) / scene.dt))
        frame_substeps = min(frame_substeps, scene.substeps)
        reps_e2e = 3
        h2d = sum(q.nbytes() for q in h2d_particles)
        d2h = 0
        # one untimed step first: the process's first create / graph capture
        # / download pays one-off costs (module loading, the first mapping of
        # the output arrays' pages, which later steps' fresh arrays reuse
        # from the host allocator); every timed step still creates its
        # handle, uploads, captures its graphs, steps and downloads into
        # fresh arrays
        for rep in range(reps_e2e + 1):
            if rep == 1:
                t0 = time.perf_counter()
            st_ = make_gpu()
            params = RunParameters(target_time=frame_substeps * scene.dt * (1 - 1e-9), max_time_step=scene.dt)
            io, err = st_.produce_next_state(Harness(), FrameInput(scene.consts, scene.gravity), params)
            d2h = sum(getattr(io.particles, k).nbytes for k in
                      ("flags", "positions", "position_gradients", "velocities", "velocity_gradients",
                       "elastic_energies", "collider_bits", "plastic_j"))
            st_.close()
        t1 = time.perf_counter()
        e2e = {
            "value": n * frame_substeps * reps_e2e / (t1 - t0),
            "unit": METRIC,
            "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h),
            "substeps_per_step": frame_substeps,
            "step": "sv_create (upload) + one frame of substeps + sv_download, mean of 3 after 1 untimed",
        }

    bake = None
    if primary and args.bake > 0 and rank == 0:
        bake = bake_frames(scene, make_gpu, args.bake)

    error = None
    if args.error_substeps > 0 and rank == 0:
        error = error_vs_fp64(scene, args.error_substeps)

    config = {
        "workload": name,
        "particles": n,
        "scenes": len(batch) if batch else 1,
        "live_particles": live,
        "grid_blocks": st["grid_blocks"],
        "binning_sort_interval": st["sort_interval"],
        "binning_sorts_in_timed_region": int(stats1["sorts"] - stats0["sorts"]),
        "graph_replays_in_timed_region": int(stats1["graph_replays"] - stats0["graph_replays"]),
        "timed_repeats": len(reps),
        "timed_seconds_total": round(sum(reps), 4),
        "ms_per_step_min_median_max": [round(min(reps) / args.steps * 1e3, 5), round(elapsed / args.steps * 1e3, 5),
                                       round(max(reps) / args.steps * 1e3, 5)],
        "cta_per_sm": st["cta_per_sm"],
        "tile_miss_fraction": round((stats1["tile_misses"] - stats0["tile_misses"]) /
                                    max(1, live * args.steps * len(reps)), 5),
        "autotuned": tuned,
        "substep_dt": scene.dt,
        "position_form": "int32 cell + fp32 offset" if cell_form else "fp32",
        "l2": "state larger than L2 (no flush)",
        "parallelism": "replicas" if world > 1 else "single GPU",
    }
    return {
        "value": value,
        "ms_per_step": elapsed / args.steps * 1e3,
        "config": config,
        "roofline": roofline,
        "e2e": e2e,
        "adaptive": adaptive,
        "gpu_launches": int(round(launches)),
        "clocks": clocks.summary(),
        "fp64_svd_particles": st["fp64_svd"],
        "error_vs_fp64": error,
        "closure": closure_info,
        "bake": bake,
        "scene": scene,
    }


def train_closure(gpu, scene, args):
    """Training pairs harvested from plain runs of the --closure-source
    workloads (by default the 64-scene batched one -- its snow and sand
    scenes -- and the measured scene's own first 200 substeps) into the
    measured handle's pool, fp64 labels over the batched workload's material
    ranges, then the GPU training loop.  None of this is inside the timed
    region."""
    import torch

    from squishy_volumes_gb300 import CudaState, scenes
    from squishy_volumes_gb300.state import BatchedCudaState

    t0 = time.perf_counter()
    sources = [x for x in args.closure_source.split(",") if x]
    per_source = int(math.ceil(args.closure_pairs / max(1, len(sources))))
    pool, harvested = 0, {}
    for si, name in enumerate(sources):
        if name == "self":
            made, run = scene, gpu
        else:
            made = scenes.SCENES[name]()
            if isinstance(made, list):
                run = BatchedCudaState.from_scenes([s.io_state for s in made], [s.consts for s in made],
                                                   made[0].extras)
            else:
                run = CudaState.from_io_state(made.io_state, made.consts, made.extras)
        ref = made[0] if isinstance(made, list) else made
        rounds = 10
        # the batched scenes over their stated run; the measured scene over
        # its first 200 substeps (the timed region comes after them)
        per_round = max(1, (200 if name == "self" else ref.substeps) // rounds)
        before = pool
        for k in range(rounds):
            status, _ = run.step(per_round, ref.dt, ref.gravity)
            if status:
                raise RuntimeError(f"closure harvest run status {status:#x}")
            # half of the pairs widened by F (I + a R), R symmetric in
            # [-1, 1)^6: the batched scenes fall gently and barely yield, so
            # their own strains do not reach a collision's
            pool = gpu.closure_harvest_from(run, ref.dt, int(math.ceil(per_source / rounds)), args.closure_augment,
                                            seed=k + 100 * si)
        harvested[name] = pool - before
        if run is not gpu:
            run.close()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    # the batched workload's material ranges (nu in [0.2, 0.4], friction
    # angle in [25, 40] deg), a little wider so that their ends lie inside
    # the hull: the labels draw from them
    gpu.closure_set_material_ranges((0.18, 0.42), (23.0, 42.0))
    loss = gpu.closure_train(args.closure_iters, 65536, 3e-3, seed=1)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    yielding = gpu.closure_pool()["yielding_pairs"]
    gpu.closure_set_mode(1)
    return {"mode": "learned", "sources": harvested, "augment": args.closure_augment,
            "material_ranges": {"nu": [0.18, 0.42], "friction_deg": [23.0, 42.0]},
            "pairs": pool, "yielding_pairs": yielding,
            "harvest_s": round(t1 - t0, 3), "train_s": round(t2 - t1, 3), "train_iterations": args.closure_iters,
            "batch": 65536, "loss_normalised": loss}


def closure_accuracy(gpu, scene):
    """Errors of the learned closure against the fp64 return map, and the
    per-phase costs, on the state the timed run reached (the scene starts
    undeformed, where every stress is zero)."""
    ev = gpu.closure_evaluate(scene.dt)
    phases = gpu.closure_phase_times(scene.dt)
    return {"stress_rel_err_learned": ev["stress_err_learned"],
            "stress_rel_err_plain_fp32": ev["stress_err_plain32"],
            "projected_f_rel_err_learned": ev["f_err_learned"],
            "projected_f_rel_err_plain_fp32": ev["f_err_plain32"],
            "fallback_fraction": ev["fallbacks"] / max(ev["particles"], 1.0),
            "network_fraction": ev["network"] / max(ev["particles"], 1.0),
            "residual_rejects": ev["residual_rejects"],
            "stress_rel_err_network_part": ev["stress_err_network_part"],
            "stress_rel_err_elastic_part": ev["stress_err_elastic_part"],
            "phase_ms": {k: phases[k] for k in ("plain_ms", "closed_form_ms", "network_all_ms",
                                                "network_yielding_ms")},
            "phase_particles": phases["particles"], "phase_yielding": phases["yielding"]}


def compare_closure(gpu, scene, args, stream, value, live, world, stats0, stats1, substeps):
    """The same K substeps with the return maps, from the state reached."""
    import torch

    out = closure_accuracy(gpu, scene)
    out["learned_fraction"] = (stats1["closure_learned"] - stats0["closure_learned"]) / max(1, live * substeps)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    gpu.closure_set_mode(0)
    gpu.step(args.warmup, scene.dt, scene.gravity)
    torch.cuda.synchronize()
    ev0.record(stream)
    gpu.step(args.steps, scene.dt, scene.gravity)
    ev1.record(stream)
    torch.cuda.synchronize()
    out["plain_value"] = live * args.steps * world / (ev0.elapsed_time(ev1) * 1e-3)
    out["learned_over_plain"] = value / out["plain_value"]
    gpu.closure_set_mode(1)
    return out


def run_ours(args, rank, world, local):
    import torch

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    main = measure_scene(args, args.scene, rank, world, local, dev, primary=True)
    scene = main.pop("scene")
    # further workloads: each in its own handle, after the headline; a
    # failure is reported in its record and does not cost the headline line
    others = {}
    for name in [x for x in args.secondary.split(",") if x and x != args.scene]:
        try:
            sec = measure_scene(args, name, rank, world, local, dev, primary=False)
            sec.pop("scene")
            rec = {k: sec[k] for k in ("value", "ms_per_step", "config", "roofline", "e2e", "gpu_launches",
                                       "clocks", "fp64_svd_particles", "error_vs_fp64")}
            rec["unit"] = METRIC
        except Exception as exc:  # noqa: BLE001 -- recorded in the line
            rec = {"error": f"{type(exc).__name__}: {exc}"[:400]}
        others[name] = rec
        torch.cuda.synchronize()
    names = [x for x in args.secondary.split(",") if x and x != args.scene]
    secondary = others.get(names[0]) if names else None
    additional = {k: v for k, v in others.items() if not names or k != names[0]} or None
    closure_check = None
    if args.closure_workload and args.closure == "plain" and world == 1:
        import copy

        cargs = copy.copy(args)
        cargs.closure, cargs.no_autotune, cargs.no_e2e, cargs.error_substeps = "learned", True, True, 0
        try:
            rec = measure_scene(cargs, args.closure_workload, rank, world, local, dev, primary=True)
            closure_check = {"workload": args.closure_workload, "value_learned": rec["value"], "unit": METRIC,
                             **(rec["closure"] or {})}
        except Exception as exc:  # noqa: BLE001 -- recorded in the line
            closure_check = {"workload": args.closure_workload, "error": f"{type(exc).__name__}: {exc}"[:400]}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(scene, args.cpu_seconds)
    line = {
        "metric": METRIC,
        "value": main["value"],
        "unit": METRIC,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": main["ms_per_step"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded jittered boxes)",
        "config": main["config"],
        "roofline": main["roofline"],
        "cpu_baseline": cpu,
        "e2e": main["e2e"],
        "adaptive": main["adaptive"],
        "gpu_launches": main["gpu_launches"],
        "clocks": main["clocks"],
        "fp64_svd_particles": main["fp64_svd_particles"],
        "error_vs_fp64": main["error_vs_fp64"],
        "closure": main["closure"],
        "bake": main["bake"],
        "secondary": secondary,
        "additional": additional,
        "closure_check": closure_check,
    }
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def run_reference(args, rank, world):
    if rank != 0:
        return
    from squishy_volumes_gb300 import scenes

    scene = scenes.SCENES[args.scene]()
    n = scene.io_state.particles.n
    import oracle

    threads = os.cpu_count() or 1
    o = oracle.OracleState(scene.io_state.particles, scene.consts, scene.extras, fp64=False, threads=threads)
    # each step is one substep of the full scene: the requested warm-up and
    # timed steps, unless they would take longer than about 150 s, in which
    # case fewer timed steps are run (and reported)
    warm = max(1, args.warmup)
    t0 = time.perf_counter()
    o.step(warm, scene.dt, scene.gravity)
    per_step = (time.perf_counter() - t0) / warm
    steps = max(1, min(args.steps, int(150.0 / max(per_step, 1e-6))))
    t0 = time.perf_counter()
    o.step(steps, scene.dt, scene.gravity)
    el = time.perf_counter() - t0
    o.close()
    v = n * steps / el
    line = {
        "metric": METRIC,
        "value": v,
        "unit": METRIC,
        "impl": "reference",
        "n_gpus": world,
        "steps": steps,
        "warmup": warm,
        "ms_per_step": el / steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded jittered boxes)",
        "config": {"workload": args.scene, "particles": n, "substep_dt": scene.dt},
        "cpu_baseline": {
            "value": v,
            "unit": METRIC,
            "cores": threads,
            "kind": "port",
            "sample": f"{steps} substeps of the full scene after {warm} warm-up substeps; the reference is Rust "
                      "(no cargo/rustc here), so this is its CPU substep restated in C++ (oracle/)",
        },
        "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
