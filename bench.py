"""Benchmark of the path-tracer hot path on the mid-size mixed-material scene.

Workload (one GPU): 64 icospheres of 327,680 triangles (20,971,520 + ground +
4 light triangles), 1920x1080, max depth 12, Russian roulette after depth 3,
1024x512 lognormal environment map + 4 triangle lights, thin lens 0.05.  A
step renders one 1-sample frame of the film (2,073,600 paths) through the
wavefront: raygen -> (closest hit -> shade -> occlusion) x 12 -> accumulate.
Synthetic seeded data; the BVH (~2.7 GB) is far larger than L2 (129 MB), so
no L2 flush is needed between steps.

Metric: Mrays/s = (camera + continuation + occlusion rays traced) / time.
`value` is device time of K steps (CUDA events on the library's stream);
`e2e` is wall time of the same steps through the C ABI with the film read
back to pinned host memory every step.  `roofline` is the closest-hit
traversal kernel: algorithmic bytes = BVH nodes x 64 B + triangles x 48 B per
ray (counted by a separate instrumented frame), over its event-timed
duration, against the measured HBM copy bandwidth.

--impl reference: the reference's own implementation of the path — its GLSL
shaders compiled as host C++ (oracle/_ref) — on all host cores over a
bounded seeded pixel sample of the same workload, without Russian roulette
(the reference has none); the process builds the workload with the oracle's
host helpers and never loads the library.  Where the reference's shaders are
not built, the oracle's restatement (bit-identical to them) stands in.

Parity: the N=1 line also carries `parity`, the per-path comparison of the
GPU against the oracle on a seeded 16,384-pixel subset of the workload over 4
frames (outside the timed region), with Russian roulette as benchmarked and
without it.
Under torchrun (N > 1) every rank renders its own frames of the shot
(replicas, weak scaling); rank 0 reports the max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s"
CONFIG = {"workload": "mixed-material scene, 64 x level-7 icospheres (20.97M tris), 1920x1080, depth 12, RR>3, "
                      "1024x512 env + 4 triangle lights, aperture 0.05",
          "triangles": 20971526, "width": 1920, "height": 1080, "max_depth": 12, "rr_depth": 3,
          "l2": "inputs larger than L2 (BVH ~2.7 GB), no flush"}


def dist_env():
    r = int(os.environ.get("RANK", "0"))
    w = int(os.environ.get("WORLD_SIZE", "1"))
    lr = int(os.environ.get("LOCAL_RANK", "0"))
    return r, w, lr


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for k, n in enumerate(names):
                    if r[5 + k].lower() in ("active", "1", "yes"):
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def build_workload(args, verbose):
    from asuna_gb300 import scenes

    b, shot = scenes.mixed_scene(args.width, args.height, frames=1, max_depth=12, n_spheres=args.spheres,
                                 level=args.level, seed=1234, rr_depth=3, verbose=verbose)
    return b, shot


def _one_frame(shot, frame0=0, rr=True):
    import copy

    from asuna_gb300 import _abi as A

    s = copy.copy(shot)
    s.frames, s.frame0 = 1, frame0
    if not rr:
        s.flags &= ~A.SHOT_RR
    return s


class CpuSampler:
    """Throughput of a CPU implementation of the path over seeded pixel
    samples of the workload: the reference's own shaders compiled as host C++
    (kind "reference"; without Russian roulette, which the reference does not
    have) or the oracle's restatement (kind "port", as benchmarked).  The
    scene set-up (the oracle's BVH build) is excluded from the timings."""

    def __init__(self, b, shot, kind, threads):
        from oracle import oracle_py

        self.kind, self.threads = kind, threads
        self.shot = _one_frame(shot, rr=(kind == "port"))
        self.desc = b.desc()
        t0 = time.time()
        if kind == "reference":
            self.impl = oracle_py.RefSampler(self.desc, self.shot)
        else:
            self.impl = oracle_py.OracleScene(self.desc)
        self.setup_s = time.time() - t0
        self.npix = shot.width * shot.height

    def run(self, px, frame0=0):
        s = _one_frame(self.shot, frame0, rr=(self.kind == "port"))
        if self.kind == "reference":
            return self.impl.run(s, px, self.threads)
        _, _, st = self.impl.render(s, records=False, film=None, pixels=px, threads=self.threads)
        return st

    def calibrate(self, seconds):
        """A seeded pixel sample that takes about `seconds` of CPU time."""
        rng = np.random.default_rng(0)
        n = 2048
        while True:
            px = np.sort(rng.choice(self.npix, size=min(n, self.npix), replace=False)).astype(np.uint32)
            st = self.run(px)
            if st["seconds"] >= seconds * 0.5 or n >= self.npix:
                return px, st
            n = int(min(self.npix, n * max(2.0, seconds / max(st["seconds"], 1e-3))))

    def describe(self, px, st):
        rays = st["extend_rays"] + st["shadow_rays"]
        what = ("the reference's shaders compiled as host C++, no Russian roulette (the reference has none)"
                if self.kind == "reference" else "the oracle's restatement, Russian roulette after depth 3")
        return {"value": rays / st["seconds"] / 1e6, "unit": METRIC, "cores": st["threads"], "kind": self.kind,
                "sample": f"{len(px)} seeded pixels x 1 frame (1 spp) of the benchmark workload, {what} "
                          f"({st['paths']} paths, {rays} rays, {st['seconds']:.1f} s; scene set-up and the "
                          f"oracle's BVH build, {self.setup_s:.1f} s, excluded)",
                "msamples_per_s": st["paths"] / st["seconds"] / 1e6}

    def close(self):
        self.impl.close()


def cpu_kind():
    from oracle import oracle_py

    return "reference" if oracle_py.ref() is not None else "port"


def cpu_leg(b, shot, seconds, threads, kind=None):
    """CPU throughput on a bounded seeded pixel sample of the same workload."""
    cs = CpuSampler(b, shot, kind or cpu_kind(), threads)
    try:
        px, st = cs.calibrate(seconds)
        return cs.describe(px, st)
    finally:
        cs.close()


def mapped_libraries():
    """The repository's shared libraries mapped into this process."""
    try:
        with open("/proc/self/maps") as f:
            paths = {ln.split()[-1] for ln in f if ln.rstrip().endswith(".so")}
    except OSError:
        return []
    return sorted(os.path.relpath(p, ROOT) for p in paths if p.startswith(ROOT))


def parity_check(ctx, scene, b, shot, npixels=16384, frames=4, seed=0):
    """Per-path GPU vs oracle agreement on a seeded pixel subset of the
    workload (oracle/parity.py's bar), with Russian roulette as benchmarked
    and without it (the reference's own estimator)."""
    import copy

    from asuna_gb300 import _abi as A
    from oracle import oracle_py, parity

    desc = b.desc()
    osc = oracle_py.OracleScene(desc)
    res = parity.sample_parity(ctx, scene, desc, shot, npixels, frames, seed, oracle_scene=osc)
    off = copy.copy(shot)
    off.flags &= ~A.SHOT_RR
    res["rr_off"] = parity.sample_parity(ctx, scene, desc, off, npixels, frames, seed, oracle_scene=osc)
    osc.close()
    res.update({"rr_depth": int(shot.rr_depth),
                "bar": f"per path every radiance channel within {parity.REL:g} relative + {parity.ABS:g}"})
    return res


def run_reference(args):
    """The reference's own CPU implementation of the path, timed step by
    step on a bounded pixel sample (rank 0 only; other ranks exit)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from asuna_gb300 import scene as sc
    from oracle import oracle_py

    with sc.host_helpers(oracle_py.OracleHelpers()):
        b, shot = build_workload(args, verbose=False)
    threads = os.cpu_count() or 1
    kind = cpu_kind()
    cs = CpuSampler(b, shot, kind, threads)
    per_step = max(1.0, min(args.ref_seconds, args.ref_budget / max(1, args.steps + args.warmup)))
    px, _ = cs.calibrate(per_step)
    for i in range(args.warmup):
        cs.run(px, frame0=1 + i)
    vals, secs, rays = [], 0.0, 0
    st = None
    for i in range(args.steps):
        st = cs.run(px, frame0=1 + args.warmup + i)
        vals.append((st["extend_rays"] + st["shadow_rays"]) / st["seconds"] / 1e6)
        secs += st["seconds"]
        rays += st["extend_rays"] + st["shadow_rays"]
    cs.close()
    v = rays / secs / 1e6
    cb = cs.describe(px, st)
    cb.update({"value": v, "steps_mrays": [round(x, 3) for x in vals]})
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural scene)", "config": workload_config(shot),
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if kind == "reference":
        # the oracle's restatement on the same sample, as a second figure
        line["cpu_port"] = cpu_leg(b, shot, per_step, threads, kind="port")
    libs = mapped_libraries()
    line["libraries"] = libs
    if any("libasuna_rt" in p for p in libs):
        raise RuntimeError(f"the reference arm loaded the library: {libs}")
    print(json.dumps(line), flush=True)
    return 0


def workload_config(shot):
    """The `config` both arms print (identical by construction)."""
    return {**CONFIG, "width": shot.width, "height": shot.height}


def run(args):
    rank, world, local = dist_env()
    import asuna_gb300 as ag
    from asuna_gb300 import _abi as A

    torch_dist = None
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        torch_dist = dist
    b, shot = build_workload(args, verbose=(rank == 0 and args.verbose))
    ctx = ag.Context(local)
    t0 = time.time()
    scene = ctx.create_scene(b.desc())
    sstats = scene.stats()
    if rank == 0 and args.verbose:
        print(f"scene built in {time.time() - t0:.1f} s: {sstats}", file=sys.stderr, flush=True)
    film = ctx.create_film(shot.width, shot.height)
    tuned = None
    if args.frames_per_step <= 0:
        # autotune the wavefront size (frames per call) and the persistent grids
        from asuna_gb300 import autotune

        tuned = autotune.tune(ctx, scene, shot, film)
        args.frames_per_step = tuned["frames"]
        if rank == 0 and args.verbose:
            print(f"autotune: {tuned}", file=sys.stderr, flush=True)
    else:
        ctx.set_path_budget(args.frames_per_step * shot.width * shot.height * BYTES_PER_PATH)
        if args.traversal:
            trav = [int(x) for x in args.traversal.split(",")]
            ctx.set_traversal(*trav)
            if args.shadow_occupancy:
                ctx.set_traversal_occupancy(trav[4] if len(trav) > 4 else 0, args.shadow_occupancy)
        if args.shape:
            ctx.set_traversal_shape(*(int(x) for x in args.shape.split(",")))
        ctx.set_ray_sort(args.ray_sort)
    # per-rank frames: replicas render disjoint frames of the same shot
    from asuna_gb300 import replicas

    per_rank = (args.warmup + 2 * args.steps + 2) * args.frames_per_step
    frame_base = replicas.frame_shard(rank, world, 1, world * per_rank)[0]

    def step(i, stats=True):
        shot.frame0 = frame_base + i * args.frames_per_step
        shot.frames = args.frames_per_step
        return ctx.render(scene, shot, film, stats=stats)

    # instrumented frame: traversal counters for the algorithmic bytes per ray
    ctx.set_counters(True)
    cst = step(0)
    ctx.set_counters(False)
    bytes_per_ext = (cst["nodes_visited"] * NODE_BYTES + cst["tris_tested"] * 48) / max(cst["extend_rays"], 1)
    bytes_per_sh = (cst["shadow_nodes_visited"] * NODE_BYTES + cst["shadow_tris_tested"] * 48) / max(cst["shadow_rays"], 1)
    for i in range(args.warmup):
        step(1 + i)
    if torch_dist:
        torch_dist.barrier()
    ctx.sync()
    tot = {k: 0.0 for k in ("extend_rays", "shadow_rays", "paths", "ms_total", "ms_extend", "ms_connect",
                            "ms_shade", "ms_sort", "extend_launches", "connect_launches", "kernel_launches")}
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            st = step(1 + args.warmup + i)
            for k in tot:
                tot[k] += st[k]
    ctx.sync()
    ms = tot["ms_total"]
    rays = tot["extend_rays"] + tot["shadow_rays"]
    # e2e: the same steps through the C ABI with a host read-back of the film each step
    host = np.empty((shot.height, shot.width, 4), np.float32)
    try:
        import torch

        pinned = torch.empty(host.nbytes, dtype=torch.uint8).pin_memory()
        host = np.frombuffer(pinned.numpy(), dtype=np.float32).reshape(shot.height, shot.width, 4)
    except Exception:
        pass
    e2e_rays = 0
    ctx.sync()
    te = time.perf_counter()
    for i in range(args.steps):
        st = step(1 + args.warmup + args.steps + i, stats=True)
        film.read(0, out=host)
        e2e_rays += st["extend_rays"] + st["shadow_rays"]
    e2e_s = time.perf_counter() - te
    if torch_dist:
        import torch

        t = torch.tensor([ms, e2e_s], dtype=torch.float64, device=f"cuda:{local}")
        torch_dist.all_reduce(t, op=torch_dist.ReduceOp.MAX)
        r = torch.tensor([rays, e2e_rays], dtype=torch.float64, device=f"cuda:{local}")
        torch_dist.all_reduce(r, op=torch_dist.ReduceOp.SUM)
        ms, e2e_s = float(t[0]), float(t[1])
        rays, e2e_rays = float(r[0]), float(r[1])
    if rank != 0:
        if torch_dist:
            torch_dist.destroy_process_group()
        return 0
    peak, peak_kind = peaks()
    ext_ms_per_launch = tot["ms_extend"] / max(tot["extend_launches"], 1)
    ext_bytes_per_launch = bytes_per_ext * tot["extend_rays"] / max(tot["extend_launches"], 1)
    achieved = ext_bytes_per_launch / (ext_ms_per_launch * 1e-3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "extend_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            tj = json.load(f)
        traffic = tj.get("dram_bytes_per_ray", 0) * tot["extend_rays"] / max(tot["extend_launches"], 1)
    # counted by the engine: per wavefront raygen + accumulate; per depth
    # extend, classify, one kernel per shading class the scene uses, connect
    launches = int(tot["kernel_launches"])
    line = {
        "metric": METRIC, "value": rays / (ms * 1e-3) / 1e6, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": workload_config(shot),
        "run": {"parallelism": f"replicas{world}", "frames_per_step": args.frames_per_step,
                "autotune": None if tuned is None else {k: tuned[k] for k in tuned if k != "trials"}},
        "msamples_per_s": tot["paths"] * world / (ms * 1e-3) / 1e6 if world == 1 else None,
        "rays_per_step": rays / args.steps,
        "instrumented_step": {"extend_rays": cst["extend_rays"], "shadow_rays": cst["shadow_rays"],
                              "nodes_visited": cst["nodes_visited"], "tris_tested": cst["tris_tested"]},
        "e2e": {"value": e2e_rays / e2e_s / 1e6, "unit": METRIC, "h2d_bytes_per_step": C_SHOT_BYTES,
                "d2h_bytes_per_step": int(host.nbytes)},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "k_trace<closest-hit>", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": traffic, "bytes_per_ray": bytes_per_ext, "shadow_bytes_per_ray": bytes_per_sh,
                     "ms_per_launch": ext_ms_per_launch},
        "kernel_ms": {"extend": tot["ms_extend"], "shade": tot["ms_shade"], "connect": tot["ms_connect"],
                      "sort": tot["ms_sort"]},
        "clocks": clk.summary(),
        "scene": {"triangles": sstats["triangles"], "device_bytes": sstats["device_bytes"],
                  "build_ms": sstats["build_ms"]},
    }
    if world == 1 and not args.no_parity:
        line["parity"] = parity_check(ctx, scene, b, shot)
    if not args.no_cpu and world == 1:
        line["cpu_baseline"] = cpu_leg(b, shot, args.cpu_seconds, os.cpu_count() or 1)
    print(json.dumps(line), flush=True)
    if torch_dist:
        torch_dist.destroy_process_group()
    return 0


def ladder_next(n, e, lo, target):
    """Sample count of the next rung of a progressive time-to-RMSE ladder
    after a rung at n samples with error e: doubling (at least lo), or,
    once e is within 4x of the target, the count the 1/sqrt(spp) law
    predicts for the target (+2%), at least n + 1 and at most double."""
    nxt = max(lo, 2 * n)
    if n and e < 4 * target:
        nxt = min(nxt, max(n + 1, int(np.ceil(n * (e / target) ** 2 * 1.02))))
    return nxt


def ladder_time(ladder, tgt, target):
    """Seconds at which a ladder (rungs {spp, seconds, rmse} in order)
    reaches RMSE tgt, and how: the first rung at or below it when tgt is
    the ladder's own target (or the first rung is already below it),
    otherwise interpolated between the two rungs around it on the 1/sqrt(spp)
    law (error linear in 1/sqrt(spp), seconds proportional to spp).  (None,
    None) when no rung reaches it."""
    for i, r in enumerate(ladder):
        if r["rmse"] <= tgt:
            if i == 0 or tgt == target:
                return r["seconds"], "measured"
            p = ladder[i - 1]
            x0, x1 = p["spp"] ** -0.5, r["spp"] ** -0.5
            x = x1 + (tgt - r["rmse"]) * (x0 - x1) / (p["rmse"] - r["rmse"])
            return r["seconds"] / r["spp"] * x ** -2, "interpolated"
    return None, None


def run_denoise_rmse(args):
    """Time to image RMSE 0.01 against the FP64 reference (a seeded 1,024-pixel
    subset of the 1080p workload at 262,144 spp, tests/golden) for the plain
    wavefront path and for the denoised path.

    Plain: progressive rendering, the sample count doubling rung by rung;
    RMSE on the subset with the reference's own variance subtracted.
    Denoised: two progressive films A and B on disjoint frames; the output
    blends the denoise of all their samples with their plain average at the
    weight that minimises the error estimated from the two halves
    (asuna_denoise_blended; weight 0 is the plain path).  Its time
    counts every render and every estimate.  Both ladders step alike: once
    a rung's error is within 4x of the target, the next rung is the count
    the 1/sqrt(spp) law predicts for the target from that rung (plus 2%, at
    most double), so each path stops at the first measured rung below the
    target, close to its crossing; the time at the target is that rung's.
    The other targets' times are interpolated on the same law between the
    rungs around them, for both paths alike.  The network is trained first,
    on the GPU, on pairs the renderer makes of other seeded scenes of the
    same recipe (inputs at several sample counts, a high-count target)."""
    import torch

    import asuna_gb300 as ag
    from asuna_gb300 import denoise as dn

    target = args.rmse_target
    ref = np.load(os.path.join(ROOT, "tests", "golden", "rmse_ref_mixed_1080p.npz"))
    px, mean, refvar = ref["pixels"], ref["mean"], float(ref["var"].mean())

    def rmse(img):
        v = img.reshape(-1, 4)[px, :3].astype(np.float64)
        return float(np.sqrt(max(0.0, np.mean((v - mean) ** 2) - refvar)))

    ctx = ag.Context(0)
    stream = dn.ctx_stream(ctx)
    out = {"metric": f"time to RMSE {target} vs FP64 reference (s)", "unit": "s", "higher_is_better": False,
           "config": {**CONFIG, "reference": f"{len(px)} seeded pixels x {int(ref['spp'])} spp FP64 CPU oracle",
                      "reference_rms_noise": float(np.sqrt(refvar))}}
    # 1. train the denoiser on renderer-made pairs
    t0 = time.time()
    spp_in = tuple(int(x) for x in args.train_spp_in.split(","))
    data = dn.render_pairs(ctx, range(1000, 1000 + args.train_scenes), args.train_size, args.train_size,
                           spp_in=spp_in, spp_target=args.train_target_spp, level=args.train_level)
    gen_s = time.time() - t0
    den = dn.Denoiser(ctx, seed=0, max_pixels=args.train_batch * args.train_crop ** 2, training=True,
                      loss=args.train_loss)
    t1 = time.time()
    losses = dn.train(den, data, steps=args.train_steps, batch=args.train_batch, crop=args.train_crop, lr=1e-3)
    train_s = time.time() - t1
    out["training"] = {"loss": args.train_loss, "scenes": args.train_scenes, "size": args.train_size,
                       "input_spp": list(spp_in),
                       "level": args.train_level,
                       "target_spp": args.train_target_spp, "steps": args.train_steps, "batch": args.train_batch,
                       "crop": args.train_crop, "data_seconds": gen_s, "train_seconds": train_s,
                       "loss_first": float(np.mean(losses[:20])), "loss_last": float(np.mean(losses[-50:]))}
    del data
    # 2. the workload
    b, shot = build_workload(args, verbose=False)
    scene = ctx.create_scene(b.desc())
    W, H = shot.width, shot.height
    inf = dn.Denoiser(ctx, max_pixels=((H + 15) // 16 * 16) * ((W + 15) // 16 * 16))
    inf.set_params(den.get_params())
    del den
    ctx.set_path_budget(16 * W * H * BYTES_PER_PATH)
    chunk = 16

    def render_frames(film, first, count, seed):
        ms = 0.0
        f = first
        while f < first + count:
            k = min(chunk, first + count - f)
            shot.frame0, shot.frames, shot.seed = f, k, seed
            ms += ctx.render(scene, shot, film, stats=True)["ms_total"]
            f += k
        return ms

    def next_count(n, e, lo):
        return ladder_next(n, e, lo, target)

    # 2a. plain path (clocks sampled from here through both ladders)
    clk = ClockSampler(int(os.environ.get("LOCAL_RANK", 0))).__enter__()
    film = ctx.create_film(W, H)
    plain, spp, ms, e = [], 0, 0.0, float("inf")
    t_plain = None
    while spp < args.plain_max_spp:
        nxt = min(next_count(spp, e, 16), args.plain_max_spp)
        ms += render_frames(film, spp, nxt - spp, 0)
        spp = nxt
        e = rmse(film.read(0))
        plain.append({"spp": spp, "seconds": ms / 1e3, "rmse": e})
        if e <= target:
            t_plain = ms / 1e3
            break
    out["plain"] = {"ladder": plain, "seconds_at_target": t_plain, "reached": t_plain is not None}
    # 2b. denoised path: the all-sample denoise blended with the plain
    # average at the weight that minimises the error estimate (weight 0 is the
    # plain path); the denoiser's first calls (workspace, weight staging) run
    # before the clock starts
    fa, fb = ctx.create_film(W, H), ctx.create_film(W, H)
    render_frames(fa, 0, 1, 11)
    render_frames(fb, 0, 1, 12)
    with torch.cuda.stream(stream):
        for _ in range(2):
            inf.blended(fa, fb)
            inf.combined(fa, fb)
    torch.cuda.synchronize()
    fa.clear()
    fb.clear()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dres, half, ms, e = [], 0, 0.0, float("inf")
    t_den = None
    while 2 * half < args.denoise_max_spp:
        nh = min((next_count(2 * half, e, 4) + 1) // 2, args.denoise_max_spp // 2)
        ms += render_frames(fa, half, nh - half, 0)
        ms += render_frames(fb, half, nh - half, 7)
        half = nh
        with torch.cuda.stream(stream):
            ev0.record()
            blend, err_b, err_p, wgt = inf.blended(fa, fb)
            ev1.record()
        ev1.synchronize()
        est_ms = ev0.elapsed_time(ev1)
        ms += est_ms
        e = rmse(blend.cpu().numpy())
        # untimed, for the table: the all-sample denoise alone and its estimate
        with torch.cuda.stream(stream):
            full, err_d, _ = inf.combined(fa, fb)
        e_full = rmse(full.cpu().numpy())
        e_avg = rmse(0.5 * (fa.read(0) + fb.read(0)))
        dres.append({"spp": 2 * half, "seconds": ms / 1e3, "estimate_ms": est_ms, "weight": wgt,
                     "err_estimate": err_b, "err_plain_estimate": err_p, "err_denoised_estimate": err_d,
                     "rmse": e, "rmse_denoised_all": e_full, "rmse_plain_average": e_avg})
        if e <= target:
            t_den = ms / 1e3
            break
    clk.__exit__(None, None, None)
    out["clocks"] = clk.summary()
    out["denoised"] = {"ladder": dres, "seconds_at_target": t_den, "reached": t_den is not None}
    # the other targets: the time between the two rungs around the target,
    # interpolated on the 1/sqrt(spp) law (error linear in 1/sqrt(spp),
    # seconds proportional to spp), for both ladders; the main target is the
    # measured rung
    def at(ladder, tgt):
        return ladder_time(ladder, tgt, target)

    rows = []
    for tgt in (0.05, 0.03, 0.02, target):
        tp, kp = at(plain, tgt)
        td, kd = at(dres, tgt)
        rows.append({"rmse": tgt, "plain_seconds": tp, "denoised_seconds": td,
                     "speedup": (tp / td) if (tp and td) else None, "how": kd or kp})
    out["targets"] = rows
    # denoiser forward throughput at 1080p
    with torch.cuda.stream(stream):
        for _ in range(3):
            inf.denoise(fa)
        ev0.record()
        for _ in range(10):
            inf.denoise(fa)
        ev1.record()
    ev1.synchronize()
    fwd_ms = ev0.elapsed_time(ev1) / 10
    fl = dn.forward_flops(dn.DEFAULT_CHANNELS, (H + 15) // 16 * 16, (W + 15) // 16 * 16)
    out["denoiser_forward"] = {"ms": fwd_ms, "tflops": fl / (fwd_ms * 1e-3) / 1e12, "flop": fl}
    out["value"] = t_den
    out["speedup"] = (t_plain / t_den) if (t_plain and t_den) else None
    print(json.dumps(out), flush=True)
    return 0


def run_denoise_forward(args):
    """Denoiser forward pass at the workload resolution (padded to 16):
    device time per call on the context stream, tcgen05 and mma.sync
    convolutions, against the measured dense bf16 peak."""
    import torch

    import asuna_gb300 as ag
    from asuna_gb300 import denoise as dn

    ctx = ag.Context(0)
    stream = dn.ctx_stream(ctx)
    H, W = args.height, args.width
    rng = np.random.default_rng(0)
    imgs = [torch.from_numpy(rng.uniform(0, 1, (1, H, W, 4)).astype(np.float32)).cuda() for _ in range(4)]
    hp, wp = (H + 15) // 16 * 16, (W + 15) // 16 * 16
    fl = dn.forward_flops(dn.DEFAULT_CHANNELS, hp, wp)
    peak, kind = 1900.0, "fallback"
    pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pp):
        with open(pp) as f:
            peak, kind = float(json.load(f)["bf16_tflops"]), "measured"
    torch.cuda.synchronize()
    res = {}
    for tm in (True, False):
        d = dn.Denoiser(ctx, seed=1, max_pixels=hp * wp, tensor_memory=tm)
        out = torch.empty_like(imgs[0])
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                d.forward(*imgs, out=out)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(args.steps):
                d.forward(*imgs, out=out)
            e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        res["tcgen05" if tm else "mma_sync"] = {"ms": ms, "tflops": fl / (ms * 1e-3) / 1e12}
        d.close()
    tc = res["tcgen05"]
    print(json.dumps({"metric": "denoiser forward TFLOP/s", "value": tc["tflops"], "unit": "TFLOP/s",
                      "higher_is_better": True, "steps": args.steps, "warmup": args.warmup, "ms_per_step": tc["ms"],
                      "config": {"workload": f"U-Net 32/48/64/96/128, 1 x {hp} x {wp}, bf16 NHWC, fp32 accumulation",
                                 "flop": fl},
                      "roofline": {"bound": "tensor", "achieved": tc["tflops"], "peak": peak, "unit": "TFLOP/s",
                                   "frac": tc["tflops"] / peak, "peak_kind": kind},
                      "variants": res}), flush=True)
    return 0


SERVE_CATALOG = [(4, 7), (8, 6), (8, 7), (16, 6), (16, 7), (24, 7), (32, 6), (32, 7), (48, 7), (64, 6), (64, 7),
                 (12, 7)]  # (spheres, level): 0.33M-21M triangles


def run_serve(args):
    """Serving loop: requests arrive as a Poisson process (wall clock) at
    --serve-rate per second; each names a scene of a catalog of the mixed
    recipe (4-64 spheres, 0.33-21M triangles) registered with the server,
    which builds a scene on the device when its first request is admitted
    (charged to the memory budget, 150 GB by default; idle scenes are
    dropped, least recently used first, when an admission needs the room),
    a resolution from {512x512, 1280x720, 1920x1080}, a sample count from
    {4, 16, 64}, a seeded camera and, for a quarter of them, the denoise flag (two half renders blended with their denoise).  The
    denoiser's weights are its initialisation: request latency does not
    depend on their values.  Reports latency percentiles (arrival to
    finish), Msamples/s, the rejection and queueing rates and the scene
    builds."""
    from asuna_gb300 import denoise as dn
    from asuna_gb300 import scenes
    from asuna_gb300.serving import Server, poisson_load

    rng = np.random.default_rng(7)
    srv = Server(slots=args.serve_slots, frames_per_chunk=args.serve_chunk, max_batch=8,
                 max_queue=args.serve_max_queue, memory_budget=int(args.serve_budget_gb * (1 << 30)))
    t0 = time.time()
    pool = []
    for k, (n, lvl) in enumerate(SERVE_CATALOG):
        b, _ = scenes.mixed_scene(64, 64, frames=1, n_spheres=n, level=lvl, seed=3000 + k)
        pool.append((srv.register_scene(b.desc()), b, n * 20 * 4 ** lvl))
    gen_s = time.time() - t0
    import asuna_gb300 as ag

    ctx = ag.Context(0)
    net = dn.Denoiser(ctx, seed=0, max_pixels=1088 * 1920)
    srv.set_denoiser(net.get_params(), max_pixels=1088 * 1920)
    net.close()
    res = [(512, 512), (1280, 720), (1920, 1080)]
    reqs, flags = [], []
    for i in range(args.serve_requests):
        sid, b, _ = pool[int(rng.integers(len(pool)))]
        w, h = res[int(rng.integers(3))]
        spp = int((4, 16, 64)[int(rng.integers(3))])
        ang = float(rng.uniform(0, 2 * np.pi))
        eye = (30.0 * np.sin(ang), float(rng.uniform(0.0, 10.0)), 30.0 * np.cos(ang))
        reqs.append((sid, scenes.mixed_shot(b, w, h, spp, eye=eye, seed=i)))
        flags.append(bool(rng.random() < args.serve_denoise_frac))
    out = poisson_load(srv, reqs, rate_hz=args.serve_rate, seed=11, denoise=flags)
    st = srv.stats()
    srv.close()
    out.pop("films")
    line = {"metric": "serving latency p99 (s)", "value": out["p99_s"], "unit": "s", "higher_is_better": False,
            "n_gpus": 1, "data": "synthetic (seeded procedural scenes)",
            "config": {"workload": f"Poisson {args.serve_rate} req/s, {args.serve_requests} requests, "
                                   f"{len(pool)} registered scenes of 0.33-21M triangles built at admission, "
                                   "512^2 / 1280x720 / 1920x1080, 4 / 16 / 64 spp, depth 12, "
                                   f"{args.serve_denoise_frac:.0%} denoised",
                       "slots": args.serve_slots, "frames_per_chunk": args.serve_chunk,
                       "max_queue": args.serve_max_queue, "memory_budget_gb": args.serve_budget_gb,
                       "scene_triangles": [p[2] for p in pool], "scene_generation_s": gen_s},
            **out, "denoised_requests": int(sum(flags)), "server_stats": st}
    print(json.dumps(line), flush=True)
    return 0


def run_batch(args):
    """Batched shots: 32 shots of the mixed recipe with 8 instances (2.6M
    triangles) on a sphere of radius 15 around the origin, resolutions from
    {256^2, 512^2, 1280x720, 1920x1080} and sample counts from {1, 4, 16, 64}
    (seeded), depth 12; all shots in one asuna_render_batch call (one
    wavefront per path budget, replayed as a CUDA graph) against the same
    shots as 32 sequential asuna_render calls.  Device time of each, after
    warm-up; Msamples/s and Mrays/s."""
    import asuna_gb300 as ag
    from asuna_gb300 import scenes

    rng = np.random.default_rng(5)
    b, _ = scenes.mixed_scene(64, 64, frames=1, n_spheres=8, level=7, seed=4321)
    ctx = ag.Context(0)
    scene = ctx.create_scene(b.desc())
    res = [(256, 256), (512, 512), (1280, 720), (1920, 1080)]
    shots, films = [], []
    for k in range(32):
        w, h = res[int(rng.integers(4))]
        spp = int((1, 4, 16, 64)[int(rng.integers(4))])
        z = float(rng.uniform(-1.0, 1.0))
        a = float(rng.uniform(0.0, 2.0 * np.pi))
        r = np.sqrt(1.0 - z * z)
        eye = (15.0 * r * np.cos(a), 15.0 * z, 15.0 * r * np.sin(a))
        shots.append(scenes.mixed_shot(b, w, h, spp, eye=eye, at=(0.0, 0.0, 0.0), seed=k))
        films.append(ctx.create_film(w, h))
    samples = sum(s.width * s.height * s.frames for s in shots)

    def batched():
        return ctx.render_batch(scene, shots, films, stats=True)

    def sequential():
        tot = {"ms_total": 0.0, "extend_rays": 0, "shadow_rays": 0}
        for s, f in zip(shots, films):
            st = ctx.render(scene, s, f, stats=True)
            for k in tot:
                tot[k] += st[k]
        return tot

    out = {}
    for name, fn in (("sequential", sequential), ("batched", batched)):
        for _ in range(args.warmup):
            fn()
        ms, rays = [], 0
        for _ in range(args.steps):
            st = fn()
            ms.append(st["ms_total"])
            rays = st["extend_rays"] + st["shadow_rays"]
        m = float(np.median(ms))
        out[name] = {"ms": m, "msamples_per_s": samples / (m * 1e-3) / 1e6, "mrays_per_s": rays / (m * 1e-3) / 1e6}
    line = {"metric": "batched shots speed-up", "value": out["sequential"]["ms"] / out["batched"]["ms"],
            "unit": "x", "higher_is_better": True, "n_gpus": 1, "data": "synthetic (seeded procedural scene)",
            "config": {"workload": "32 shots, mixed recipe with 8 level-7 instances (2.6M triangles), radius-15 "
                                   "sphere of cameras, 256^2..1920x1080, 1..64 spp, depth 12",
                       "samples_per_call": samples, "steps": args.steps, "warmup": args.warmup},
            **out}
    print(json.dumps(line), flush=True)
    return 0


C_SHOT_BYTES = 340  # sizeof(asuna_shot): the only host->device input of a step
NODE_BYTES = 64  # one binary BVH node
BYTES_PER_PATH = 244  # wavefront state per path slot (asuna_gb300/csrc/engine.cu)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=48)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--spheres", type=int, default=64)
    ap.add_argument("--level", type=int, default=7)
    ap.add_argument("--frames-per-step", type=int, default=0, help="0 = autotune")
    ap.add_argument("--ray-sort", type=int, default=3, choices=(0, 1, 2, 3),
                    help="with --frames-per-step: extend-queue sort mode")
    ap.add_argument("--traversal", default="",
                    help="with --frames-per-step: refill extend,refill shadow,speculate extend,speculate shadow,"
                         "blocks per SM (the autotuner's traversal tuple)")
    ap.add_argument("--shape", default="",
                    help="with --frames-per-step: traversal threads per block,shared-memory stack entries")
    ap.add_argument("--shadow-occupancy", type=int, default=0, choices=(0, 8, 10, 12),
                    help="with --frames-per-step and --traversal: the occlusion pass's blocks per SM")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-seconds", type=float, default=10.0, help="--impl reference: CPU seconds per step at most")
    ap.add_argument("--ref-budget", type=float, default=100.0,
                    help="--impl reference: CPU seconds of the warm-up and timed steps together")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-parity", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--denoise-rmse", action="store_true",
                    help="time to RMSE 0.01 vs the FP64 reference, plain vs denoised path")
    ap.add_argument("--rmse-target", type=float, default=0.01)
    ap.add_argument("--plain-max-spp", type=int, default=32768)
    ap.add_argument("--denoise-max-spp", type=int, default=32768)
    ap.add_argument("--train-scenes", type=int, default=160)
    ap.add_argument("--train-size", type=int, default=256)
    ap.add_argument("--train-spp-in", default="4,16,64,256,1024,4096")
    ap.add_argument("--train-target-spp", type=int, default=65536)
    ap.add_argument("--train-level", type=int, default=6)
    ap.add_argument("--train-steps", type=int, default=40000)
    ap.add_argument("--train-batch", type=int, default=16)
    ap.add_argument("--train-crop", type=int, default=128)
    ap.add_argument("--train-loss", default="l1log", choices=("l1log", "relmse"),
                    help="L1 on log radiance, or relative MSE (unbiased with noisy targets)")
    ap.add_argument("--denoise-forward", action="store_true", help="denoiser forward pass at the workload size")
    ap.add_argument("--serve", action="store_true", help="serving loop: Poisson arrivals, latency percentiles")
    ap.add_argument("--batch", action="store_true", help="32 batched shots vs 32 sequential calls")
    ap.add_argument("--serve-rate", type=float, default=20.0)
    ap.add_argument("--serve-requests", type=int, default=10000)
    ap.add_argument("--serve-denoise-frac", type=float, default=0.25)
    ap.add_argument("--serve-slots", type=int, default=3)
    ap.add_argument("--serve-chunk", type=int, default=16)
    ap.add_argument("--serve-max-queue", type=int, default=256)
    ap.add_argument("--serve-budget-gb", type=float, default=150.0,
                    help="device memory budget for scenes and films (a small one makes the server drop and rebuild)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.denoise_rmse:
        return run_denoise_rmse(args)
    if args.denoise_forward:
        return run_denoise_forward(args)
    if args.serve:
        return run_serve(args)
    if args.batch:
        return run_batch(args)
    return run(args)


if __name__ == "__main__":
    sys.exit(main())
