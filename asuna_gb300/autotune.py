"""Autotuner of the wavefront launch configuration.

Picks, for one scene and shot, the number of frames packed into one wavefront
(the path-queue capacity: more frames keep the deep-bounce passes full) and
the persistent-grid sizes of the traversal and shading kernels, by timing
short renders of the real workload on the device (CUDA events inside the
library).  Frames rendered while tuning use frame indices far from the
caller's, so they never touch its sample streams.
"""
import itertools

from ._abi import ERR_OOM, AsunaError

BYTES_PER_PATH = 244  # wavefront state per path slot (asuna_gb300/csrc/engine.cu)


def tune(ctx, scene, shot, film, frames_options=(1, 2, 4, 8, 16, 32, 64, 128, 256), trace_options=(0, 6),
         shade_options=(0, 2), refill_options=(4, 8, 16, 24), occupancy_options=(8, 10, 12),
         shape_options=((64, 24), (256, 24), (128, 16), (128, 32)), memory_bytes=160 << 30, reps=2,
         frame_base=1 << 20):
    """Returns {"frames": f, "trace_blocks_per_sm": t, "shade_blocks_per_sm": s, "traversal": (refill
    extend, refill shadow, speculate extend, speculate shadow, traversal blocks per SM), "shape": (threads
    per block, shared-memory stack entries), "shadow_occupancy": the occlusion pass's blocks per SM,
    "ray_sort": 0..3, "mrays": best, "trials": [...]} and leaves the context configured with the best
    choice.  Coordinate search: frames, then grids, then the traversal kernel variant and the refill
    thresholds and speculation of each pass, then extend-queue sorting, then the refill thresholds again
    under it, then the traversal block size and the traversal stack's shared-memory depth, then the
    occlusion pass's kernel variant on its own."""
    npix = shot.width * shot.height
    saved = (shot.frame0, shot.frames)
    trials = []
    best = None

    trav = [8, 8, 1, 1, 8]
    ctx.set_ray_sort(0)

    def run(frames, t, s):
        ctx.set_traversal(*trav)
        return run_set(frames, t, s)

    def run_set(frames, t, s):  # with the traversal settings already made
        ctx.set_launch(t, s)
        ctx.set_path_budget(max(frames * npix * BYTES_PER_PATH, 1))
        shot.frames = frames
        vals = []
        for r in range(reps):
            shot.frame0 = frame_base + r * frames
            st = ctx.render(scene, shot, film, stats=True)
            vals.append((st["extend_rays"] + st["shadow_rays"]) / (st["ms_total"] * 1e3))
        return max(vals)

    try:
        cands = [f for f in frames_options if f * npix * BYTES_PER_PATH <= memory_bytes]
        # frames first with the default grids, then the grids at the best frame count
        for f in cands:
            try:
                v = run(f, 0, 0)
            except AsunaError as e:
                # the device has less free memory than the cap assumed: larger
                # wavefronts will not fit either
                if e.code != ERR_OOM or best is None:
                    raise
                trials.append({"frames": f, "trace": 0, "shade": 0, "mrays": None, "error": "out of memory"})
                break
            trials.append({"frames": f, "trace": 0, "shade": 0, "mrays": v})
            if best is None or v > best["mrays"]:
                best = {"frames": f, "trace_blocks_per_sm": 0, "shade_blocks_per_sm": 0, "mrays": v}
        for t, s in itertools.product(trace_options, shade_options):
            if t == 0 and s == 0:
                continue
            v = run(best["frames"], t, s)
            trials.append({"frames": best["frames"], "trace": t, "shade": s, "mrays": v})
            if v > best["mrays"]:
                best = {**best, "trace_blocks_per_sm": t, "shade_blocks_per_sm": s, "mrays": v}
        best["traversal"] = tuple(trav)
        # traversal: kernel occupancy, then refill threshold and speculation of each pass
        steps = [(4, o) for o in occupancy_options if o != 8]
        for k in (1, 0):
            steps += [(k, r) for r in refill_options if r != 8] + [(k + 2, 0)]
        for index, value in steps:
            trav = list(best["traversal"])
            trav[index] = value
            v = run(best["frames"], best["trace_blocks_per_sm"], best["shade_blocks_per_sm"])
            trials.append({"frames": best["frames"], "traversal": tuple(trav), "mrays": v})
            if v > best["mrays"]:
                best = {**best, "traversal": tuple(trav), "mrays": v}
        # extend-queue sorting before secondary passes (mode 1: octant x 4^3
        # origin cells, 2: octant x 8^3 in Morton order, 3: the same, origin major)
        trav = list(best["traversal"])
        best["ray_sort"] = 0
        for mode in (1, 2, 3):
            ctx.set_ray_sort(mode)
            v = run(best["frames"], best["trace_blocks_per_sm"], best["shade_blocks_per_sm"])
            trials.append({"frames": best["frames"], "ray_sort": mode, "mrays": v})
            if v > best["mrays"]:
                best = {**best, "ray_sort": mode, "mrays": v}
        ctx.set_ray_sort(best["ray_sort"])
        # sorted queues walk the BVH more coherently: the refill thresholds
        # again, with the chosen sort
        for index, value in [(0, r) for r in refill_options + (32,)] + [(1, r) for r in refill_options]:
            trav = list(best["traversal"])
            if trav[index] == value:
                continue
            trav[index] = value
            v = run(best["frames"], best["trace_blocks_per_sm"], best["shade_blocks_per_sm"])
            trials.append({"frames": best["frames"], "traversal": tuple(trav), "ray_sort": best["ray_sort"],
                           "mrays": v})
            if v > best["mrays"]:
                best = {**best, "traversal": tuple(trav), "mrays": v}
        # block shape and the shared-memory part of the traversal stack
        trav = list(best["traversal"])
        best["shape"] = (0, 0)
        for shape in shape_options:
            ctx.set_traversal_shape(*shape)
            v = run(best["frames"], best["trace_blocks_per_sm"], best["shade_blocks_per_sm"])
            trials.append({"frames": best["frames"], "shape": shape, "mrays": v})
            if v > best["mrays"]:
                best = {**best, "shape": shape, "mrays": v}
        ctx.set_traversal_shape(*best["shape"])
        # the occlusion pass's kernel variant apart from the extend pass's
        # (shorter queues, no hit record to keep: its best occupancy differs)
        trav = list(best["traversal"])
        ext = trav[4]
        best["shadow_occupancy"] = ext
        for occ in occupancy_options:
            if occ == ext:
                continue
            ctx.set_traversal(*trav)
            ctx.set_traversal_occupancy(ext, occ)
            v = run_set(best["frames"], best["trace_blocks_per_sm"], best["shade_blocks_per_sm"])
            trials.append({"frames": best["frames"], "shadow_occupancy": occ, "mrays": v})
            if v > best["mrays"]:
                best = {**best, "shadow_occupancy": occ, "mrays": v}
    finally:
        shot.frame0, shot.frames = saved
    ctx.set_traversal(*best["traversal"])
    if "shadow_occupancy" in best:
        ctx.set_traversal_occupancy(best["traversal"][4], best["shadow_occupancy"])
    ctx.set_traversal_shape(*best.get("shape", (0, 0)))
    ctx.set_launch(best["trace_blocks_per_sm"], best["shade_blocks_per_sm"])
    ctx.set_path_budget(best["frames"] * npix * BYTES_PER_PATH)
    film.clear()
    best["trials"] = trials
    return best
