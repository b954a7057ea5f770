"""Benchmark of the rendering hot path on one GB300 (or N replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload: the large plain-pipeline frame -- a 1,048,576-triangle displaced
grid-sphere (3-octave value noise, 5%) seen from a camera close to the
surface, the clipping geometry shader, 3840x2160 RGBA8 + f32 depth, bilinear
textured Blinn-Phong (seeded synthetic inputs; no dataset).  One step = one
frame: framebuffer clear + vertex stage + clip GS + setup/binning + raster.

Reported (one JSON line on rank 0):
  value  input triangles per second (Mtris/s) with mesh, texture and
         framebuffer resident in HBM, device time of the K steps (CUDA events
         on the pipeline's stream; L2 flushed with a 256 MiB write between
         steps, outside the timed events)
  e2e    the same metric through the C ABI with host buffers: every step
         copies mesh + texture from pinned host memory, renders, and reads the
         colour and depth planes back (wall clock per step)
  roofline  HBM roofline of the raster kernel (and of the whole frame)
  cpu_baseline  the CPU restatement of the reference path (oracle/), all
         host threads, timed on one whole frame
  other_frames  the small plain frame (icosphere, 1024^2) and the ordering /
         tiny-triangle stress frame (16.8M tiny + 4,096 alpha triangles)
  batched  256 draws of uneven sizes: one batch (one launch per stage, CUDA
         graph) against the plain per-draw pipeline
  served   a Poisson request stream (2,000 req/s) through the serving loop
         and through the plain per-request loop: p50/p99 latency, throughput,
         saturated throughput of both, and a sweep of offered rates against
         the latency bound (2 x the plain single-request p99)

--impl reference times the reference's CPU path (the oracle restatement; the
Rust reference cannot be built here) on the same workload and metric.
Multi-GPU: replicas only (each rank renders its own frame; no collective on
the data path).
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
sys.path.insert(0, os.path.join(ROOT, "rust-softrender_gb300"))

WORKLOAD = "gridsphere_1048576tri_clipgs_3840x2160_rgba8_depth_textured_blinn_phong"
METRIC = "Mtris/s (1,048,576-tri clipped textured grid-sphere, 3840x2160 RGBA8+f32 depth, 1 GB300)"
L2_FLUSH_BYTES = 256 << 20


# ---------------------------------------------------------------- helpers
def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value, device):
    """The largest `value` over all ranks (every rank gets it); the job's time
    is the slowest replica's."""
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, max_ms):
    """Whole-job throughput in millions of units per second: every rank
    processes units_per_rank in the timed steps, the job takes max_ms per step."""
    return units_per_rank * world / (max_ms * 1e-3) / 1e6


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples every 200 ms while running."""
    FIELDS = ("uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid):
        self.uuid = uuid
        self.out = tempfile.NamedTemporaryFile(prefix="clocks", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.out.close()
        with open(self.out.name) as f:
            res = parse_clock_samples(f, self.uuid)
        os.unlink(self.out.name)
        return res


def parse_clock_samples(lines, uuid=""):
    """Median SM clock, the maximum clock and the throttle reasons seen in
    nvidia-smi samples of ClockSampler.FIELDS (csv, no header, no units),
    keeping the lines of the GPU `uuid` (all when empty); None without
    samples."""
    sm, mx, reasons = [], None, set()
    names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
    for line in lines:
        c = [x.strip() for x in line.split(",")]
        if len(c) < 9 or (uuid and uuid not in c[0]):
            continue
        try:
            sm.append(float(c[1]))
            mx = float(c[2])
        except ValueError:
            continue
        for n, v in zip(names, c[5:9]):
            if v.lower().startswith("active"):
                reasons.add(n)
    if not sm:
        return None
    return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def subsample_scene(scene, every):
    """Every `every`-th triangle of the scene (all vertices kept)."""
    import copy
    sc = copy.copy(scene)
    tris = scene.indices.reshape(-1, 3)[::every]
    sc.indices = np.ascontiguousarray(tris.reshape(-1))
    return sc


def scenes_tiles(scene):
    """The scene's semantic tiles (fragment.rs:188-216), from the oracle."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    return oracle.tiles(scene.width, scene.height, *scene.tile)


def cpu_frame_estimate(scene, every, tiles, tile_begin=0, threads=None):
    """Times the oracle (the reference path restated, all host threads) on a
    bounded sample and extrapolates to one full frame, from the stage times
    the oracle measures inside one render call:
      vertex    vertex stage over all vertices
      geometry  geometry stage (clip GS + finish) on every `every`-th triangle
      raster    fragment stage of that sample over `tiles` of the frame's
                tiles, spread over the frame (1 in n_tiles // tiles, the
                offset rotating with tile_begin)
    frame = vertex + every * geometry + every * raster * n_tiles / tiles
    (the reference's geometry cost and its per-tile cost are linear in the
    primitive count: every tile visits every primitive; screen content is
    uneven, so a contiguous run of tiles would extrapolate its own density
    to the frame)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    threads = threads or os.cpu_count()
    sc = subsample_scene(scene, every)
    n_tiles = len(oracle.tiles(scene.width, scene.height, *scene.tile))
    tiles = min(tiles, n_tiles)
    step = max(1, n_tiles // tiles)
    first = tile_begin % step
    picked = range(first, min(n_tiles, first + step * tiles), step)
    t0 = time.perf_counter()
    _, st, _ = oracle.render(sc, n_threads=threads, tile_begin=first, tile_end=picked.stop, tile_step=step)
    wall = time.perf_counter() - t0
    frame = st["vertex_s"] + every * st["geometry_s"] + every * st["raster_s"] * n_tiles / len(picked)
    if every == 1 and len(picked) == n_tiles:
        sample = ("one full frame: all %d triangles through vertex+clip GS, rasterised over all %d tiles; "
                  "%.1f s of CPU wall time" % (scene.n_tris, n_tiles, wall))
    else:
        sample = ("1 in %d of %d triangles through vertex+clip GS, rasterised over %d of %d tiles "
                  "(1 in %d, spread over the frame), stage times extrapolated linearly to the frame; "
                  "%.1f s of CPU wall time" % (every, scene.n_tris, len(picked), n_tiles, step, wall))
    return frame, sample, threads


# ------------------------------------------------------------------ ours
def run_ours(args, rank, world, local):
    import torch
    import softrender as sr
    from softrender import scenes

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    scene = scenes.grid_sphere_scene()
    n_tris = scene.n_tris
    pl, mesh, tex = sr.prepare_scene(scene)
    stream = torch.cuda.Stream(device=dev)
    pl.set_stream(stream.cuda_stream)
    clear = list(scene.clear_bytes())
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def frame():
        pl.clear(clear)
        sr.submit_scene(pl, mesh, tex, scene)

    for _ in range(max(3, args.warmup)):
        frame()
        st = pl.sync()
        if st != 0:
            raise RuntimeError("warm-up draw failed: status %d" % st)
    stats = pl.stats()
    launches_per_step = stats["kernel_launches"] + 2          # + colour and depth clear fills

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    uuid = str(getattr(torch.cuda.get_device_properties(local), "uuid", "") or "")
    clocks = ClockSampler(uuid)
    # The timed steps last tens of milliseconds, shorter than the sampler's
    # 200 ms period: keep the GPU under the same frames for about a second
    # before them (untimed), so the clock samples cover the load the timed
    # steps run under.
    t_load = time.perf_counter()
    with torch.cuda.stream(stream):
        while time.perf_counter() - t_load < 1.2:
            for _ in range(16):
                flush.zero_()
                frame()
            st = pl.sync()
            if st != 0:
                raise RuntimeError("load draws failed: status %d" % st)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t_wall = time.perf_counter()
    with torch.cuda.stream(stream):
        for e0, e1 in evs:
            flush.zero_()                      # L2 flush, outside the timed events
            e0.record(stream)
            frame()
            e1.record(stream)
    st = pl.sync()
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    if clk is not None:
        clk["window"] = "1.2 s of the same frames (untimed) followed by the timed steps"
    if st != 0:
        raise RuntimeError("timed draws failed: status %d" % st)
    step_ms = [a.elapsed_time(b) for a, b in evs]
    ms = float(np.mean(step_ms))
    if world > 1:
        ms = max_over_ranks(ms, dev)
    stats = pl.stats()

    # per-stage device times (a separate profiled pass, same work)
    pl.set_profiling(True)
    stage = {}
    for _ in range(5):
        flush.zero_()
        frame()
        pl.sync()
        for k, v in pl.stats()["stage_ms"].items():
            stage.setdefault(k, []).append(v)
    pl.set_profiling(False)
    stage = {k: float(np.median(v)) for k, v in stage.items()}

    # end to end through the C ABI with host buffers: every step uploads the
    # mesh and texture from pinned host memory, renders, and copies colour and
    # depth back to pinned host memory.  Two pipelines (each with its own
    # mesh, texture and stream) alternate, so step i's copies overlap step
    # i+1's work; a pipeline's host result is complete when it is synced
    # before its next use and at the end.
    e2e = None
    if not args.no_e2e:
        keep = []

        def pinned(a):
            t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
            keep.append(t)
            return t.numpy()
        from softrender._lib import lib
        h_planes = [pinned(p) for p in scene.planes]
        h_idx = pinned(scene.indices)
        h_tex = pinned(scene.texture)
        pl2, mesh2, tex2 = sr.prepare_scene(scene)
        stream2 = torch.cuda.Stream(device=dev)
        pl2.set_stream(stream2.cuda_stream)
        sets = []
        for p_, m_, t_, s_ in ((pl, mesh, tex, stream), (pl2, mesh2, tex2, stream2)):
            hc = pinned(np.zeros((scene.height, scene.width), dtype=np.uint32))
            hd = pinned(np.zeros((scene.height, scene.width), dtype=np.float32))
            sets.append((p_, m_, t_, s_, hc, hd))
        h2d = sum(p.nbytes for p in h_planes) + h_idx.nbytes + h_tex.nbytes
        d2h = sets[0][4].nbytes + sets[0][5].nbytes

        def e2e_step(i):
            p_, m_, t_, s_, hc, hd = sets[i % 2]
            st_ = p_.sync()                                  # its previous result is complete
            if st_ != 0:
                raise RuntimeError("e2e step failed: %d" % st_)
            m_.update(h_planes, h_idx, s_.cuda_stream)
            t_.update(h_tex, s_.cuda_stream)
            p_.clear(clear)
            sr.submit_scene(p_, m_, t_, scene)
            rc = lib().sr_framebuffer_read_async(p_.handle, hc.ctypes.data, hd.ctypes.data, None)
            if rc != 0:
                raise RuntimeError("e2e read failed: %d" % rc)
        for i in range(4):
            e2e_step(i)
        for st_ in sets:
            st_[0].sync()
        e2e_steps = max(6, min(args.steps, 20))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(e2e_steps):
            e2e_step(i)
        for st_ in sets:
            if st_[0].sync() != 0:
                raise RuntimeError("e2e final sync failed")
        e2e_ms = (time.perf_counter() - t0) / e2e_steps * 1e3
        pl2.destroy()
        mesh2.free()
        tex2.free()
        e2e = {"value": round(n_tris / (e2e_ms * 1e-3) / 1e6 * world, 3), "unit": "Mtris/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "ms_per_step": round(e2e_ms, 4),
               "note": "two pipelines alternate so a step's copies overlap the next step's work"}

    pl.destroy()
    return dict(ms=ms, step_ms=step_ms, stats=stats, stage=stage, clocks=clk, e2e=e2e, scene=scene,
                launches=launches_per_step * args.steps, wall_s=t_wall)


# ------------------------------------------------------- batched / served
def run_batched():
    """256 independent draws of uneven sizes (triangles log-uniform in
    [500, 200000], frames of 256^2 .. 2048^2, random cameras; seeded), rendered
    (a) per request through the plain pipeline -- clear, sr_render, sr_sync --
    and (b) as one batch (sr_batch_render: one launch per stage, CUDA graph
    replay, tuned launch configuration).  Wall time per set of 256, best of
    several repetitions after warm-up."""
    import softrender as sr
    from softrender import scenes
    inst = scenes.batch_instances()
    T = []
    for sc in inst:
        fb = sr.Framebuffer(sc.width, sc.height, sc.color_format, sc.depth, sc.stencil)
        pl = sr.Pipeline.from_framebuffer(fb, sc.uniforms)
        m = sr.Mesh(sc.planes, sc.indices)
        T.append((pl, m, sr.draw_for_scene(sc, m), sc))
    tris = sum(sc.n_tris for sc in inst)
    px = sum(sc.width * sc.height for sc in inst)

    def plain_once():
        for pl, m, d, sc in T:
            pl.clear(list(sc.clear_bytes()))
            sr.submit_scene(pl, m, None, sc)
            pl.sync()
    plain_once()
    plain_once()
    plain = min(_timed(plain_once) for _ in range(5))
    b = sr.Batch(use_graphs=True, autotune=True)
    arr = b.items([(pl, d, sc.clear_bytes()) for pl, m, d, sc in T])

    def batch_once():
        st = b.render_items(arr)
        if st != 0 or b.sync() != 0:
            raise RuntimeError("batch failed: %d" % st)
    batch_once()                                   # tunes this size class, records the graph
    for _ in range(3):
        batch_once()
    batched = min(_timed(batch_once) for _ in range(10))
    st = b.stats()
    cfg = b.config()
    # one target checked against its plain rendering
    plain_once()
    ref = T[0][0].read()[0].copy()
    batch_once()
    same = bool(np.array_equal(ref, T[0][0].read()[0]))
    b.destroy()
    for pl, m, d, sc in T:
        pl.destroy()
        m.free()
    return {"workload": "256 instances, grid-spheres of 500-200,000 tris (log-uniform), frames 256^2-2048^2, "
                        "RGBA8 + f32 depth, Blinn-Phong, no GS, random cameras (seed 4)",
            "triangles": int(tris), "pixels": int(px), "fragments": int(st["fragments"]),
            "batched_ms": round(batched * 1e3, 3), "batched_mtris_per_s": round(tris / batched / 1e6, 1),
            "plain_ms": round(plain * 1e3, 3), "plain_mtris_per_s": round(tris / plain / 1e6, 1),
            "speedup_vs_plain": round(plain / batched, 2), "cuda_graph": True,
            "launch_config": {"bins_per_primitive": cfg[0], "big_threshold": cfg[1], "raster_ctas_per_sm": cfg[2]},
            "kernel_launches_per_batch": int(st["kernel_launches"]), "target0_equals_plain": same,
            "timing": "host wall clock per 256 draws incl. sync, best of repetitions"}


def run_frames():
    """The other frame workloads, device time per frame (CUDA events on the
    pipeline's stream, median of a few frames after warm-up): the small plain
    pipeline (icosphere 5,120 tris, 1024^2 RGBA f32 + f32 depth, Blinn-Phong)
    and the ordering/tiny-triangle stress (16,777,216 tiny tris + 4,096 alpha
    tris, 2048^2 RGBA8 + f32 depth + u8 stencil, over-blend, stencil
    increment, wrapping and saturating)."""
    import torch
    import softrender as sr
    from softrender import _abi as A
    from softrender import scenes
    import copy
    out = {}
    stress = scenes.stress_scene()                 # stencil Increment, wrapping
    stress_sat = copy.copy(stress)                 # the same frame, Increment saturating
    stress_sat.stencil_wrap = 0
    for key, sc, n in (("icosphere_5120tri_1024x1024_rgba32f", scenes.icosphere_scene(1024, 1024), 20),
                       ("stress_16777216tiny_4096alpha_2048x2048_stencil", stress, 3),
                       ("stress_16777216tiny_4096alpha_2048x2048_stencil_saturate", stress_sat, 3)):
        pl, mesh, tex = sr.prepare_scene(sc)
        stream = torch.cuda.Stream()
        pl.set_stream(stream.cuda_stream)
        clear = list(sc.clear_bytes()) if sc.color_format == A.SR_COLOR_RGBA8 else sc.clear_color
        def frame():
            pl.clear(clear)
            sr.submit_scene(pl, mesh, tex, sc)
        for _ in range(2):
            frame()
            if pl.sync() != 0:
                raise RuntimeError("%s failed" % key)
        ts = []
        for _ in range(n):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            frame()
            e1.record(stream)
            pl.sync()
            ts.append(e0.elapsed_time(e1))
        ms = float(np.median(ts))
        st = pl.stats()
        out[key] = {"ms_per_frame": round(ms, 4), "mtris_per_s": round(sc.n_tris / ms / 1e3, 2),
                    "gfrag_per_s": round(st["fragments"] / ms / 1e6, 3), "triangles": int(sc.n_tris),
                    "fragments": int(st["fragments"]),
                    "frame_algorithmic_bytes": int(sc.algorithmic_bytes()),
                    "frame_roofline_gbs": round(sc.algorithmic_bytes() / ms / 1e6, 2)}
        pl.destroy()
        mesh.free()
    return out


def profile_stress(args):
    """The ordered stress frame at a quarter of its area, for ncu captures of
    the ordered kernels on a case that holds about 1 GB on the device: the
    same densities (4 tiny triangles per pixel, 4,096 large alpha triangles
    over the frame, so about as many blended fragments per pixel) at
    1024x1024, stencil Increment wrapping; --warmup untimed and --steps timed
    frames, their device time printed."""
    import torch
    import softrender as sr
    from softrender import scenes
    sc = scenes.stress_scene(n_tiny=4194304, n_large=4096, size=1024)
    pl, mesh, tex = sr.prepare_scene(sc)
    stream = torch.cuda.Stream()
    pl.set_stream(stream.cuda_stream)

    def frame():
        pl.clear(list(sc.clear_bytes()))
        sr.submit_scene(pl, mesh, tex, sc)
    for _ in range(args.warmup):
        frame()
        if pl.sync() != 0:
            raise RuntimeError("stress frame failed")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        frame()
    e1.record(stream)
    if pl.sync() != 0:
        raise RuntimeError("stress frame failed")
    st = pl.stats()
    print(json.dumps({"profile": "stress_4M_tiny_4096_alpha_1024x1024", "ms_per_frame":
                      round(e0.elapsed_time(e1) / max(1, args.steps), 3), "triangles": int(sc.n_tris),
                      "fragments": int(st["fragments"]), "kernel_launches": int(st["kernel_launches"])}))
    pl.destroy()
    mesh.free()


def profile_batched(args):
    """The batched leg's draws alone, for launch lists and ncu captures: the
    first N instances of the batched workload rendered as one batch with the
    launch configuration the tuner picks for the full workload (primitives of
    up to 16 bins listed, large-primitive threshold 16384 pixels, 8 bin raster
    CTAs per SM)."""
    import softrender as sr
    from softrender import scenes
    inst = scenes.batch_instances()[:args.profile_batched]
    T = []
    for sc in inst:
        fb = sr.Framebuffer(sc.width, sc.height, sc.color_format, sc.depth, sc.stencil)
        pl = sr.Pipeline.from_framebuffer(fb, sc.uniforms)
        m = sr.Mesh(sc.planes, sc.indices)
        T.append((pl, m, sr.draw_for_scene(sc, m), sc))
    b = sr.Batch(use_graphs=False, autotune=False)
    b.set_config(16, 16384, 8)
    arr = b.items([(pl, d, sc.clear_bytes()) for pl, m, d, sc in T])
    for _ in range(args.warmup):
        if b.render_items(arr) != 0 or b.sync() != 0:
            raise RuntimeError("batch failed")
    t0 = time.perf_counter()
    for _ in range(args.steps):
        if b.render_items(arr) != 0:
            raise RuntimeError("batch failed")
    if b.sync() != 0:
        raise RuntimeError("batch failed")
    ms = (time.perf_counter() - t0) / max(1, args.steps) * 1e3
    st = b.stats()
    print(json.dumps({"profile": "batched", "instances": len(inst), "ms_per_batch": round(ms, 3),
                      "triangles": int(sum(sc.n_tris for sc in inst)),
                      "pixels": int(sum(sc.width * sc.height for sc in inst)),
                      "fragments": int(st["fragments"]), "kernel_launches": int(st["kernel_launches"])}))
    b.destroy()
    for pl, m, d, sc in T:
        pl.destroy()
        m.free()


def _timed(fn):
    t0 = time.perf_counter()
    fn()
    return time.perf_counter() - t0


SWEEP_RATES = (2000.0, 5000.0, 10000.0, 20000.0, 40000.0)


def served_wait(srv, ticket):
    """Waits for one served request (30 s at most: a request takes
    milliseconds, so a longer wait means the serving loop stopped)."""
    st = srv.wait(ticket, 30000)
    if st != 0:
        raise RuntimeError("served request %d failed or timed out: status %d" % (ticket, st))


def run_served(rate=2000.0, duration=10.0, sat_duration=1.0, sweep=SWEEP_RATES, served_inflight=2):
    """Poisson request stream against the serving loop and against the plain
    per-request loop (same server code, one request at a time through
    sr_render + sr_sync): p50/p99 latency and throughput at `rate`, the plain
    pipeline's single-request latency, each mode's saturated throughput
    (offered load far above capacity), and a sweep of offered rates giving,
    per mode, the highest rate whose p99 stays within twice the plain
    pipeline's single-request p99.  The sweep's streams are the `rate` stream
    with its arrival times scaled (a Poisson process at rate R, time-scaled
    by R / r, is one at rate r): at least 4,000 requests or half a second of
    arrivals per rate."""
    import collections
    import softrender as sr
    from softrender import scenes
    meshes, reqs = scenes.served_workload(rate=rate, duration=duration)
    dev_meshes = [sr.Mesh(p, i) for p, i in meshes]
    built = [sr.Server.request(sr.draw_for_scene(sc, dev_meshes[mi]), sc.uniforms, sc.width, sc.height,
                               sc.color_format, sc.clear_bytes()) for _, mi, sc in reqs]
    arrivals = np.asarray([a for a, _, _ in reqs])

    def stream(srv, arr=arrivals, burst=False, limit=None):
        """Submits requests at their arrival times (busy-waiting the last
        fraction of a millisecond) and releases finished ones in between, on
        this one thread; latency is stamped by the server from submission to
        completion."""
        n = len(built) if limit is None else min(limit, len(built))
        out = collections.deque()
        t0 = time.perf_counter()
        for k in range(n):
            if not burst:
                while True:
                    left = arr[k] - (time.perf_counter() - t0)
                    if left <= 0:
                        break
                    if out and srv.release(out[0]) == 0:
                        out.popleft()
                    elif left > 0.0006:
                        time.sleep(0.0002)
            st, t = srv.submit(built[k])
            if st != 0:
                raise RuntimeError("submit failed: %d" % st)
            out.append(t)
            while out and srv.release(out[0]) == 0:
                out.popleft()
        offered = n / max(1e-9, time.perf_counter() - t0)
        while out:
            served_wait(srv, out[0])
            srv.release(out.popleft())
        st = srv.stats()
        st["offered_rps"] = offered
        return st

    def warm(srv):
        for k in range(min(2000, len(built))):
            st, t = srv.submit(built[k])
            served_wait(srv, t)
            srv.release(t)
        ts = [srv.submit(built[k])[1] for k in range(min(2000, len(built)))]
        for t in ts:
            served_wait(srv, t)
            srv.release(t)
        srv.reset_stats()

    out = {"workload": "Poisson arrivals at %g req/s for %g s (seed 5); pool of 12 resident sphere meshes, "
                       "1,000-500,000 tris (log-uniform); frames log-uniform 128..1920 x 128..1080; RGBA8 + f32 "
                       "depth; Blinn-Phong; HBM admission budget 64 GB" % (rate, duration),
           "requests": len(built), "served_max_inflight": served_inflight}
    res, sweeps = {}, {}
    for name, plain in (("served", False), ("plain", True)):
        srv = sr.Server(hbm_budget=64 << 30, max_inflight=served_inflight, max_batch=256, plain=plain)
        warm(srv)
        s = stream(srv)
        srv.reset_stats()
        # saturation: the stream's requests submitted back to back (the
        # offered load exceeds either mode's capacity), 20x `rate` x 1 s worth
        sat = stream(srv, burst=True, limit=int(rate * 20 * sat_duration))
        srv.reset_stats()
        res[name] = {"p50_ms": round(s["p50_ms"], 3), "p99_ms": round(s["p99_ms"], 3),
                     "mean_ms": round(s["mean_ms"], 3), "throughput_rps": round(s["throughput_rps"], 1),
                     "mean_batch": round(s["mean_batch"], 2), "peak_bytes": int(s["peak_bytes"]),
                     "saturated_throughput_rps": round(sat["throughput_rps"], 1),
                     "saturated_mean_batch": round(sat["mean_batch"], 2),
                     "saturated_p99_ms": round(sat["p99_ms"], 3)}
        sw = []
        for r in sweep:
            scale = rate / r
            n = int(min(len(built), max(4000, r * 0.5)))
            x = stream(srv, arr=arrivals * scale, limit=n)
            srv.reset_stats()
            sw.append({"rate_rps": r, "requests": n, "offered_rps": round(x["offered_rps"], 1),
                       "p50_ms": round(x["p50_ms"], 3), "p99_ms": round(x["p99_ms"], 3),
                       "throughput_rps": round(x["throughput_rps"], 1), "mean_batch": round(x["mean_batch"], 2)})
        sweeps[name] = sw
        if plain:
            lat = []
            for k in range(min(1000, len(built))):
                t0 = time.perf_counter()
                st, t = srv.submit(built[k])
                served_wait(srv, t)
                lat.append((time.perf_counter() - t0) * 1e3)
                srv.release(t)
            res[name]["single_request_ms"] = {"mean": round(float(np.mean(lat)), 3),
                                              "p50": round(float(np.percentile(lat, 50)), 3),
                                              "p99": round(float(np.percentile(lat, 99)), 3)}
        srv.destroy()
    for m in dev_meshes:
        m.free()
    out.update(res)
    out["saturated_throughput_ratio"] = round(res["served"]["saturated_throughput_rps"] /
                                              max(1e-9, res["plain"]["saturated_throughput_rps"]), 2)
    bound = 2.0 * res["plain"]["single_request_ms"]["p99"]
    best = {}
    for name in ("served", "plain"):
        ok = [x["rate_rps"] for x in sweeps[name] if x["p99_ms"] <= bound]
        best[name] = max(ok) if ok else None
    out["rate_sweep"] = {"bound_p99_ms": round(bound, 3),
                         "bound": "2 x the plain pipeline's single-request p99",
                         "served": sweeps["served"], "plain": sweeps["plain"],
                         "served_max_rate_within_bound": best["served"],
                         "plain_max_rate_within_bound": best["plain"],
                         "rate_ratio_within_bound": (round(best["served"] / best["plain"], 2)
                                                     if best["served"] and best["plain"] else None)}
    out["timing"] = "latency = host clock from submission to the completion callback / sync"
    return out


# -------------------------------------------------------------- reporting
def config_block(world):
    return {"workload": WORKLOAD, "triangles": 1048576, "vertices": 525825, "resolution": "3840x2160",
            "framebuffer": "RGBA8 + f32 depth", "geometry_shader": "clip_primitives",
            "shader": "textured_blinn_phong (1024x1024 RGBA8, bilinear, clamp)", "semantic_tile": "128x128",
            "step": "clear + vertex + clip GS + setup/binning + raster (one frame)",
            "l2": "flushed by a 256 MiB write between timed steps",
            "parallelism": "single GPU" if world == 1 else "replicas x%d (no collective)" % world}


def raster_bytes(scene):
    """Algorithmic bytes of the raster kernel: colour + depth planes read and
    written once, texture read once."""
    return 2 * scene.width * scene.height * 8 + scene.texture.nbytes


TRAFFIC_FILE = os.path.join(ROOT, "profiles", "raster_stage_gridsphere_1M_3840x2160.md")


def traffic_from_profiles():
    """dram__bytes_read.sum + dram__bytes_write.sum of the raster stage's kernels
    for one frame of this workload, from the committed ncu summary (the line
    `raster stage DRAM bytes per launch: N`)."""
    try:
        with open(TRAFFIC_FILE) as f:
            for ln in f:
                if ln.startswith("raster stage DRAM bytes per launch:"):
                    return int(ln.split(":")[1].strip().split()[0].replace(",", ""))
    except (OSError, ValueError):
        return None
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU baseline leg (profiling runs)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiling runs)")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-draws measurement")
    ap.add_argument("--no-frames", action="store_true", help="skip the small and stress frame measurements")
    ap.add_argument("--no-served", action="store_true", help="skip the serving-loop measurement")
    ap.add_argument("--served-inflight", type=int, default=2, help="batches the serving loop keeps on the GPU")
    ap.add_argument("--profile-stress", action="store_true",
                    help="profiling aid: the ordered stress frame at 1024x1024 (--warmup untimed, --steps timed "
                         "frames), its timing only")
    ap.add_argument("--profile-batched", type=int, default=0, metavar="N",
                    help="profiling aid: render the first N batched instances (--warmup untimed and --steps timed "
                         "batches, fixed launch configuration, no tuner, no graphs) and print their timing only")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.profile_batched:
        profile_batched(args)
        return
    if args.profile_stress:
        profile_stress(args)
        return

    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    r = run_ours(args, rank, world, local)
    scene = r["scene"]
    n_tris = scene.n_tris
    peak, peak_kind = measured_peaks()
    ms = r["ms"]
    value = whole_job_rate(n_tris, world, ms)
    frags = r["stats"]["fragments"]
    line = None
    if rank == 0:
        rb = raster_bytes(scene)
        r_ms = r["stage"].get("raster", float("nan"))
        ach = rb / (r_ms * 1e-3) / 1e9
        fb = scene.algorithmic_bytes()
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Mtris/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded displaced grid-sphere, procedural texture)",
            "config": config_block(world),
            "gfrag_per_s": round(frags * world / (ms * 1e-3) / 1e9, 4),
            "fragments_per_frame": int(frags),
            "triangles_generated_per_frame": int(r["stats"]["triangles_generated"]),
            "triangles_rasterised_per_frame": int(r["stats"]["triangles_raster"]),
            "roofline": {"bound": "hbm",
                         "kernel": "opaque raster stage over 32x32 bins: ext_direct_kernel + bin_scan_kernel + "
                                   "bin_scatter_kernel + bin_raster_kernel + "
                                   "bin_resolve_kernel<textured_blinn_phong,RGBA8>",
                         "achieved": round(ach, 2), "peak": peak, "unit": "GB/s",
                         "frac": round(ach / peak, 4), "traffic": traffic_from_profiles(),
                         "algorithmic_bytes": int(rb), "kernel_ms": round(r_ms, 4),
                         "peak_source": peak_kind},
            "frame_roofline": {"algorithmic_bytes": int(fb), "achieved": round(fb / (ms * 1e-3) / 1e9, 2),
                               "unit": "GB/s", "frac": round(fb / (ms * 1e-3) / 1e9 / peak, 4)},
            "stage_ms": {k: round(v, 4) for k, v in r["stage"].items()},
            "e2e": r["e2e"],
            "gpu_launches": int(r["launches"]),
            "clocks": r["clocks"],
        }
        if not args.no_frames:
            line["other_frames"] = run_frames()
        if not args.no_batched:
            line["batched"] = run_batched()
        if not args.no_served:
            line["served"] = run_served(served_inflight=args.served_inflight)
        if not args.no_cpu_baseline:
            frame_s, sample, threads = cpu_frame_estimate(scene, every=1, tiles=510)
            line["cpu_baseline"] = {"value": round(n_tris / frame_s / 1e6, 5), "unit": "Mtris/s",
                                    "cores": threads, "kind": "port", "sample": sample}
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    if line is not None:
        print(json.dumps(line), flush=True)


def run_reference(args, rank, world):
    """The reference's CPU path (restated in oracle/, as the Rust crate cannot
    be built here) on the host cores, same workload and metric."""
    if rank != 0:
        return
    from softrender import scenes
    scene = scenes.grid_sphere_scene()
    n_tris = scene.n_tris
    # warm-up steps: small samples (the CPU path has no state to warm beyond
    # caches); timed steps: whole frames -- every triangle through the vertex
    # stage and the clip GS, every tile rasterised -- measured, not
    # extrapolated (about 12-15 s each on 16 host cores).  Runs of more than
    # 24 steps time 1 in n of the tiles per step instead (n chosen so the run
    # stays near 24 frames' worth) and extrapolate the raster stage linearly.
    for i in range(args.warmup):
        cpu_frame_estimate(scene, every=64, tiles=4, tile_begin=4 * i)
    frames, sample, threads = [], "", os.cpu_count()
    n_tiles = len(scenes_tiles(scene))
    shrink = max(1, -(-args.steps // 24))
    for i in range(args.steps):
        f, sample, threads = cpu_frame_estimate(scene, every=1, tiles=n_tiles // shrink, tile_begin=i)
        frames.append(f)
    frame_s = float(np.mean(frames))
    value = n_tris / frame_s / 1e6
    line = {
        "metric": METRIC, "value": round(value, 5), "unit": "Mtris/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(frame_s * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded displaced grid-sphere, procedural texture)",
        "config": config_block(1), "impl": "reference",
        "cpu_baseline": {"value": round(value, 5), "unit": "Mtris/s", "cores": threads, "kind": "port",
                         "sample": "per step: " + sample},
        "e2e": {"value": round(value, 5), "unit": "Mtris/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
