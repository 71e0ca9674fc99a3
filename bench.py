#!/usr/bin/env python
"""Frame benchmark of the GB300 photon mapper.

One step = one frame of the physically based pipeline on benchmark preset 2
(8 seeded spheres in the box, 1M surface + 1M volume photons, a kd-tree over
each map, 1024x1024 eye rays with specular chains, a k=100 nearest-photon
surface estimate and a volume march of step 0.01 with a k=100 volume
estimate per step): pm_emit + pm_build + pm_render through the C ABI.

Prints one JSON line. `value` is k-NN gathers (surface + volume radiance
estimates) per second of whole-frame device time; photon throughput and the
per-phase times are reported beside it. Two more workloads ride on the same
line: `cache` (the learned radiance cache on the same scene: online frame
and cached render against the k-NN render, with the cached image's error
against the k-NN image) and `batch` (64 independent scenes per frame in
persistent multi-scene launches, captured as a CUDA graph).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank renders its own replica of the scene on its GPU
(replicas only: the path has no exchange step); value = all ranks' gathers
over the slowest rank's time. --impl reference times the CPU restatement of
the same path (the reference has no physically based tracer of its own) on
this host's cores, on a bounded sample of the same frame.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cuda-photon-mapper_gb300")
sys.path.insert(0, PKG)

PRESET_DESC = {
    1: "box with 2 spheres, 100k surface + 100k volume photons, 512x512, k=64, r<=0.1, march 0.01",
    2: "box with 8 seeded spheres, 1M surface + 1M volume photons, kd-tree per map, 1024x1024, "
       "k=100, r<=0.05, volume march step 0.01",
    3: "box with 64 spheres, heterogeneous 128^3 medium, 8M + 8M photons, 1920x1080, k=128, "
       "r<=0.05, march 0.01",
}
L2_FLUSH_BYTES = 256 << 20
CPU_SAMPLE_PIXELS = 2048


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--preset", type=int, default=2)
    ap.add_argument("--seed", type=lambda s: int(s, 0), default=0x5EED0002)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cache", action="store_true", help="skip the radiance-cache A/B")
    ap.add_argument("--cache-warm-frames", type=int, default=384)
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-scene batched frame")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=2)
    ap.add_argument("--no-legacy", action="store_true", help="skip the legacy-mode frames")
    ap.add_argument("--resolution", default=None,
                    help="WxH instead of the preset's image size (small profiling cases)")
    return ap.parse_args()


def preset_config(args):
    """The preset's scene and configuration, with --resolution applied."""
    import photonmap
    scene, cfg = photonmap.preset(args.preset, args.seed)
    if args.resolution:
        w, h = (int(v) for v in args.resolution.lower().split("x"))
        cfg.width, cfg.height = w, h
    return scene, cfg


def dist_info():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_traffic(preset):
    """DRAM bytes per k-NN estimate launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "query_knn_tile_kernel_preset%d_traffic.txt" % preset)
    try:
        for line in open(p):
            if line.startswith("dram_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def reduce_ranks(times, counts, device):
    """Whole-job aggregation over the ranks of the default process group:
    the slowest rank's times (max) and the sum of every rank's counts."""
    import torch
    import torch.distributed as dist
    t = torch.tensor(times, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor(counts, dtype=torch.float64, device=device)
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return t.tolist(), c.tolist()


def cpu_frame_sample(scene, cfg, pixels, seed=1234):
    """The CPU restatement on a bounded sample of one frame: full photon
    emission, neighbour grids over both maps, `pixels` random pixels shaded
    with all host threads. Returns frame-equivalent numbers."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle
    het = oracle.noise_grid(scene, cfg)
    t0 = time.perf_counter()
    maps = oracle.emit(scene, cfg, het)
    t_emit = time.perf_counter() - t0
    npix = cfg.width * cfg.height
    rs = np.random.RandomState(seed)
    pix = np.sort(rs.choice(npix, size=min(pixels, npix), replace=False)).astype(np.uint32)
    _, gathers, secs = oracle.render_timed(scene, cfg, het, maps, pix)
    scale = npix / float(len(pix))
    g_frame = float(gathers.sum()) * scale
    t_frame = t_emit + secs[0] + secs[1] * scale
    return {
        "gathers_per_s": g_frame / t_frame,
        "frame_s": t_frame,
        "emit_s": t_emit,
        "grid_s": float(secs[0]),
        "shade_sample_s": float(secs[1]),
        "sample_pixels": int(len(pix)),
        "paths": int(max(maps.paths)),
        "cores": os.cpu_count(),
    }


def peaks_bf16():
    """(dense bf16 TFLOP/s, source) of the GB300s."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        for key in ("bf16_tflops", "bf16_tflops_burst"):
            if key in d:
                return float(d[key]), "measured " + key
    except (OSError, ValueError):
        pass
    return 1900.0, "fallback"


# Tensor-core FLOPs per query of the cache network as the kernels issue
# them: 4 hidden 64x64 layers and the 64x16 output layer (inference); the
# training kernel adds the activation-gradient GEMMs (same shapes) and the
# weight-gradient GEMMs, issued as two 128x128x128 and one 128x16x128 per
# 128-sample tile (half of the 128x128 products are unused blocks).
CACHE_INFER_FLOPS = 2 * (4 * 64 * 64 + 64 * 16)
CACHE_TRAIN_FLOPS = 2 * CACHE_INFER_FLOPS + 2 * (2 * 128 * 128 + 128 * 16)


def cache_ab(ctx, lib, stream, rad, flush, args, cfg, knn_render_ms, bf16_peak):
    """The learned radiance cache on the same scene and photon maps: after
    `cache_warm_frames` online training frames, each timed step is one online
    frame (2^20 k-NN training samples + their Adam steps, then the cached
    render of every query). Error is the relative RMSE of the cached image
    against the k-NN render of the same frame (the cache's judge)."""
    import numpy as np
    import torch
    sh = stream.cuda_stream
    with torch.cuda.stream(stream):
        ctx.render(rad.data_ptr(), None, sh)
        stream.synchronize()
        knn_img = rad[:, :3].double().cpu().numpy()
        cc = ctx.cache_enable()
        t0 = time.perf_counter()
        ctx.cache_train(args.cache_warm_frames, sh)
        stream.synchronize()
        warm_s = time.perf_counter() - t0
        for _ in range(2):
            ctx.render_cached(rad.data_ptr(), None, 0, sh)
        frame_ms, train_ms, render_ms, targets_ms, values_ms = [], [], [], [], []
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e2 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.cache_train(1, sh)
            e1.record(stream)
            ctx.render_cached(rad.data_ptr(), None, 0, sh)
            e2.record(stream)
            e2.synchronize()
            cs = ctx.cache_stats()
            frame_ms.append(e0.elapsed_time(e2))
            train_ms.append(e0.elapsed_time(e1))
            render_ms.append(e1.elapsed_time(e2))
            targets_ms.append(cs.ms_targets)
            values_ms.append(cs.ms_values)
        cached = rad[:, :3].double().cpu().numpy()
    err = float(np.sqrt(np.mean((cached - knn_img) ** 2)) / np.sqrt(np.mean(knn_img ** 2)))
    nq = cs.queries
    values_s = statistics.mean(values_ms) / 1e3
    infer_tflops = nq * CACHE_INFER_FLOPS / values_s / 1e12
    steps_per_frame = -(-cc.train_samples // cc.batch)
    train_s = statistics.mean(train_ms) / 1e3 - statistics.mean(targets_ms) / 1e3
    train_tflops = cc.train_samples * CACHE_TRAIN_FLOPS / train_s / 1e12
    return {
        "workload": "preset-2 scene and maps; 16-level hash grid (2^19 x 2 fp16 per level), "
                    "4x64 ReLU MLP in bf16 on tcgen05 with fp32 TMEM accumulation; %d k-NN "
                    "training samples per frame, batch %d; inference on every render query"
                    % (cc.train_samples, cc.batch),
        "warm_frames": args.cache_warm_frames, "warm_s": warm_s,
        "train_steps": int(cs.train_steps), "steps_per_frame": steps_per_frame,
        "frame_ms": statistics.mean(frame_ms),
        "train_ms": statistics.mean(train_ms), "targets_ms": statistics.mean(targets_ms),
        "render_ms": statistics.mean(render_ms), "infer_ms": statistics.mean(values_ms),
        "knn_render_ms": knn_render_ms,
        "speedup_online_frame": knn_render_ms / statistics.mean(frame_ms),
        "speedup_render": knn_render_ms / statistics.mean(render_ms),
        "rel_rmse_vs_knn": err,
        "queries_per_frame": int(nq), "queries_per_s": nq / values_s,
        "loss": float(cs.loss),
        "tensor": {"infer_tflops": infer_tflops, "train_tflops": train_tflops,
                   "peak_tflops": bf16_peak[0], "peak_source": bf16_peak[1],
                   "infer_frac": infer_tflops / bf16_peak[0],
                   "train_frac": train_tflops / bf16_peak[0],
                   "flops_per_query_infer": CACHE_INFER_FLOPS,
                   "flops_per_sample_train": CACHE_TRAIN_FLOPS},
        "tc_status": int(cs.tc_status),
        "l2": "flushed before each timed frame",
    }


def batch_frames(ctx, lib, args, device):
    """The batched workload: `batch_scenes` independent scenes (2..32
    spheres, sigma_s in [0, 0.2], 1e5..4e6 photons, 256^2..1024^2 pixels,
    k of 32/64/128) per frame -- one persistent trace launch per pass over
    all scenes, per-scene kd builds on side streams, one persistent render
    launch -- captured as a CUDA graph and replayed. One eager frame is
    timed beside the replays."""
    import torch
    import photonmap
    pairs = [photonmap.batch_scene(i) for i in range(args.batch_scenes)]
    scenes = [p[0] for p in pairs]
    cfgs = [p[1] for p in pairs]
    b = photonmap.Batch(ctx, scenes, cfgs)
    st = torch.cuda.Stream()
    sh = st.cuda_stream

    def timed(fn):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        fn()
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1)

    with torch.cuda.stream(st):
        b.frame(sh)  # warm-up (allocations, first-touch)
        st.synchronize()
        eager_ms = timed(lambda: b.frame(sh))
        b.capture(sh)
        b.launch(sh)
        st.synchronize()
        clocks = ClockSampler(device)
        clocks.start()
        l0 = lib.pm_kernel_launches()
        graph_ms = [timed(lambda: b.launch(sh)) for _ in range(args.batch_steps)]
        launches = lib.pm_kernel_launches() - l0
        clk = clocks.stop()
    gathers = paths = records = 0
    for i in range(b.n):
        s = b.stats(i)
        gathers += s.surface_gathers + s.volume_gathers
        paths += s.paths_traced
        records += s.map_size[0] + s.map_size[1]
    pixels = sum(c.width * c.height for c in cfgs)
    b.close()
    frame_s = statistics.mean(graph_ms) / 1e3
    return {
        "workload": "%d scenes per frame: 2..32 seeded spheres, sigma_s U[0, 0.2], photons "
                    "log-U[1e5, 4e6] split between the maps, 256^2/512^2/1024^2 pixels, k in "
                    "{32, 64, 128}, kd-tree per map, march 0.01" % args.batch_scenes,
        "frame_ms_graph": statistics.mean(graph_ms), "frame_ms_eager": eager_ms,
        "gathers_per_frame": gathers, "photon_paths_per_frame": paths,
        "records_per_frame": records, "pixels_per_frame": pixels,
        "gathers_per_s": gathers / frame_s, "photon_paths_per_s": paths / frame_s,
        "graph_kernels_per_frame": launches // max(1, args.batch_steps),
        "knobs": "defaults (leaf 32, query-list render; per-pixel knobs tile 1, collect 128, "
                 "merge 16); pm_batch_autotune picks per k",
        "clocks": clk,
    }


def legacy_frames(ctx, args, with_cpu):
    """The reference's own frame, through its drop-in exports' explicit-
    context twins: photon emission into the 32^3 voxel grid and a 512x512
    render, media and interpolation on (the slowest of the reference's
    modes), bit-exact with the reference. CPU baseline: the C restatement of
    the same frame on one host thread (the reference's code is serial)."""
    import torch
    import photonmap
    flags = photonmap.PM_LEGACY_INTERPOLATE | photonmap.PM_LEGACY_MEDIA
    img = torch.zeros((512, 512, 4), dtype=torch.uint8, device="cuda")
    st = torch.cuda.Stream()
    sh = st.cuda_stream
    with torch.cuda.stream(st):
        ctx.legacy_init_random(sh)
        for i in range(args.warmup):
            ctx.legacy_emit(0.01 * i, flags, sh)
            ctx.legacy_render(img.data_ptr(), 512, 512, 0.01 * i, flags, stream=sh)
        st.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        n = max(args.steps, 5)
        e0.record(st)
        for i in range(n):
            ctx.legacy_emit(0.01 * i, flags, sh)
            ctx.legacy_render(img.data_ptr(), 512, 512, 0.01 * i, flags, stream=sh)
        e1.record(st)
        e1.synchronize()
    gpu_ms = e0.elapsed_time(e1) / n
    out = {"workload": "reference frame: 10,000 photons into the 32^3 grid, 512x512 render with the "
                       "media march and the bilinear blend ('p' and 'i' keys on)",
           "frame_ms": gpu_ms, "frames": n}
    if with_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        ora = oracle.LegacyOracle()
        ora.init_random()
        t0 = time.perf_counter()
        cpu_n = 2
        for i in range(cpu_n):
            ora.emit(0.01 * i, 1, 1)
            ora.render(512, 512, 0.01 * i, 1, 1)
        cpu_ms = (time.perf_counter() - t0) * 1e3 / cpu_n
        threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
        out["cpu_baseline"] = {"frame_ms": cpu_ms, "cores": threads, "kind": "port",
                               "sample": "%d full frames of the C restatement (bit-exact with the "
                                         "reference's serial semantics): emission on one thread "
                                         "(the deposits' order is the result), the render's "
                                         "independent pixels on %d OpenMP threads" % (cpu_n, threads)}
        out["speedup_vs_cpu"] = cpu_ms / gpu_ms
        # the reference's own CUDA kernels on this GPU, when their module was
        # built (it needs the reference checkout at build time)
        try:
            ref = oracle.ReferenceGPU()
        except OSError as e:
            out["reference_gpu"] = {"unavailable": str(e)}
            return out
        ref.init_random()
        for i in range(args.warmup):
            ref.frame(512, 512, 0.01 * i, 1, 1)
        emit_ms, render_ms = [], []
        for i in range(n):
            a, b = ref.frame(512, 512, 0.01 * i, 1, 1)
            emit_ms.append(a)
            render_ms.append(b)
        ref_ms = statistics.mean(emit_ms) + statistics.mean(render_ms)
        out["reference_gpu"] = {
            "frame_ms": ref_ms, "emit_ms": statistics.mean(emit_ms),
            "render_ms": statistics.mean(render_ms), "frames": n,
            "source": "the reference's photonMappingKernel.cu compiled unmodified for sm_103a "
                      "(cutil shims), launched with its own grid shapes and synchronisations, "
                      "CUDA events; its output is racy and not compared"}
        out["speedup_vs_reference_gpu"] = ref_ms / gpu_ms
    return out


def run_reference(args):
    world, rank, _ = dist_info()
    if rank != 0:
        return 0
    import photonmap
    scene, cfg = preset_config(args)
    threads = os.cpu_count()
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    for _ in range(args.warmup):
        cpu_frame_sample(scene, cfg, CPU_SAMPLE_PIXELS)
    vals, frames = [], []
    for i in range(args.steps):
        r = cpu_frame_sample(scene, cfg, CPU_SAMPLE_PIXELS, seed=1234 + i)
        vals.append(r["gathers_per_s"])
        frames.append(r["frame_s"])
    value = statistics.mean(vals)
    sample = ("per step: full CPU photon emission (%d paths, 1 thread), neighbour grids, "
              "%d random pixels of %dx%d shaded on %d threads; frame time extrapolated to all "
              "pixels" % (r["paths"], CPU_SAMPLE_PIXELS, cfg.width, cfg.height, threads))
    line = {
        "impl": "reference",
        "metric": "gathers/s", "value": value, "unit": "gathers/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.mean(frames), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "preset %d: %s" % (args.preset, PRESET_DESC[args.preset]),
                   "preset": args.preset},
        "cpu_baseline": {"value": value, "unit": "gathers/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "gathers/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_ours(args):
    import torch
    import photonmap

    world, rank, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    lib = photonmap.load()
    scene, cfg = preset_config(args)
    cfg.scene_id = rank  # each replica traces its own photon streams
    ctx = photonmap.Context(local)
    ctx.set_scene(scene, cfg)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    npix = cfg.width * cfg.height
    rad = torch.empty((npix, 4), dtype=torch.float32, device="cuda")
    rgba = torch.empty((npix, 4), dtype=torch.uint8, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def frame():
        ctx.emit(sh)
        ctx.build(sh)
        ctx.render(rad.data_ptr(), rgba.data_ptr(), sh)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.zero_()
            frame()
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        clocks = ClockSampler(local)
        clocks.start()
        l0 = lib.pm_kernel_launches()
        frame_ms, emit_ms, build_ms, render_ms, gather_ms = [], [], [], [], []
        gathers = surf = vol = paths = 0
        for _ in range(args.steps):
            flush.zero_()  # L2 flush between frames, before the start event
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            frame()
            ev1.record(stream)
            ev1.synchronize()
            st = ctx.stats()
            frame_ms.append(ev0.elapsed_time(ev1))
            emit_ms.append(st.ms_emit)
            build_ms.append(st.ms_build)
            render_ms.append(st.ms_render)
            gather_ms.append(st.ms_gather)
            surf += st.surface_gathers
            vol += st.volume_gathers
            paths += st.paths_traced
        launches = lib.pm_kernel_launches() - l0
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        clk = clocks.stop()
        map_sizes = list(st.map_size)
    gathers = surf + vol
    t_total = sum(frame_ms) / 1e3

    # end to end through the C ABI: per step the scene goes in from host
    # memory (pm_update_scene), the frame's radiance and 8-bit image come
    # back to pinned host buffers.
    host_rad = torch.empty((npix, 4), dtype=torch.float32).pin_memory()
    host_rgba = torch.empty((npix, 4), dtype=torch.uint8).pin_memory()
    e2e_g = 0
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for _ in range(args.e2e_steps):
            ctx.update_scene(scene)
            frame()
            host_rad.copy_(rad, non_blocking=True)
            host_rgba.copy_(rgba, non_blocking=True)
            stream.synchronize()
            st = ctx.stats()
            e2e_g += st.surface_gathers + st.volume_gathers
    t_e2e = time.perf_counter() - t0
    barrier()

    if world > 1:
        (t_total, t_e2e), (gathers, e2e_g, paths, launches) = reduce_ranks(
            [t_total, t_e2e], [gathers, e2e_g, paths, launches], "cuda")
        gathers, e2e_g, paths, launches = int(gathers), int(e2e_g), int(paths), int(launches)
    if rank != 0:
        return 0

    peak, peak_kind = load_peaks()
    k = cfg.k
    gather_s = statistics.mean(gather_ms) / 1e3
    q_per_frame = (surf + vol) / args.steps
    # per query: k records of 32 B (position + power), the 32 B query record,
    # its 4 B index in spatial order and the 16 B value written
    alg_bytes = q_per_frame * (32.0 * k + 52.0)
    achieved = alg_bytes / gather_s / 1e9
    traffic = load_traffic(args.preset)
    line = {
        "metric": "gathers/s",
        "value": gathers / t_total,
        "unit": "gathers/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t_total / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {
            "workload": "preset %d: %s" % (args.preset, PRESET_DESC[args.preset]),
            "preset": args.preset, "seed": args.seed, "resolution": [cfg.width, cfg.height],
            "photons": [cfg.surface_photons, cfg.volume_photons], "k": k,
            "radius": cfg.radius, "march_step": cfg.march_step,
            "l2": "flushed between timed frames (256 MiB write, outside the timed events)",
            "parallelism": "replicas x%d" % world,
        },
        "phases": {
            "emit_ms": statistics.mean(emit_ms), "build_ms": statistics.mean(build_ms),
            "render_ms": statistics.mean(render_ms), "gather_ms": statistics.mean(gather_ms),
            "frame_ms": statistics.mean(frame_ms),
            "paths_per_frame": paths / args.steps / world,
            "photons_per_s": paths / (sum(emit_ms) / 1e3) / world,
            "records_per_s": sum(map_sizes) * args.steps / (sum(emit_ms) / 1e3),
            "map_sizes": map_sizes,
            "surface_gathers_per_frame": surf / args.steps,
            "volume_gathers_per_frame": vol / args.steps,
        },
        "e2e": {"value": e2e_g / t_e2e, "unit": "gathers/s",
                "h2d_bytes_per_step": int(photonmap.ctypes.sizeof(photonmap.Scene)),
                "d2h_bytes_per_step": int(npix * (16 + 4)),
                "steps": args.e2e_steps},
        "roofline": {"bound": "hbm", "kernel": "query_knn_tile_kernel", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind,
                     "traffic": traffic,
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "formula": "gathers x (32 B x k + 52 B), over the CUDA-event time of the "
                                "k-NN estimate pass (anchor, shared-candidate and deferred "
                                "launches; events on the render stream)"},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if not args.no_cache:
        line["cache"] = cache_ab(ctx, lib, stream, rad, flush, args, cfg,
                                 statistics.mean(render_ms), peaks_bf16())
    if not args.no_batch:
        line["batch"] = batch_frames(ctx, lib, args, local)
    if not args.no_legacy:
        line["legacy"] = legacy_frames(ctx, args, with_cpu=(world == 1 and not args.no_cpu_baseline))
    if world == 1 and not args.no_cpu_baseline:
        r = cpu_frame_sample(scene, cfg, CPU_SAMPLE_PIXELS)
        line["cpu_baseline"] = {
            "value": r["gathers_per_s"], "unit": "gathers/s", "cores": r["cores"], "kind": "port",
            "sample": "full CPU photon emission (%d paths, 1 thread) + neighbour grids + %d "
                      "random pixels shaded on %d threads, frame time extrapolated to %dx%d"
                      % (r["paths"], r["sample_pixels"], r["cores"], cfg.width, cfg.height),
            "frame_s": r["frame_s"],
        }
    print(json.dumps(line))
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
