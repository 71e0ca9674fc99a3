#!/usr/bin/env python
"""Frame benchmark of the GB300 photon mapper.

One step = one frame of the physically based pipeline on benchmark preset 3,
the 16M-photon volumetric scene (64 seeded spheres in the box, a
heterogeneous 128^3 value-noise medium, 8M surface + 8M volume photons with
up to 8 bounces, a kd-tree over each map, 1920x1080 eye rays with specular
chains, a k=128 nearest-photon surface estimate and a volume march of step
0.01 with a k=128 volume estimate per step): pm_emit + pm_build + pm_render
through the C ABI.

Prints one JSON line. `value` is k-NN gathers (surface + volume radiance
estimates) per second of whole-frame device time; photon throughput and the
per-phase times are reported beside it, with the relative RMSE of sampled
pixels against the FP64 oracle render (`fp64`) and their bit-equality with
the FP32 oracle (`parity_sample`). `roofline` is the k-NN estimate pass
against the measured HBM bandwidth (with the full-size DRAM traffic per
launch from the committed ncu summary) and `frame_roofline` the whole frame
by the frame byte formula. More workloads ride on the same line:
`preset2` (the 2M-photon scene, same metric), `cache` (the learned radiance
cache on the preset-2 scene: online frame and cached render against the k-NN
render, errors against the k-NN and FP64 renders), `batch` (64 independent
scenes per frame captured as a CUDA graph; `batch.cached`: the same batch
with a radiance cache per scene trained and queried inside the replayed
frame, its images against the k-NN images) and `legacy` (the reference's own
voxel frame).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank renders its own replica of the scene on its GPU
(replicas only: the path has no exchange step); value = all ranks' gathers
over the slowest rank's time. --impl reference times the CPU restatement of
the same path in oracle/ (the reference has no physically based tracer of
its own) on this host's cores, without loading the product library: all
threads, emission of a sample of the frame's photon paths and the gathers of
a sample of its pixels through a kd-tree per map, per step.
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
    ap.add_argument("--preset", type=int, default=3)
    ap.add_argument("--seed", type=lambda s: int(s, 0), default=None,
                    help="scene seed (default 0x5EED0000 + preset)")
    ap.add_argument("--secondary-preset", type=int, default=2,
                    help="second scene timed on the same line (0: none)")
    ap.add_argument("--fp64-pixels", type=int, default=8192,
                    help="pixels sampled for the FP64 and FP32 oracle checks (0: none)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cache", action="store_true", help="skip the radiance-cache A/B")
    ap.add_argument("--cache-warm-frames", type=int, default=384)
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-scene batched frame")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=2)
    ap.add_argument("--batch-cache-warm", type=int, default=96,
                    help="training frames of the per-scene radiance caches before the timed batch frames "
                         "(0: skip the cached batch frames)")
    ap.add_argument("--batch-cache-samples", type=int, default=1 << 20,
                    help="k-NN training samples per scene and frame of the per-scene caches")
    ap.add_argument("--no-legacy", action="store_true", help="skip the legacy-mode frames")
    ap.add_argument("--resolution", default=None,
                    help="WxH instead of the preset's image size (small profiling cases)")
    return ap.parse_args()


def preset_config(args, preset=None, seed=None, product=True):
    """The preset's scene and configuration, with --resolution applied: from
    the product library (pm_preset) or, for the CPU-only reference arm, from
    the oracle's byte-equal restatement."""
    preset = args.preset if preset is None else preset
    if seed is None:
        seed = args.seed if (args.seed is not None and preset == args.preset) else 0x5EED0000 + preset
    if product:
        import photonmap
        scene, cfg = photonmap.preset(preset, seed)
    else:
        import oracle
        scene, cfg = oracle.preset(preset, seed)
    if args.resolution:
        w, h = (int(v) for v in args.resolution.lower().split("x"))
        cfg.width, cfg.height = w, h
    return scene, cfg


def workload_config(args, preset, cfg, world=1):
    """The `config` object both arms print for the same workload."""
    return {
        "workload": "preset %d: %s" % (preset, PRESET_DESC[preset]),
        "preset": preset, "seed": int(cfg.seed), "resolution": [cfg.width, cfg.height],
        "photons": [int(cfg.surface_photons), int(cfg.volume_photons)], "k": int(cfg.k),
        "radius": float(cfg.radius), "march_step": float(cfg.march_step),
        "max_bounces": int(cfg.max_bounces),
        "l2": "flushed between timed GPU frames (256 MiB write, outside the timed events)",
        "parallelism": "replicas x%d" % world,
    }


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


def load_traffic(preset, args):
    """DRAM bytes per k-NN estimate launch from the committed ncu summary of
    the preset's full-size frame, if any (none at another resolution)."""
    if args.resolution:
        return None
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


class CpuFrame:
    """The CPU restatement of one frame (oracle/, all host threads), timed on
    bounded samples: a step traces 1/path_div of the frame's photon paths and
    shades `pixels` random pixels through a kd-tree per map (built once);
    the frame time is extrapolated from them plus the measured tree build.
    maps: the frame's photon maps (None: the full CPU emission, timed)."""

    def __init__(self, scene, cfg, het, maps=None, paths_total=None, pixels=CPU_SAMPLE_PIXELS,
                 path_div=64):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        self.oracle = oracle
        self.scene, self.cfg, self.het = scene, cfg, het
        self.emit_full_s = None
        if maps is None:
            t0 = time.perf_counter()
            maps = oracle.emit(scene, cfg, het)
            self.emit_full_s = time.perf_counter() - t0
            paths_total = int(max(maps.paths))
        self.maps = maps
        self.paths_total = int(paths_total)
        self.renderer = oracle.Renderer(scene, cfg, het, maps)
        self.build_s = self.renderer.build_s
        self.npix = cfg.width * cfg.height
        self.pixels = min(pixels, self.npix)
        self.path_count = max(1, -(-self.paths_total // path_div))
        self.threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))

    def step(self, i):
        import numpy as np
        first = (i * self.path_count) % max(1, self.paths_total - self.path_count + 1)
        t0 = time.perf_counter()
        self.oracle.trace_sample(self.scene, self.cfg, self.het, first, self.path_count)
        t1 = time.perf_counter()
        rs = np.random.RandomState(1234 + i)
        pix = np.sort(rs.choice(self.npix, size=self.pixels, replace=False)).astype(np.uint32)
        _, gathers = self.renderer.pixels(pix)
        t2 = time.perf_counter()
        scale = self.npix / float(self.pixels)
        frame_s = ((t1 - t0) * self.paths_total / self.path_count + self.build_s
                   + (t2 - t1) * scale)
        return {"wall_s": t2 - t0, "frame_s": frame_s,
                "gathers_frame": float(gathers.sum()) * scale}

    def sample_text(self):
        src = ("maps from the full CPU emission (%.1f s, done once)" % self.emit_full_s
               if self.emit_full_s is not None else "the GPU frame's maps (bit-equal to the CPU "
               "emission's), copied to the host")
        return ("per step, on %d threads: %d of the frame's %d photon paths traced (1/%d) and "
                "%d random pixels of %dx%d shaded through a kd-tree per map (built once in %.2f "
                "s); %s; frame time extrapolated from the samples plus the tree build"
                % (self.threads, self.path_count, self.paths_total,
                   -(-self.paths_total // self.path_count), self.pixels, self.cfg.width,
                   self.cfg.height, self.build_s, src))

    def close(self):
        self.renderer.close()


def rel_rmse(a, b):
    import numpy as np
    a = np.asarray(a, np.float64)[:, :3]
    b = np.asarray(b, np.float64)[:, :3]
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-300))


def oracle_checks(scene, cfg, rad, npixels, fp32_maps=None, seed=77):
    """Sampled-pixel checks of a GPU frame's radiance `rad` (host [npix, 4]):
    relative RMSE against the FP64 oracle render (own FP64 emission) and,
    when the frame's maps are given, bit-equality with the FP32 oracle render
    over them. Returns (dict, pixels, fp64 radiance of those pixels)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    het = oracle.noise_grid(scene, cfg)
    npix = cfg.width * cfg.height
    rs = np.random.RandomState(seed)
    pix = np.sort(rs.choice(npix, size=min(npixels, npix), replace=False)).astype(np.uint32)
    t0 = time.perf_counter()
    m64 = oracle.emit(scene, cfg, het, double=True)
    r64 = oracle.render(scene, cfg, het, m64, pixels=pix, double=True)
    out = {"pixels": int(len(pix)), "rel_rmse": rel_rmse(rad[pix], r64),
           "seconds": time.perf_counter() - t0,
           "what": "GPU FP32 frame vs the FP64 oracle (own FP64 emission and render) on random "
                   "pixels"}
    parity = None
    if fp32_maps is not None:
        r32 = oracle.render(scene, cfg, het, fp32_maps, pixels=pix)
        same = np.all(r32.view(np.uint32) == rad[pix].view(np.uint32), axis=1)
        parity = {"pixels": int(len(pix)), "bit_equal_fraction": float(same.mean()),
                  "what": "GPU radiance vs the FP32 oracle render over the GPU's maps"}
    return out, parity, pix, r64


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


def cache_ab(ctx, lib, stream, rad, flush, args, cfg, knn_render_ms, bf16_peak, fp64=None):
    """The learned radiance cache on the same scene and photon maps: after
    `cache_warm_frames` online training frames, each timed step is one online
    frame (2^20 k-NN training samples + their Adam steps, then the cached
    render of every query). Error is the relative RMSE of the cached image
    against the k-NN render of the same frame (the yardstick the cache is trained toward)."""
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
    fp64_err = None
    if fp64 is not None:
        pix, r64 = fp64
        fp64_err = {"cached": rel_rmse(cached[pix], r64), "knn": rel_rmse(knn_img[pix], r64),
                    "pixels": int(len(pix))}
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
        "rel_rmse_vs_fp64": fp64_err,
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
    all scenes, the record extents, tree levels and tree finishes of all
    maps in shared launches, every scene's query list built by shared
    launches into one arena, one persistent estimate launch per k-list
    width and one composite launch -- captured as a CUDA graph and
    replayed. One eager frame is timed beside the replays."""
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
    cached = None
    if args.batch_cache_warm > 0:
        cached = batch_cache_frames(b, cfgs, st, timed, args)
    b.close()
    frame_s = statistics.mean(graph_ms) / 1e3
    return {
        "cached": cached,
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


def batch_cache_frames(b, cfgs, st, timed, args):
    """The same batch with a BF16 radiance cache per scene: each frame trains
    every scene's network on `batch_cache_samples` k-NN targets of its own
    query list (Adam steps of 2^17 samples) and renders every query through
    it, the whole frame one replayed CUDA graph. Error: each scene's cached
    image against its k-NN image (the same maps and camera) after
    `batch_cache_warm` training frames."""
    import numpy as np
    import photonmap
    sh = st.cuda_stream
    knn = [b.read(i)[0] for i in range(b.n)]
    cc = b.cache_enable(train_samples=args.batch_cache_samples, batch=min(1 << 17, args.batch_cache_samples))
    b.capture(sh)
    t0 = time.perf_counter()
    for _ in range(args.batch_cache_warm):
        b.launch(sh)
    st.synchronize()
    warm_s = time.perf_counter() - t0
    frame_ms = [timed(lambda: b.launch(sh)) for _ in range(args.batch_steps)]
    errs = []
    for i in range(b.n):
        img = b.read(i)[0][:, :3].astype(np.float64)
        ref = knn[i][:, :3].astype(np.float64)
        errs.append(float(np.sqrt(np.mean((img - ref) ** 2)) / max(np.sqrt(np.mean(ref ** 2)), 1e-30)))
    b.cache_disable()
    return {
        "workload": "the batch above with one radiance cache per scene (16-level hash grid, 2^%d entries "
                    "per level, 4x64 MLP in bf16 on tcgen05): %d k-NN training samples per scene and "
                    "frame, Adam steps of %d, inference on every query; training, inference and "
                    "composite inside the replayed frame" % (cc.log2_table, cc.train_samples, cc.batch),
        "warm_frames": args.batch_cache_warm, "warm_s": warm_s,
        "frame_ms_graph": statistics.mean(frame_ms),
        "rel_rmse_vs_knn": {"median": float(np.median(errs)), "mean": float(np.mean(errs)),
                            "max": float(np.max(errs)), "scenes": len(errs)},
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
    """The CPU restatement of the path (oracle/, all host threads) on the
    same workload and config; never loads the product library."""
    world, rank, _ = dist_info()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))  # before the oracle's OpenMP starts
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    scene, cfg = preset_config(args, product=False)
    het = oracle.noise_grid(scene, cfg)
    t0 = time.perf_counter()
    cpu = CpuFrame(scene, cfg, het)
    setup_s = time.perf_counter() - t0
    for i in range(args.warmup):
        cpu.step(i)
    res = [cpu.step(args.warmup + i) for i in range(args.steps)]
    frame_s = statistics.mean(r["frame_s"] for r in res)
    gathers = statistics.mean(r["gathers_frame"] for r in res)
    value = gathers / frame_s
    cores = int(os.environ.get("OMP_NUM_THREADS", threads))
    line = {
        "impl": "reference",
        "metric": "gathers/s", "value": value, "unit": "gathers/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.mean(r["wall_s"] for r in res),
        "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, args.preset, cfg, world),
        "frame_ms_extrapolated": 1e3 * frame_s,
        "setup_s": setup_s,
        "cpu_baseline": {"value": value, "unit": "gathers/s", "cores": cores, "kind": "port",
                         "sample": cpu.sample_text()},
        "e2e": {"value": value, "unit": "gathers/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    cpu.close()
    print(json.dumps(line))
    return 0


def measure_frames(ctx, lib, scene, cfg, stream, flush, steps, warmup, barrier, device):
    """Times `steps` frames (pm_emit + pm_build + pm_render) after `warmup`,
    with CUDA events on the library's stream and an L2 flush before each."""
    import torch
    ctx.set_scene(scene, cfg)
    sh = stream.cuda_stream
    npix = cfg.width * cfg.height
    rad = torch.empty((npix, 4), dtype=torch.float32, device="cuda")
    rgba = torch.empty((npix, 4), dtype=torch.uint8, device="cuda")

    def frame():
        ctx.emit(sh)
        ctx.build(sh)
        ctx.render(rad.data_ptr(), rgba.data_ptr(), sh)

    r = {"frame_ms": [], "emit_ms": [], "build_ms": [], "render_ms": [], "gather_ms": [],
         "surf": 0, "vol": 0, "paths": 0, "rad": rad, "rgba": rgba, "frame": frame}
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            flush.zero_()
            frame()
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        clocks = ClockSampler(device)
        clocks.start()
        l0 = lib.pm_kernel_launches()
        for _ in range(steps):
            flush.zero_()  # L2 flush between frames, before the start event
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            frame()
            ev1.record(stream)
            ev1.synchronize()
            st = ctx.stats()
            r["frame_ms"].append(ev0.elapsed_time(ev1))
            r["emit_ms"].append(st.ms_emit)
            r["build_ms"].append(st.ms_build)
            r["render_ms"].append(st.ms_render)
            r["gather_ms"].append(st.ms_gather)
            r["surf"] += st.surface_gathers
            r["vol"] += st.volume_gathers
            r["paths"] += st.paths_traced
        r["launches"] = lib.pm_kernel_launches() - l0
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        r["clocks"] = clocks.stop()
        r["map_sizes"] = list(st.map_size)
    return r


def phases_of(r, steps, world=1):
    return {
        "emit_ms": statistics.mean(r["emit_ms"]), "build_ms": statistics.mean(r["build_ms"]),
        "render_ms": statistics.mean(r["render_ms"]), "gather_ms": statistics.mean(r["gather_ms"]),
        "frame_ms": statistics.mean(r["frame_ms"]),
        "paths_per_frame": r["paths"] / steps / world,
        "photons_per_s": r["paths"] / (sum(r["emit_ms"]) / 1e3) / world,
        "records_per_s": sum(r["map_sizes"]) * steps / (sum(r["emit_ms"]) / 1e3),
        "map_sizes": r["map_sizes"],
        "surface_gathers_per_frame": r["surf"] / steps,
        "volume_gathers_per_frame": r["vol"] / steps,
    }


def estimate_roofline(r, steps, k, peak, peak_kind, traffic):
    """The k-NN estimate pass against HBM: per query the k records' 32 B
    (position + power), the 32 B query record, its 4 B index in spatial order
    and the 16 B value written, over the pass's CUDA-event time."""
    gather_s = statistics.mean(r["gather_ms"]) / 1e3
    q_per_frame = (r["surf"] + r["vol"]) / steps
    alg_bytes = q_per_frame * (32.0 * k + 52.0)
    achieved = alg_bytes / gather_s / 1e9
    return {"bound": "hbm", "kernel": "query_knn_tile_kernel", "achieved": achieved,
            "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
            "traffic": traffic, "algorithmic_bytes_per_launch": alg_bytes,
            "formula": "gathers x (32 B x k + 52 B), over the CUDA-event time of the k-NN "
                       "estimate pass (anchor, shared-candidate and deferred launches; events "
                       "on the render stream)"}


def frame_roofline(r, steps, k, peak, peak_kind):
    """The whole frame against HBM by the frame formula: 32 B per stored
    record (emission), 116 B per record of each map's kd build (positions
    read, keys and indices written, the permutation's key and index read
    and written, the 32 B records read and written) and 32 B x k + 16 B per
    k-NN gather (the k records and the value written), over the frame's
    CUDA-event time."""
    records = float(sum(r["map_sizes"]))
    q_per_frame = (r["surf"] + r["vol"]) / steps
    alg_bytes = 32.0 * records + 116.0 * records + q_per_frame * (32.0 * k + 16.0)
    achieved = alg_bytes / (statistics.mean(r["frame_ms"]) / 1e3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": peak_kind, "algorithmic_bytes_per_frame": alg_bytes,
            "formula": "32 B x stored records + 116 B x records (kd build per map) + gathers x "
                       "(32 B x k + 16 B), over the frame's CUDA-event time"}


def host_maps(ctx):
    """The context's two photon maps copied to the host as oracle maps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    spos, spow = ctx.photons_soa(0)
    vpos, vpow = ctx.photons_soa(1)
    return oracle.maps_from_arrays(spos, spow, vpos, vpow)


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
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    head = measure_frames(ctx, lib, scene, cfg, stream, flush, args.steps, args.warmup, barrier,
                          local)
    frame = head["frame"]
    rad, rgba = head["rad"], head["rgba"]
    npix = cfg.width * cfg.height
    gathers = head["surf"] + head["vol"]
    t_total = sum(head["frame_ms"]) / 1e3
    paths, launches = head["paths"], head["launches"]

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
        "config": workload_config(args, args.preset, cfg, world),
        "phases": phases_of(head, args.steps, world),
        "e2e": {"value": e2e_g / t_e2e, "unit": "gathers/s",
                "h2d_bytes_per_step": int(photonmap.ctypes.sizeof(photonmap.Scene)),
                "d2h_bytes_per_step": int(npix * (16 + 4)),
                "steps": args.e2e_steps},
        "roofline": estimate_roofline(head, args.steps, cfg.k, peak, peak_kind,
                                      load_traffic(args.preset, args)),
        "frame_roofline": frame_roofline(head, args.steps, cfg.k, peak, peak_kind),
        "gpu_launches": int(launches),
        "clocks": head["clocks"],
    }
    single = world == 1
    if single and (args.fp64_pixels or not args.no_cpu_baseline):
        gpu_maps = host_maps(ctx)
        rad_host = host_rad.numpy().copy()
        if args.fp64_pixels:
            line["fp64"], line["parity_sample"], _, _ = oracle_checks(
                scene, cfg, rad_host, args.fp64_pixels, gpu_maps)
        if not args.no_cpu_baseline:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle
            cpu = CpuFrame(scene, cfg, oracle.noise_grid(scene, cfg), maps=gpu_maps,
                           paths_total=head["paths"] / args.steps)
            res = [cpu.step(i) for i in range(2)]
            fs = statistics.mean(r["frame_s"] for r in res)
            line["cpu_baseline"] = {
                "value": statistics.mean(r["gathers_frame"] for r in res) / fs,
                "unit": "gathers/s", "cores": cpu.threads, "kind": "port",
                "sample": cpu.sample_text(), "frame_s_extrapolated": fs,
                "wall_s_per_step": statistics.mean(r["wall_s"] for r in res)}
            cpu.close()
        del gpu_maps
    if single and args.secondary_preset:
        p2 = args.secondary_preset
        sc2, cf2 = preset_config(args, p2)
        steps2 = max(3, args.steps // 4)
        sec = measure_frames(ctx, lib, sc2, cf2, stream, flush, steps2, min(args.warmup, 3),
                             barrier, local)
        g2 = sec["surf"] + sec["vol"]
        line["preset%d" % p2] = {
            "config": workload_config(args, p2, cf2),
            "value": g2 / (sum(sec["frame_ms"]) / 1e3), "unit": "gathers/s",
            "ms_per_step": statistics.mean(sec["frame_ms"]), "steps": steps2,
            "phases": phases_of(sec, steps2),
            "roofline": estimate_roofline(sec, steps2, cf2.k, peak, peak_kind, load_traffic(p2, args)),
            "frame_roofline": frame_roofline(sec, steps2, cf2.k, peak, peak_kind),
            "clocks": sec["clocks"],
        }
        fp64_2 = None
        if args.fp64_pixels:
            rad2 = sec["rad"].cpu().numpy()
            chk, par, pix2, r64_2 = oracle_checks(sc2, cf2, rad2, args.fp64_pixels, host_maps(ctx))
            line["preset%d" % p2]["fp64"] = chk
            line["preset%d" % p2]["parity_sample"] = par
            fp64_2 = (pix2, r64_2)
        if not args.no_cache:
            line["cache"] = cache_ab(ctx, lib, stream, sec["rad"], flush, args, cf2,
                                     statistics.mean(sec["render_ms"]), peaks_bf16(), fp64_2)
    if single and not args.no_batch:
        line["batch"] = batch_frames(ctx, lib, args, local)
    if single and not args.no_legacy:
        line["legacy"] = legacy_frames(ctx, args, with_cpu=not args.no_cpu_baseline)
    print(json.dumps(line))
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
