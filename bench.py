"""Frame benchmark: 1M-triangle 1920x1080 soup (16x16 bins, depth test on,
seeded), one frame per step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value   triangles/s of the whole job with the scene resident in HBM (CUDA
        events around each frame, on the renderer's stream; L2 flushed by a
        256 MB write before every timed frame, outside the events).
e2e     the same metric through the C ABI with host buffers: each step
        copies the vertices from pinned host memory, renders, and reads the
        framebuffer back into pinned host memory; three renderers on three
        streams, so each step's copies run under the other steps' frames
        (wall clock over all steps, an L2 flush queued with every step).
roofline  the raster kernel (the dominant kernel): algorithmic bytes
        (4 B per bin entry read + 8 B per pixel written) / its CUDA-event
        time against the measured HBM copy bandwidth.
cpu_baseline  the reference's own CPU renderer (ERenderer.cpp, built from
        the staged reference sources, single-threaded as written) on one
        full frame of the same soup; the oracle port (CPU restatement of the
        reference's GPU pipeline) on all host cores where it does not build.

config  also carries, measured in the same run: predicted-capacity binning
        of the same frame (the committed model, and the plain sampled-count
        rule) with its frame and binning ratios against exact binning; the
        lit 4K icosphere-7 with 8x8 and 16x16 bins ("icosphere7_4k"); the
        256-scene batch with the autotuner's pick over bins {8, 16, 32} x
        queue chunks {32, 64, 128} x raster variants, wider chunks as an
        extra, and N concurrent reference ERenderers on the host cores as
        its CPU baseline ("batch_256").  --soup-only skips the last two.

--impl reference times that CPU renderer on the same workload: one full
frame of the 1M soup per step (about 3 s on one core).
Under torchrun each rank renders its own seeded frame (independent
replicas, weak scaling); rank 0 prints the max-over-ranks line.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "custom-gpgpu-rasterizer_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

N_TRI = 1_000_000
WIDTH, HEIGHT, BIN = 1920, 1080, 16
CHUNK = 4096
E2E_DEPTH = 3   # end-to-end leg: renderers (and streams) in flight
METRIC = "triangles/s (1M-tri 1080p soup frame, exact two-pass binning)"
UNIT = "triangles/s"
WORKLOAD = "soup-1M-1080p"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(values, dist, device):
    """Element-wise maximum of `values` over the ranks (a replica job takes
    as long as its slowest rank); unchanged with one rank."""
    if dist is None:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def make_scene(seed: int):
    import scenes
    return scenes.soup_scene(N_TRI, WIDTH, HEIGHT, BIN, seed=seed)


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per raster launch from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "raster_kernel_soup1m_1080p.md")
    try:
        m = re.search(r"dram_bytes_per_launch:\s*([0-9.e+]+)", open(path).read())
        return float(m.group(1)) if m else None
    except OSError:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms.

    A timed region of a few milliseconds can fall between two samples, so
    after the timed region `hold(step)` keeps running the same step (not
    timed) until at least `min_samples` samples were taken since the timed
    region began.  The report says how many samples fell inside the timed
    region itself and how many frames the hold added."""
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    REASONS = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.t0 = self.t1 = None
        self.hold_frames = 0
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        deadline = time.time() + 5.0
        while self.p is not None and not self._rows() and time.time() < deadline:
            time.sleep(0.05)

    def _rows(self):
        out = []
        for line in open(self.f.name).read().strip().splitlines():
            r = [x.strip() for x in line.split(",")]
            if len(r) < len(self.FIELDS.split(",")):
                continue
            try:
                ts = datetime.datetime.strptime(r[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                out.append((ts, float(r[2]), float(r[3]),
                            [n for k, n in enumerate(self.REASONS) if r[6 + k].lower().startswith("active")]))
            except ValueError:
                continue
        return out

    def begin(self):
        self.t0 = time.time()

    def end(self):
        self.t1 = time.time()

    def hold(self, step, min_samples: int = 3, limit_s: float = 5.0):
        """Runs `step()` until `min_samples` samples are newer than begin()."""
        if self.p is None or self.t0 is None:
            return
        deadline = time.time() + limit_s
        while time.time() < deadline:
            if sum(1 for r in self._rows() if r[0] >= self.t0 - 1e-3) >= min_samples:   # ms timestamps
                break
            step()
            self.hold_frames += 1

    def stop(self):
        if self.p is None:
            return None
        t_stop = time.time()
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = self._rows()
        os.unlink(self.f.name)
        t0 = self.t0 - 1e-3 if self.t0 is not None else 0.0   # timestamps are whole milliseconds
        t1 = self.t1 if self.t1 is not None else t_stop
        under_load = [r for r in rows if t0 <= r[0] <= t_stop]
        if not under_load:
            return None
        return {"sm_mhz": statistics.median(r[1] for r in under_load),
                "sm_max_mhz": max(r[2] for r in under_load),
                "reasons": sorted({n for r in under_load for n in r[3]}),
                "samples": len(under_load),
                "samples_in_timed_region": sum(1 for r in under_load if r[0] <= t1),
                "hold_frames": self.hold_frames}


def cpu_baseline(scene, threads: int):
    from oracle import oracle
    oracle.lib()
    t0 = time.perf_counter()
    out = oracle.render(scene, oracle.RASTER_REFERENCE, num_threads=threads, want_bins=False)
    dt = time.perf_counter() - t0
    return dt, out


def reference_cpu(scene, frames: int, stride: int):
    """The reference's own CPU renderer (Elite::Renderer, ERenderer.cpp,
    single-threaded as written) on `scene`, built from the staged reference
    sources by oracle/ref/build_ref.py: mean wall time per frame after one
    warm-up frame, rendering every stride-th triangle.  None where the
    staged sources or a host compiler are missing."""
    try:
        from oracle.ref import build_ref, ref_io
        exe = build_ref.build_erenderer()
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "scene.bin")
            ref_io.write_scene(scene, path)
            out = subprocess.run([exe, path, str(frames), str(stride)], capture_output=True, text=True, check=True)
        return json.loads(out.stdout.strip().splitlines()[-1])
    except Exception as e:  # noqa: BLE001 -- reported, and the oracle port is timed instead
        print(f"reference CPU renderer unavailable ({type(e).__name__}: {e}); timing the oracle port",
              file=sys.stderr)
        return None


REF_STRIDE = 1   # the reference arm renders every triangle of the soup each step


def run_reference(args, rank, world):
    """The reference's CPU implementation of the path: its ERenderer
    (single-threaded as written), each step one full frame of the same soup;
    the oracle port on all host cores where the reference does not build
    here."""
    if rank != 0:
        return
    scene = make_scene(0)
    r = reference_cpu(scene, args.steps, REF_STRIDE)
    if r is not None:
        t = r["ms_per_frame"] / 1e3
        tris = r["triangles"]
        cores, kind = 1, "reference"
        sample = (f"one full frame of the 1M soup ({tris} triangles) at 1920x1080 per step after a warm-up "
                  f"frame, the reference's ERenderer (single-threaded as written)")
    else:
        threads = os.cpu_count() or 1
        times = []
        for i in range(args.warmup + args.steps):
            dt, _ = cpu_baseline(scene, threads)
            if i >= args.warmup:
                times.append(dt)
        t = sum(times) / len(times)
        tris, cores, kind = N_TRI, threads, "port"
        sample = "one full frame per step: setup, binning, raster and shading of the 1M soup (oracle port)"
    value = tris / t
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "triangles": int(tris), "resolution": [WIDTH, HEIGHT], "bins": [BIN, BIN],
                       "frames_per_s": 1.0 / t},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def predicted_binning(r, scene, args, stream, flush, sampled=False):
    """The same device-resident frame with learned-capacity binning (the
    committed model; with `sampled`, the plain sampled-count rule instead):
    time per frame, binning time, frame overflow rate and over-allocation of
    the predicted capacities, on the same renderer as exact binning."""
    import torch
    import gbr
    import predictor

    if not os.path.exists(predictor.WEIGHTS):
        return None
    sptr = stream.cuda_stream
    predictor.install(r, sampled=sampled)
    out = {"ms_per_step": [], "ms_binning": [], "overflow": 0, "over_allocation": []}
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            r.render_scene(scene, sptr)
            r.stats(sptr)
        for total_only in (False, True):
            r.set_timing(True, total_only=total_only)
            for _ in range(args.steps):
                flush.zero_()
                r.render_scene(scene, sptr)
                st = r.stats(sptr)
                if total_only:
                    out["ms_per_step"].append(st["ms_total"])
                else:
                    out["ms_binning"].append(st["ms_setup"] + st["ms_bin"])
                out["overflow"] += int(st["predicted_overflow"])
                out["over_allocation"].append(st["predicted_capacity"] / max(st["num_pairs"], 1) - 1.0)
    r.set_binning(gbr.BINNING_EXACT)
    r.set_timing(True)
    t = statistics.mean(out["ms_per_step"]) / 1e3
    return {"ms_per_step": t * 1e3, "triangles_per_s": N_TRI / t, "ms_binning": statistics.mean(out["ms_binning"]),
            "frame_overflow_rate": out["overflow"] / (2 * args.steps),
            "over_allocation": statistics.mean(out["over_allocation"]),
            "model": ("sampled pairs x 8, no network" if sampled else
                      "12-64-64-1 MLP, BF16 weights (custom-gpgpu-rasterizer_gb300/predictor_weights.npz)")}


def run_ours(args, rank, world, local):
    import torch
    import gbr

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    # replicas: one seeded frame per rank (weak scaling); rows: one frame
    # split across the ranks by bin rows (strong scaling, composited once)
    split_rows = world > 1 and args.split == "rows"
    scene = make_scene(0 if split_rows else rank)
    mesh = scene.meshes[0]
    vbytes = mesh.vertices.nbytes
    nv = len(mesh.vertices)
    d_vert = torch.from_numpy(mesh.vertices.view(np.uint8)).to(dev)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream

    # device-resident frame ---------------------------------------------------
    r = gbr.Renderer(WIDTH, HEIGHT)
    r.setup_bins(scene.num_bins_x, scene.num_bins_y, BIN, BIN, CHUNK)
    r.bind_mesh_device(d_vert.data_ptr(), nv, mesh.vertex_format)
    band = None
    if split_rows:
        import sharding
        band = sharding.row_bands(scene.num_bins_y, world)[rank]
        r.set_bin_rows(*band)
    r.set_timing(True)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            r.render_scene(scene, sptr)
        st = r.stats(sptr)
    torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    # stage breakdown: an event between stages (keeps launches from overlapping)
    ms_setup, ms_bin, ms_raster, ms_shade = [], [], [], []
    with torch.cuda.stream(stream):
        for _ in range(args.steps):
            flush.zero_()
            r.render_scene(scene, sptr)
            st = r.stats(sptr)
            ms_setup.append(st["ms_setup"]); ms_bin.append(st["ms_bin"])
            ms_raster.append(st["ms_raster"]); ms_shade.append(st["ms_shade"])
    # the raster with setup records staged by bulk asynchronous copies
    # (GBR_STAGING_TMA) on the same frames, for comparison
    ms_raster_tma = []
    r.set_raster_staging(True)
    with torch.cuda.stream(stream):
        for _ in range(args.steps):
            flush.zero_()
            r.render_scene(scene, sptr)
            ms_raster_tma.append(r.stats(sptr)["ms_raster"])
    r.set_raster_staging(False)
    # the timed frames: frame events only
    r.set_timing(True, total_only=True)
    with torch.cuda.stream(stream):
        r.render_scene(scene, sptr)
        r.stats(sptr)
    torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    sampler = ClockSampler(local)
    ms_total = []
    torch.cuda.synchronize(dev)
    sampler.begin()
    with torch.cuda.stream(stream):
        for _ in range(args.steps):
            flush.zero_()
            r.render_scene(scene, sptr)
            st = r.stats(sptr)
            ms_total.append(st["ms_total"])
    torch.cuda.synchronize(dev)
    sampler.end()

    def frame():
        with torch.cuda.stream(stream):
            flush.zero_()
            r.render_scene(scene, sptr)
            r.stats(sptr)
    sampler.hold(frame)
    clocks = sampler.stop()
    r.set_timing(True)
    predicted = predicted_binning(r, scene, args, stream, flush)
    if predicted is not None:
        # learned against exact binning on the same renderer and frame
        ms_exact = statistics.mean(ms_total)
        bin_exact = statistics.mean(ms_setup) + statistics.mean(ms_bin)
        predicted["frame_ratio"] = ms_exact / predicted["ms_per_step"]
        predicted["binning_ratio"] = bin_exact / predicted["ms_binning"]
        predicted["ms_binning_exact"] = bin_exact
        predicted["sampled_count_rule"] = predicted_binning(r, scene, args, stream, flush, sampled=True)
    pairs = st["num_pairs"]
    t_frame = sum(ms_total) / len(ms_total) / 1e3
    (t_frame,) = max_over_ranks([t_frame], dist, dev)
    value = (1 if split_rows else world) * N_TRI / t_frame
    composite_ok = None
    if split_rows:   # the bands gathered into the frame once, against a one-GPU render of it
        import sharding
        colour, _ = r.readback(stream=sptr)
        y0, y1 = sharding.band_pixel_rows(band, BIN, HEIGHT)
        frame = sharding.gather_composite(dist, np.ascontiguousarray(colour[y0:y1]), y0, y1, HEIGHT, WIDTH)
        r.set_bin_rows(0, 0)
        r.render_scene(scene, sptr)
        whole, _ = r.readback(stream=sptr)
        composite_ok = bool(np.array_equal(frame, whole))
    t_raster = sum(ms_raster) / len(ms_raster) / 1e3
    raster_bytes = 4 * pairs + 8 * WIDTH * HEIGHT
    frame_bytes = vbytes + 8 * pairs + 8 * WIDTH * HEIGHT
    peak, peak_kind = measured_peak()
    achieved = raster_bytes / t_raster / 1e9
    r.close()

    # end to end through the C ABI with host buffers -----------------------
    # Every step uploads its vertices from pinned host memory, renders, and
    # reads its framebuffer back to pinned host memory.  Three renderers on
    # three streams (triple buffering, as a streaming host would do): steps
    # k+1 and k+2 are queued before step k's readback waits, so the copies
    # run under the other steps' frames.  The L2 flush is queued on every
    # step's stream inside the timed region.
    depth = E2E_DEPTH
    streams_e = [stream] + [torch.cuda.Stream(device=dev) for _ in range(depth - 1)]
    rs = []
    for _ in range(depth):
        rr = gbr.Renderer(WIDTH, HEIGHT)
        rr.load_scene(scene, CHUNK)
        rs.append(rr)
    host_v = torch.from_numpy(mesh.vertices.view(np.uint8).copy()).pin_memory()
    host_c = [torch.empty(WIDTH * HEIGHT, dtype=torch.int32).pin_memory() for _ in range(depth)]
    colour_np = [h.numpy().view(np.uint32) for h in host_c]

    def e2e_steps(n):
        for k in range(n):
            i = k % depth
            with torch.cuda.stream(streams_e[i]):
                flush.zero_()
            sp = streams_e[i].cuda_stream
            rs[i].update_vertices(0, host_v.data_ptr(), nv, sp)
            rs[i].render_scene(scene, sp)
            if k >= depth - 1:   # step k - depth + 1 is read back
                j = (k - depth + 1) % depth
                rs[j].readback(colour_np[j], stream=streams_e[j].cuda_stream, want_depth=False)
        for k in range(max(n - depth + 1, 0), n):
            j = k % depth
            rs[j].readback(colour_np[j], stream=streams_e[j].cuda_stream, want_depth=False)

    e2e_steps(max(args.warmup, depth))
    torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    e2e_steps(args.steps)
    torch.cuda.synchronize(dev)
    t_e2e = (time.perf_counter() - t0) / args.steps
    (t_e2e,) = max_over_ranks([t_e2e], dist, dev)
    for rr in rs:
        rr.close()

    # the workload's other configurations, measured in the same run and
    # nested in this line: the lit 4K icosphere and the 256-scene batch
    extra = {}
    if world == 1 and not args.soup_only:
        import copy
        sub = copy.copy(args)
        sub.steps, sub.warmup = min(args.steps, 10), max(3, min(args.warmup, 5))
        ico = run_icosphere(sub, rank, world, local, nested=True)
        extra["icosphere7_4k"] = {"metric": ico["metric"], "value": ico["value"], "unit": UNIT,
                                  "ms_per_step": ico["ms_per_step"], "steps": sub.steps, **ico["config"]}
        bat = run_batch(sub, rank, world, local, nested=True)
        extra["batch_256"] = {"metric": bat["metric"], "value": bat["value"], "unit": UNIT,
                              "ms_per_step": bat["ms_per_step"], "steps": sub.steps, "e2e": bat["e2e"],
                              "cpu_baseline": bat["cpu_baseline"], **bat["config"]}

    line = None
    if rank == 0:
        cpu = None
        if world == 1 and not args.no_cpu_baseline:
            ref = reference_cpu(scene, 1, 1)
            if ref is not None:
                cpu = {"value": ref["triangles"] / (ref["ms_per_frame"] / 1e3), "unit": UNIT, "cores": 1,
                       "kind": "reference",
                       "sample": "one full frame of the same 1M soup at 1920x1080 after a warm-up frame, rendered by "
                                 "the reference's ERenderer (single-threaded as written)"}
            else:
                threads = os.cpu_count() or 1
                dt, _ = cpu_baseline(scene, threads)
                cpu = {"value": N_TRI / dt, "unit": UNIT, "cores": threads, "kind": "port",
                       "sample": "one full frame of the same 1M soup (setup, binning, raster, shading)"}
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_frame * 1e3, "higher_is_better": True,
                "scaling": "strong" if split_rows else "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (one seeded soup split by bin rows)" if split_rows else "synthetic (seeded soup per rank)",
                "config": {"workload": WORKLOAD, "triangles": N_TRI, "resolution": [WIDTH, HEIGHT],
                           "bins": [BIN, BIN], "queue_chunk": CHUNK, "binning": "exact two-pass",
                           "l2": "256 MB write between timed frames", "pairs": int(pairs),
                           "frames_per_s": (1 if split_rows else world) / t_frame,
                           "ms_setup": statistics.mean(ms_setup), "ms_bin": statistics.mean(ms_bin),
                           "ms_raster": statistics.mean(ms_raster), "ms_shade": statistics.mean(ms_shade),
                           "ms_raster_tma_staging": statistics.mean(ms_raster_tma),
                           "frame_hbm_frac": frame_bytes / t_frame / 1e9 / peak,
                           "predicted_binning": predicted, **extra,
                           "split": ({"bin_rows": list(band), "composite_equals_one_gpu_frame": composite_ok}
                                     if split_rows else "replicas")},
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": profile_traffic(), "kernel": "raster_kernel",
                             "peak_source": peak_kind, "algorithmic_bytes_per_launch": raster_bytes},
                "e2e": {"value": world * N_TRI / t_e2e, "unit": UNIT, "h2d_bytes_per_step": vbytes,
                        "d2h_bytes_per_step": WIDTH * HEIGHT * 4},
                # setup, scan, fill, raster, shade, and a list-zeroing pass for frames of
                # >= 2^20 pairs counted without block rows (block rows zero it in setup)
                "gpu_launches": (6 if pairs >= 1 << 20 and not st["count_blocks"] else 5) * args.steps,
                "clocks": clocks,
                "cpu_baseline": cpu}
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return line


def run_icosphere(args, rank, world, local, nested=False):
    """The dense sub-pixel workload: the displaced icosphere (7 subdivisions,
    327,680 triangles) at 3840x2160 with the 2048^2 noise texture, bilinear
    filtering and a directional plus a point light, with 8x8 and with 16x16
    bins.  Prints its line, or with `nested` returns it (the default run
    nests it in the soup's line)."""
    import torch
    import gbr
    import scenes

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    per_bins = {}
    sampler = ClockSampler(local)
    sampler.begin()
    for bins in (8, 16):
        s = scenes.icosphere_lit_scene(bin_size=bins)
        with gbr.Renderer(s.width, s.height) as r:
            r.load_scene(s, CHUNK)
            r.set_timing(True)
            with torch.cuda.stream(stream):
                for _ in range(args.warmup):
                    r.render_scene(s, sptr)
                    st = r.stats(sptr)
                stages = st
                r.set_timing(True, total_only=True)
                ms = []
                for _ in range(args.steps):
                    flush.zero_()
                    r.render_scene(s, sptr)
                    st = r.stats(sptr)
                    ms.append(st["ms_total"])
                torch.cuda.synchronize(dev)
                if bins == 16:
                    sampler.end()

                    def frame():
                        flush.zero_()
                        r.render_scene(s, sptr)
                        r.stats(sptr)
                    sampler.hold(frame)
            per_bins[bins] = {"ms_frame": statistics.mean(ms), "pairs": int(st["num_pairs"]),
                              "visible": int(st["num_visible"]), "ms_setup": stages["ms_setup"],
                              "ms_bin": stages["ms_bin"], "ms_raster": stages["ms_raster"],
                              "ms_shade": stages["ms_shade"]}
    clocks = sampler.stop()
    n_tri = s.num_triangles
    best = min(per_bins, key=lambda k: per_bins[k]["ms_frame"])
    t = per_bins[best]["ms_frame"] / 1e3
    line = {"metric": "triangles/s (icosphere-7 3840x2160, bilinear, directional + point light)",
            "value": n_tri / t, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded mesh)",
            "config": {"workload": "icosphere7-4k-lit", "triangles": n_tri,
                       "resolution": [3840, 2160], "best_bins": best,
                       "bins_8x8": per_bins[8], "bins_16x16": per_bins[16],
                       "l2": "256 MB write between timed frames"},
            # setup, scan, fill, raster, shade queue, shade; two bin sizes
            "gpu_launches": 6 * args.steps * 2, "clocks": clocks}
    if rank == 0 and not nested:
        print(json.dumps(line), flush=True)
    return line


BATCH_SCENES = 256
BATCH_METRIC = "triangles/s (256 uneven soups, one batched frame)"


def reference_cpu_batch(sl, workers: int, every: int = 8):
    """The batch workload's CPU baseline: N concurrent instances of the
    reference's ERenderer (ERenderer.cpp:42-164, single-threaded as written),
    one scene per instance, `workers` at a time, on every `every`-th scene of
    the batch (a bounded sample).  Each instance renders one warm-up and one
    timed frame; the aggregate is the sample's triangles over its instances'
    timed frame times divided among the workers that ran them concurrently.
    None where the reference does not build here."""
    import concurrent.futures as cf
    try:
        from oracle.ref import build_ref, ref_io
        exe = build_ref.build_erenderer()
        sample = sl[::every]
        with tempfile.TemporaryDirectory() as d:
            paths = []
            for i, s in enumerate(sample):
                p = os.path.join(d, f"scene{i}.bin")
                ref_io.write_scene(s, p)
                paths.append(p)

            def one(p):
                out = subprocess.run([exe, p, "1", "1"], capture_output=True, text=True, check=True)
                return json.loads(out.stdout.strip().splitlines()[-1])
            t0 = time.perf_counter()
            with cf.ThreadPoolExecutor(max_workers=workers) as ex:
                res = list(ex.map(one, paths))
            wall = time.perf_counter() - t0
        tris = sum(r["triangles"] for r in res)
        busy = sum(r["ms_per_frame"] for r in res) / 1e3
        return {"value": tris / (busy / workers), "unit": UNIT, "cores": workers, "kind": "reference",
                "sample": (f"{len(sample)} of the {len(sl)} scenes (every {every}th, {tris} triangles), one "
                           f"ERenderer process per scene, {workers} at a time, one timed frame each after a "
                           f"warm-up frame; wall {wall:.1f} s including scene loading")}
    except Exception as e:  # noqa: BLE001 -- reported, the batch line then has no CPU baseline
        print(f"reference CPU renderer unavailable for the batch ({type(e).__name__}: {e})", file=sys.stderr)
        return None


# The batch autotuner's space: the workload's bin sizes, queue chunks and
# threads per bin, and the raster variants (CTAs of 256 threads per SM).
# Wider chunks are tuned separately and reported beside it.
BATCH_BINS = (8, 16, 32)
BATCH_CHUNKS = (32, 64, 128)
BATCH_WIDE_CHUNKS = (512, 2048, 4096)
BATCH_RASTER_CTAS = (5, 6)
BATCH_RASTER_THREADS = (128, 256)


def run_batch(args, rank, world, local, nested=False, dist=None):
    """The batched workload: 256 seeded soups (1k-500k triangles, resolutions
    256^2 .. 1920x1080), one graph-replayed launch chain per batch frame, bin
    size / queue chunk / raster variant chosen by the autotuner; beside it,
    the same scenes rendered one frame per scene on the same stream, and N
    concurrent reference ERenderers on the host.  Prints its line, or with
    `nested` returns it."""
    import torch
    import gbr
    import scenes

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1 and dist is None:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    # one batch of scenes for the whole job; under torchrun each rank takes
    # its share by estimated cost (sharding.scene_partition, no collective)
    import sharding
    nscenes = getattr(args, "batch_scenes", BATCH_SCENES)
    specs = scenes.batch_scene_specs(nscenes, seed=0)
    part = sharding.scene_partition([sharding.scene_cost(n, w, h) for n, w, h, _ in specs], world)[rank]
    sl = scenes.batch_scenes(nscenes, seed=0, only=part)
    n_tri = sum(n for n, _, _, _ in specs)   # the job's triangles, all ranks
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    rs = []
    for s in sl:
        r = gbr.Renderer(s.width, s.height)
        r.load_scene(s, CHUNK)
        rs.append(r)
    b = gbr.Batch()
    for r, s in zip(rs, sl):
        b.add_scene(r, s)
    t0 = time.perf_counter()
    wide = None
    with torch.cuda.stream(stream):
        # wider queue chunks than the workload names: tuned first, timed, reported as an extra
        wide_cfg = b.autotune(bin_sizes=BATCH_BINS, chunks=BATCH_WIDE_CHUNKS, raster_ctas=BATCH_RASTER_CTAS, frames=2,
                              stream=sptr, raster_threads=BATCH_RASTER_THREADS)
        b.set_timing(True)
        ms_w = []
        for _ in range(3):
            flush.zero_()
            b.render(sptr)
            ms_w.append(b.stats(sptr)["ms_frame"])
        wide = {"tuned": wide_cfg, "ms_frame": statistics.median(ms_w)}
        best = b.autotune(bin_sizes=BATCH_BINS, chunks=BATCH_CHUNKS, raster_ctas=BATCH_RASTER_CTAS, frames=2,
                          stream=sptr, raster_threads=BATCH_RASTER_THREADS)
    t_tune = time.perf_counter() - t0
    b.set_timing(True)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            b.render(sptr)
        st = b.stats(sptr)
    torch.cuda.synchronize(dev)
    sampler = ClockSampler(local)
    ms = []
    sampler.begin()
    with torch.cuda.stream(stream):
        for _ in range(args.steps):
            flush.zero_()
            b.render(sptr)
            st = b.stats(sptr)
            ms.append(st["ms_frame"])
    torch.cuda.synchronize(dev)
    sampler.end()

    def frame():
        with torch.cuda.stream(stream):
            flush.zero_()
            b.render(sptr)
            b.stats(sptr)
    sampler.hold(frame)
    clocks = sampler.stop()
    t_batch = statistics.mean(ms) / 1e3

    # the same scenes, one single-scene frame each, back to back on the stream
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        for r, s in zip(rs, sl):
            r.render_scene(s, sptr)
        seq = []
        for _ in range(max(2, args.steps // 4)):
            flush.zero_()
            ev0.record(stream)
            for r, s in zip(rs, sl):
                r.render_scene(s, sptr)
            ev1.record(stream)
            ev1.synchronize()
            seq.append(ev0.elapsed_time(ev1))
    t_seq = statistics.mean(seq) / 1e3

    # end to end: vertices from pinned host memory, batch frame, colours
    # back.  Two batches of the same scenes (two renderer sets) on two
    # streams: batch step k+1's uploads and frame are queued before step k's
    # readbacks wait, as a streaming host would do; wall clock over all steps.
    hosts = [torch.from_numpy(s.meshes[0].vertices.view(np.uint8).copy()).pin_memory() for s in sl]
    outs = [[torch.empty(s.width * s.height, dtype=torch.int32).pin_memory() for s in sl] for _ in range(2)]
    h2d = sum(h.numel() for h in hosts)
    d2h = sum(o.numel() * 4 for o in outs[0])
    rs2 = []
    for s in sl:
        r = gbr.Renderer(s.width, s.height)
        r.load_scene(s, CHUNK)
        rs2.append(r)
    b2 = gbr.Batch()
    for r, s in zip(rs2, sl):
        b2.add_scene(r, s)
    b2.set_config(**best)
    stream2 = torch.cuda.Stream(device=dev)
    sets = [(b, rs, stream), (b2, rs2, stream2)]

    def batch_e2e_steps(n):
        for k in range(n):
            bb, rr, ss = sets[k % 2]
            sp = ss.cuda_stream
            for r, h, s in zip(rr, hosts, sl):
                r.update_vertices(0, h.data_ptr(), len(s.meshes[0].vertices), sp)
            bb.render(sp)
            if k > 0:
                read_batch((k - 1) % 2)
        read_batch((n - 1) % 2)

    def read_batch(j):   # every scene's colours, one wait
        bb, _, ss = sets[j]
        bb.readback_all([o.data_ptr() for o in outs[j]], stream=ss.cuda_stream)

    batch_e2e_steps(max(args.warmup, 2))
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    batch_e2e_steps(args.steps)
    torch.cuda.synchronize(dev)
    t_e2e = (time.perf_counter() - t0) / args.steps
    b2.close()
    for r in rs2:
        r.close()
    t_batch, t_e2e, t_seq = max_over_ranks([t_batch, t_e2e, t_seq], dist, dev)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = reference_cpu_batch(sl, os.cpu_count() or 1)
    line = None
    if rank == 0:
        line = {"metric": BATCH_METRIC, "value": n_tri / t_batch, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_batch * 1e3, "higher_is_better": True,
                "scaling": "strong", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded soups, partitioned across ranks by cost)",
                "config": {"workload": "batch-256-uneven-soups", "scenes": nscenes, "triangles": n_tri,
                           "scenes_per_rank": len(part),
                           "pixels": int(sum(w * h for _, w, h, _ in specs)), "tuned": best,
                           "autotune_s": t_tune, "pairs": int(st["num_pairs"]),
                           "work_items": int(st["num_work_items"]), "graph_captures": int(st["graph_captures"]),
                           "batch_frames_per_s": 1.0 / t_batch,
                           "per_scene_frames_ms": t_seq * 1e3,
                           "per_scene_triangles_per_s": n_tri / t_seq,
                           "batch_speedup_vs_per_scene": t_seq / t_batch,
                           "autotune_space": {"bins": BATCH_BINS, "queue_chunks": BATCH_CHUNKS,
                                              "raster_ctas": BATCH_RASTER_CTAS,
                                              "raster_threads": BATCH_RASTER_THREADS},
                           "wide_chunks": wide,
                           "l2": "256 MB write between timed frames"},
                "e2e": {"value": n_tri / t_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "gpu_launches": 6 * args.steps,   # reset, setup, scan, fill, raster, shade
                "clocks": clocks, "cpu_baseline": cpu}
        if not nested:
            print(json.dumps(line), flush=True)
    b.close()
    for r in rs:
        r.close()
    if dist and not nested:
        dist.barrier()
        dist.destroy_process_group()
    return line


def profile_frames(n: int, binning: str = "exact", workload: str = "soup", batch_scenes: int = BATCH_SCENES,
                   staging: str = "loads"):
    """The benchmark's frame, device resident, n times on the default stream
    (with the committed capacity model when binning is "predicted"; setup
    records staged by TMA bulk copies with staging "tma"); with workload
    "icosphere" the lit 4K icosphere frame with 16x16 bins."""
    import torch
    import gbr

    dev = torch.device("cuda", 0)
    if workload == "batch":
        import scenes
        sl = scenes.batch_scenes(batch_scenes, seed=0)
        rs = []
        b = gbr.Batch()
        for s in sl:
            rr = gbr.Renderer(s.width, s.height)
            rr.load_scene(s, CHUNK)
            rs.append(rr)
            b.add_scene(rr, s)
        # the autotuner's pick for these scenes over the workload's space
        b.set_config(32, 128, 5, 0, raster_threads=128)
        for _ in range(n):
            b.render()
        st = b.stats()
        torch.cuda.synchronize(dev)
        b.close()
        for rr in rs:
            rr.close()
        print(json.dumps({"frames": n, "pairs": st["num_pairs"], "scenes": len(sl)}))
        return
    if workload == "icosphere":
        import scenes
        s = scenes.icosphere_lit_scene(bin_size=16)
        r = gbr.Renderer(s.width, s.height)
        r.load_scene(s, CHUNK)
        for i in range(n):
            r.render_scene(s)
            if i == 0:
                r.stats()
        st = r.stats()
        torch.cuda.synchronize(dev)
        r.close()
        print(json.dumps({"frames": n, "pairs": st["num_pairs"], "visible": st["num_visible"]}))
        return
    scene = make_scene(0)
    mesh = scene.meshes[0]
    d_vert = torch.from_numpy(mesh.vertices.view(np.uint8)).to(dev)
    r = gbr.Renderer(WIDTH, HEIGHT)
    r.setup_bins(scene.num_bins_x, scene.num_bins_y, BIN, BIN, CHUNK)
    r.bind_mesh_device(d_vert.data_ptr(), len(mesh.vertices), mesh.vertex_format)
    if binning == "predicted":
        import predictor
        predictor.install(r)
    r.set_raster_staging(staging == "tma")
    for i in range(n):
        r.render_scene(scene)
        if i == 0:
            r.stats()   # the first frame sizes the bin storage (predicted capacities)
    st = r.stats()
    torch.cuda.synchronize(dev)
    r.close()
    print(json.dumps({"frames": n, "pairs": st["num_pairs"], "visible": st["num_visible"]}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--split", choices=["replicas", "rows"], default="replicas",
                    help="under torchrun: one seeded soup per rank (replicas), or one soup split by bin rows")
    ap.add_argument("--soup-only", action="store_true",
                    help="the 1M-triangle soup alone (the default run also measures the icosphere and the batch)")
    ap.add_argument("--workload", choices=["soup", "batch", "icosphere"], default="soup",
                    help="soup: the 1M-triangle 1080p frame; batch: 256 uneven soups as one batched frame; "
                         "icosphere: the lit 4K icosphere with 8x8 and 16x16 bins")
    ap.add_argument("--batch-scenes", type=int, default=BATCH_SCENES,
                    help="scenes of the batch workload (its --profile-frames too)")
    ap.add_argument("--binning", choices=["exact", "predicted"], default="exact",
                    help="binning of the --profile-frames frames")
    ap.add_argument("--staging", choices=["loads", "tma"], default="loads",
                    help="raster setup-record staging of the --profile-frames frames")
    ap.add_argument("--profile-frames", type=int, default=0,
                    help="render this many device-resident frames and exit (for a profiler)")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.profile_frames:
        import build as gbr_build
        gbr_build.build()
        profile_frames(args.profile_frames, args.binning, args.workload, args.batch_scenes, args.staging)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import build as gbr_build
    if rank == 0:
        gbr_build.build()
    else:
        while not gbr_build.up_to_date():
            time.sleep(1)
    if args.workload == "batch":
        run_batch(args, rank, world, local)
    elif args.workload == "icosphere":
        run_icosphere(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
