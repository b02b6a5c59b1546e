"""Benchmark: Mpaths/s of the wavefront path tracer on the 1M-triangle scene.

Workload (one step = one progressive frame, K steps = the K-frame job, 256
by default): 12 instances of a level-6 icosphere (81,920 triangles
each) + a 2-triangle ground plane + 100k alpha-tested quads (64 distinct
512x512 RGBA8 value-noise masks, 50% cut out), Hosek-Wilkie sky (sun
elevation 30 deg, turbidity 3) baked to a 2048x1024 FP16 lat-long map with
importance sampling, 4 point lights; 1920x1080, 1 sample per pixel per
frame, max depth 8, reference shading policy.  Synthetic, seeded procedural
data.

value     = paths / device time of the K-frame job (hx_integrator_render_frames;
            --frames-per-wavefront frames traced together, the image equal to
            K single-frame calls), CUDA events on the library stream
progressive_one_frame_per_call = the same frame rendered one call at a time
            (a viewer's loop): Mpaths/s and per-frame latency p50/p99
e2e       = one frame per C-ABI call with the frame constants passed from the
            host and the tone-mapped RGBA8 frame copied to pinned host memory
            every frame (host wall clock)
roofline  = traversal kernel (k_extend_batched: one bounce's extension rays +
            the previous bounce's shadow rays): algorithmic bytes per launch /
            its mean launch time (bytes = extension rays x (ray 36 B + hit
            16 B) + shadow rays x 48 B + node fetches x 80 B + triangle tests
            x 48 B, counted in a separate counting pass of the same wavefront)

--impl reference times the oracle's scalar transcription of the reference
shaders (the reference's Vulkan path cannot run without a graphics stack) on
all host cores, on a bounded sample of the same frame.
"""
import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WIDTH, HEIGHT, DEPTH = 1920, 1080, 8
METRIC = "Mpaths/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=256, help="frames (the 256-frame job of 1 spp each)")
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--frames-per-wavefront", type=int, default=64,
                   help="frames traced together by one wavefront (render_frames batching; same image; 64: 34 GB "
                        "of path state)")
    p.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline sample budget")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--serving", action="store_true", help="serving workload (Poisson request stream)")
    p.add_argument("--rate", type=float, default=200.0)
    p.add_argument("--duration", type=float, default=8.0)
    p.add_argument("--scenes", type=int, default=8)
    p.add_argument("--tick-paths", type=int, default=2 << 20, help="paths per tick of requests that fit in one tick")
    p.add_argument("--long-tick-paths", type=int, default=1 << 20, help="paths per tick of longer requests")
    p.add_argument("--arena-gb", type=float, default=64.0)
    p.add_argument("--concurrent-ticks", type=int, default=1)
    p.add_argument("--precision", action="store_true", help="precision-form report (terrain scene)")
    p.add_argument("--terrain-size", type=int, default=4096)
    p.add_argument("--spp", type=int, default=4096)
    p.add_argument("--ref-spp", type=int, default=16384)
    p.add_argument("--ref-pixels", type=int, default=4096)
    p.add_argument("--denoise", action="store_true", help="learned-denoiser training + time-to-RMSE report")
    p.add_argument("--denoise-kernels", action="store_true",
                   help="denoiser kernel timing: 1080p inference and a 16 x 256^2 training step (random network)")
    p.add_argument("--dn-iters", type=int, default=20, help="timed iterations of --denoise-kernels")
    p.add_argument("--dn-variants", type=int, default=768)
    p.add_argument("--dn-target-spp", type=int, default=4096)
    p.add_argument("--dn-steps", type=int, default=150000)
    p.add_argument("--dn-ref-spp", type=int, default=4096)
    p.add_argument("--dn-eval-seeds", type=int, nargs="+", default=[5000, 5001])
    p.add_argument("--dn-save", default="", help="directory for the trained parameters (one .npy per loss)")
    p.add_argument("--dn-losses", nargs="+", default=["hybrid"], choices=["l1log", "l2lin", "hybrid"],
                   help="train one network per loss on the same data (hybrid: l1log for the first 20%% of "
                        "the steps, then l2lin)")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class Dist:
    """Host-side barrier / max-reduce across replica ranks (gloo); no data-path collective."""

    def __init__(self):
        self.rank, self.world, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def allreduce(self, x, op):
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX if op == "max" else self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


def workload_config():
    return {"workload": "icospheres_1M_alpha_quads_sky_1080p_1spp_depth8", "scene": "12 x level-6 icosphere "
            "(983,040 tris) + 2-tri ground + 100k alpha quads (200k tris; 64 masks 512^2, 50% cutout)",
            "width": WIDTH, "height": HEIGHT, "spp_per_step": 1, "max_depth": DEPTH, "policy": "reference + "
            "importance-sampled environment", "env": "Hosek-Wilkie sun 30 deg turbidity 3, 2048x1024 FP16",
            "l2": "per-frame working set (path state 2.07M x 176 B + BVH/scene) larger than L2; no flush"}


def make_scene(hx):
    return hx.HostScene(hx.SCENE_ICOSPHERES)


def make_policy(hx):
    pol = hx.policy_reference()
    pol.env_sampling = hx.ENV_SAMPLE_IMPORTANCE
    return pol


def idesc(hx, pol):
    d = hx.IntegratorDesc()
    d.width, d.height, d.max_ray_bounces, d.max_samples = WIDTH, HEIGHT, DEPTH, 1 << 30
    d.policy = pol
    return d


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peaks():
    """Roofline denominators: MEASURED_PEAKS.json when present, else the
    pool's fallback figures (6.8 TB/s copy bandwidth, 1.9 / 1.7 PFLOP/s BF16
    burst / sustained), with the source named."""
    try:
        p = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return {"hbm_gbs": float(p["hbm_gbs"]), "bf16_tflops": float(p["bf16_tflops"]),
                "bf16_tflops_sustained": float(p.get("bf16_tflops_sustained", p["bf16_tflops"])),
                "source": "of measured (MEASURED_PEAKS.json)"}
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
                "source": "of fallback (MEASURED_PEAKS.json absent)"}


def cpu_sample(hs, hx, pol, seconds, threads=0, osc=None):
    """Oracle (scalar FP32 transcription of the reference shaders) on whole
    image rows of the same frame (wrapping around the frame) until the time
    budget is used.  osc: the oracle's copy of the scene (built here if None)."""
    from oracle import binding as ob
    own = osc is None
    if own:
        osc = ob.OracleScene(hs)
    d = idesc(hx, pol)
    f = hx.frame_desc(hs.camera(), WIDTH, HEIGHT)
    paths = segs = 0
    secs = 0.0
    row = HEIGHT // 2 - 8
    rows_done = 0
    chunk = 8
    thr = 0
    while secs < seconds:
        r0 = (row + rows_done) % HEIGHT
        n = min(chunk, HEIGHT - r0)
        import numpy as np
        pix = (np.arange(r0, r0 + n)[:, None] * WIDTH + np.arange(WIDTH)[None, :]).ravel().astype(np.uint32)
        _, cnt = osc.render(d, f, 1, precision=32, pixels=pix, threads=threads)
        paths += cnt.paths
        segs += cnt.extension_rays + cnt.shadow_rays
        secs += cnt.seconds
        thr = cnt.threads
        rows_done += n
        chunk = min(64, chunk * 2)
    if own:
        osc.close()
    return {"paths": paths, "segments": segs, "seconds": secs, "threads": thr, "rows": rows_done}


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def run_reference(args, dist):
    if dist.rank != 0:
        return
    import helios_gb300 as hx
    from oracle import binding as ob
    hs = make_scene(hx)
    pol = make_policy(hx)
    osc = ob.OracleScene(hs)
    per_step = []
    total_paths = 0
    total_secs = 0.0
    thr = 0
    # bounded sample per step: the whole run stays within about a minute of CPU time
    budget = min(2.5, max(0.05, 60.0 / (args.warmup + args.steps)))
    for k in range(args.warmup + args.steps):
        r = cpu_sample(hs, hx, pol, budget, osc=osc)
        if k >= args.warmup:
            per_step.append(r["seconds"] * 1000.0)
            total_paths += r["paths"]
            total_secs += r["seconds"]
            thr = r["threads"]
    value = total_paths / total_secs / 1e6
    sample = "%d frame rows of 1920 px per step (%.1f s budget), 1 spp, depth 8" % (r["rows"], budget)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mpaths/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(per_step),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(),
            "cpu_baseline": {"value": value, "unit": "Mpaths/s", "cores": thr, "kind": "port", "sample": sample,
                             "cpu": cpu_model()},
            "e2e": {"value": value, "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, dist):
    import numpy as np
    import helios_gb300 as hx
    ctx = hx.Context(dist.local)
    hs = make_scene(hx)
    scene = hx.Scene(ctx, hs)
    info = scene.info()
    pol = make_policy(hx)
    fpw = max(1, args.frames_per_wavefront)
    it = hx.PathIntegrator(ctx, scene, WIDTH, HEIGHT, max_ray_bounces=DEPTH, max_samples=1 << 30, policy=pol,
                           max_paths_in_flight=WIDTH * HEIGHT * fpw)
    frame = hx.frame_desc(hs.camera(), WIDTH, HEIGHT)
    paths_per_step = WIDTH * HEIGHT

    # 1) stage breakdown + segment counts of one wavefront (fpw frames; timing
    #    mode syncs per stage: not the timed region)
    it.set_timing(True)
    it.render(frame, fpw)
    st = it.stats()
    segs_per_step = (st.extension_rays + st.shadow_rays) / fpw
    ms_trace_per_launch = st.ms_trace / max(1, st.trace_launches)
    stage = {k: v / fpw for k, v in (("raygen", st.ms_raygen), ("traverse (extension + shadow)", st.ms_trace),
                                     ("shade", st.ms_shade), ("accumulate", st.ms_accumulate))}
    it.set_timing(False)
    # 2) counting pass: node fetches and triangle tests of the closest-hit launches
    it.set_counting(True)
    it.render(frame, fpw)
    ct = it.stats()
    it.set_counting(False)
    ext_rays = ct.extension_rays
    sh_rays = ct.shadow_rays
    trav_bytes = ct.node_visits * 80 + ct.tri_tests * 48
    alg_bytes_per_launch = (ext_rays * (36 + 16) + sh_rays * 48 + trav_bytes) / max(1, ct.trace_launches)
    simd = {"node_step_lanes": ct.node_visits / max(1, 32 * ct.warp_node_steps),
            "tri_step_lanes": ct.tri_tests / max(1, 32 * ct.warp_tri_steps),
            "loop_busy_lanes": ct.lane_loop_busy / max(1, 32 * ct.warp_loop_iters),
            "warp_tri_steps_per_node_step": ct.warp_tri_steps / max(1, ct.warp_node_steps),
            "alpha_tests_per_segment": ct.alpha_tests / max(1, ext_rays + sh_rays)}

    # 3) the K-frame job (1 spp per frame, K frames accumulated), fpw
    #    frames per wavefront; device-timed with CUDA events on the library stream
    it.render(frame, max(args.warmup, fpw))
    ctx.synchronize()
    e0, e1 = hx.Event(ctx), hx.Event(ctx)
    clocks = Clocks(dist.local)
    dist.barrier()
    ctx.synchronize()
    clocks.start()
    e0.record()
    it.render(frame, args.steps)
    e1.record()
    ctx.synchronize()
    clk = clocks.stop()
    launches = it.stats().kernel_launches
    total_ms = e0.elapsed_ms(e1)
    total_ms = dist.allreduce(total_ms, "max")
    paths_all = dist.allreduce(paths_per_step * args.steps, "sum")
    value = paths_all / (total_ms / 1000.0) / 1e6
    seg_rate = dist.allreduce(segs_per_step * args.steps, "sum") / (total_ms / 1000.0) / 1e6

    # 4) progressive display, one frame per call: per-frame device latency, then
    #    end to end through the C-ABI (frame constants from the host, the
    #    tone-mapped RGBA8 frame to pinned host memory every frame)
    prog_frames = min(args.steps, 64)
    events = [hx.Event(ctx) for _ in range(prog_frames + 1)]
    ctx.synchronize()
    events[0].record()
    for k in range(prog_frames):
        it.render(frame)
        events[k + 1].record()
    ctx.synchronize()
    frame_ms = [events[k].elapsed_ms(events[k + 1]) for k in range(prog_frames)]
    prog_value = paths_per_step * prog_frames / (events[0].elapsed_ms(events[-1]) / 1000.0) / 1e6
    out = hx.PinnedBuffer((HEIGHT, WIDTH, 4), np.uint8)
    for _ in range(2):
        it.render(frame)
        hx.check(hx.lib().hx_integrator_tonemap(it.handle, hx.TONEMAP_ACES, 1.0, out.array.ctypes.data))
    dist.barrier()
    ctx.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        it.render(frame)
        hx.check(hx.lib().hx_integrator_tonemap(it.handle, hx.TONEMAP_ACES, 1.0, out.array.ctypes.data))
    ctx.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_s = dist.allreduce(e2e_s, "max")
    e2e_value = paths_all / e2e_s / 1e6
    launches_e2e = it.stats().kernel_launches * args.steps + args.steps  # + one tone-map launch per frame
    out.close()

    peaks = load_peaks()
    hbm_peak = peaks["hbm_gbs"]
    achieved = alg_bytes_per_launch / (ms_trace_per_launch / 1000.0) / 1e9
    # the two-level model of the traversal launch: queue bytes (rays, hits,
    # shadow entries) at the HBM peak, node and triangle bytes (cache-served)
    # at this GPU's L2 read bandwidth, measured here (48 MiB working set)
    l2_gbs = ctx.read_bandwidth(48 << 20, 200)
    hbm_read_gbs = ctx.read_bandwidth(4 << 30, 3)
    queue_b = (ext_rays * (36 + 16) + sh_rays * 48) / max(1, ct.trace_launches)
    trav_b = trav_bytes / max(1, ct.trace_launches)
    t_launch = ms_trace_per_launch / 1000.0
    t_model = queue_b / (hbm_peak * 1e9) + trav_b / (l2_gbs * 1e9)
    l2_model = {"l2_read_gbs": l2_gbs, "hbm_read_gbs": hbm_read_gbs,
                "l2_source": "hx_measure_read_bandwidth: one launch reading a 48 MiB buffer 200 times, L1 bypassed "
                             "(HBM: 4 GiB, 3 passes)",
                "queue_bytes_per_launch": queue_b, "trav_bytes_per_launch": trav_b,
                "trav_achieved_gbs": trav_b / t_launch / 1e9, "trav_frac_of_l2": trav_b / t_launch / 1e9 / l2_gbs,
                "frac": t_model / t_launch}
    traffic = None
    ncu = {}
    try:
        prof = json.load(open(os.path.join(ROOT, "profiles", "trace_kernel_traffic.json")))
        if prof.get("kernel", "").startswith("k_extend"):
            traffic = prof["dram_bytes_per_segment"] * (ext_rays + sh_rays) / max(1, ct.trace_launches)
            ncu = {k: prof[k] for k in ("dram_frac_of_peak", "l2_hit_pct", "l1_hit_pct", "issue_active_pct",
                                        "source") if k in prof}
    except Exception:
        pass

    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        r = cpu_sample(hs, hx, pol, args.cpu_seconds)
        cpu = {"value": r["paths"] / r["seconds"] / 1e6, "unit": "Mpaths/s", "cores": r["threads"], "kind": "port",
               "sample": "%d rows x 1920 px of the same frame, 1 spp, depth 8 (%.1f s)" % (r["rows"], r["seconds"]),
               "cpu": cpu_model(), "mray_segments_per_s": r["segments"] / r["seconds"] / 1e6}

    it.close()
    scene.close()
    if dist.rank == 0:
        fs = sorted(frame_ms)
        line = {"metric": METRIC, "value": value, "unit": "Mpaths/s", "n_gpus": dist.world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": workload_config(),
                "parallelism": "replicas" if dist.world > 1 else "single",
                "frames_per_wavefront": fpw,
                "mray_segments_per_s": seg_rate,
                "progressive_one_frame_per_call": {"mpaths_per_s": prog_value, "frames": prog_frames,
                                                   "frame_latency_ms": {"p50": float(np.percentile(fs, 50)),
                                                                        "p99": float(np.percentile(fs, 99)),
                                                                        "max": fs[-1]}},
                "segments_per_path": segs_per_step / paths_per_step,
                "stage_ms_per_frame": stage,
                "scene": {"triangles": info.num_triangles, "bvh8_nodes": info.num_bvh8_nodes,
                          "build_ms": info.build_ms, "device_mb": info.device_bytes / 2**20},
                "e2e": {"value": e2e_value, "unit": "Mpaths/s", "h2d_bytes_per_step": 128,
                        "d2h_bytes_per_step": WIDTH * HEIGHT * 4,
                        "mode": "one frame per C-ABI call, tone-mapped RGBA8 read back every frame"},
                "gpu_launches": launches,
                "gpu_launches_e2e": launches_e2e,
                "roofline": {"bound": "hbm", "limiter": "latency: dependent L1/L2 node and triangle fetches; "
                                                        "the BVH is cache-resident, DRAM nearly idle",
                             "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                             "frac": achieved / hbm_peak, "traffic": traffic, "ncu": ncu,
                             "kernel": "k_extend_batched (closest hit + shadow)",
                             "peak_source": peaks["source"],
                             "bytes_per_launch": alg_bytes_per_launch, "ms_per_launch": ms_trace_per_launch,
                             "node_fetches_per_segment": ct.node_visits / max(1, ext_rays + sh_rays),
                             "tri_tests_per_segment": ct.tri_tests / max(1, ext_rays + sh_rays),
                             "simd_lanes": simd, "l2_model": l2_model},
                "clocks": clk,
                "cpu_baseline": cpu}
        print(json.dumps(line), flush=True)


RESOLUTIONS = [(256, 256), (1280, 720), (1920, 1080), (3840, 2160)]
SPPS = [1, 4, 16, 64]


def run_serving(args, dist):
    """Serving workload: Poisson arrivals at args.rate req/s for args.duration
    seconds over a pool of resident procedural scenes; each request draws a
    random camera, a resolution from RESOLUTIONS, spp from SPPS and a denoise
    flag.  Reports throughput and p50/p99 latency (submit -> tone-mapped image
    in host memory) of the completed requests, overall and per class."""
    import numpy as np
    import helios_gb300 as hx
    ctx = hx.Context(dist.local)
    rng = np.random.default_rng(1234)
    pol = make_policy(hx)
    srv = hx.Server(ctx, arena_bytes=int(args.arena_gb * (1 << 30)), max_paths_per_tick=args.tick_paths,
                    max_paths_per_long_tick=args.long_tick_paths,
                    max_ray_bounces=DEPTH, policy=pol, max_concurrent_ticks=args.concurrent_ticks)
    dn = hx.Denoiser(ctx)
    wpath = os.path.join(ROOT, "helios_gb300", "weights", "denoiser.npy")
    if os.path.exists(wpath):
        import numpy as np_
        dn.set_params(np_.load(wpath))
        weights = "trained (helios_gb300/weights/denoiser.npy)"
    else:
        dn.init_params(0)
        weights = "seeded initial weights (latency does not depend on the weights)"
    srv.set_denoiser(dn)
    pool = []
    t0 = time.time()
    for k in range(args.scenes):
        if k < 2:
            hs = hx.HostScene(hx.SCENE_BOX)
        else:
            hs = hx.HostScene(hx.SCENE_ICOSPHERES, seed=1000 + k)
        sc = hx.Scene(ctx, hs)
        pool.append((hs, sc, srv.add_scene(sc)))
    build_s = time.time() - t0
    srv.start()
    # warm up every scene's graph once
    for hs, sc, sid in pool:
        rid = srv.submit(sid, hx.frame_desc(hs.camera(), 64, 64), 64, 64, 1)
        while not [r for r in srv.poll(wait_seconds=1.0)]:
            pass
        srv.fetch(rid)
    n_req = int(args.rate * args.duration)
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, size=n_req))
    meta = {}
    submit_t = {}
    results = []
    start = time.perf_counter()
    s0 = srv.stats()
    i = 0
    while i < n_req:
        now = time.perf_counter() - start
        while i < n_req and arrivals[i] <= now:
            hs, sc, sid = pool[int(rng.integers(len(pool)))]
            w, h = RESOLUTIONS[int(rng.integers(4))]
            spp = SPPS[int(rng.integers(4))]
            cam = hs.camera()
            for a in range(3):
                cam.position[a] += float(rng.normal(0, 0.05 if sid < 2 else 1.0))
            denoise = int(rng.random() < 0.5)
            rid = srv.submit(sid, hx.frame_desc(cam, w, h), w, h, spp, user_tag=i, denoise=bool(denoise))
            meta[rid] = (w, h, spp, denoise, sid)
            submit_t[rid] = time.perf_counter() - start
            i += 1
        for r in srv.poll(wait_seconds=0.0005):
            results.append(r)
            srv.fetch(r.request_id)
    elapsed = time.perf_counter() - start
    for r in srv.poll(wait_seconds=0.0):
        results.append(r)
        srv.fetch(r.request_id)
    s1 = srv.stats()
    paths = s1.paths - s0.paths
    srv.close()
    dn.close()

    def pct(v, q):
        return float(np.percentile(v, q)) if len(v) else None

    # every submitted request counts: one unfinished at the window's end is
    # right-censored at (window end - its submit time), a lower bound of its
    # latency; a percentile that lands on a censored value is reported as a
    # lower bound ("censored": true)
    done_ids = {r.request_id for r in results}
    samples = [(r.request_id, r.latency_ms, False) for r in results]
    samples += [(rid, (elapsed - submit_t[rid]) * 1000.0, True) for rid in meta if rid not in done_ids]

    def pct_c(v, q):
        if not v:
            return None
        v = sorted(v)
        k = min(len(v) - 1, int(np.ceil(q / 100.0 * len(v))) - 1)
        return {"ms": v[k][0], "censored": v[k][1]}

    lat_all = [(ms, c) for _, ms, c in samples]
    classes = {}
    classes_all = {}
    queue = {}
    lat = [r.latency_ms for r in results]
    for r in results:
        w, h, spp, dz, sid = meta[r.request_id]
        if dz:
            classes.setdefault("%dx%d/%dspp/denoise" % (w, h, spp), []).append(r.latency_ms)
        classes.setdefault("%dx%d/%dspp" % (w, h, spp), []).append(r.latency_ms)
        queue.setdefault("%dx%d/%dspp" % (w, h, spp), []).append(r.queue_ms)
    for rid, ms, c in samples:
        w, h, spp, dz, sid = meta[rid]
        classes_all.setdefault("%dx%d/%dspp" % (w, h, spp), []).append((ms, c))
    offered = sum(w * h * spp for (w, h, spp, dn, sid) in meta.values())
    line = {"metric": "serving latency p50/p99 (ms) and Mpaths/s", "mode": "serving", "n_gpus": 1,
            "rate_req_per_s": args.rate, "duration_s": args.duration, "requests_submitted": n_req,
            "requests_completed": len(results), "scenes": args.scenes, "scene_build_s": build_s,
            "throughput_mpaths_per_s": paths / elapsed / 1e6, "offered_mpaths_per_s": offered / args.duration / 1e6,
            "latency_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99)},
            "latency_ms_all_submitted": {"p50": pct_c(lat_all, 50), "p99": pct_c(lat_all, 99),
                                         "censored": len(samples) - len(results)},
            "per_class_latency_ms": {k: {"n": len(v), "p50": pct(v, 50), "p99": pct(v, 99)} for k, v in sorted(classes.items())},
            "per_class_latency_ms_all_submitted": {
                k: {"submitted": len(v), "unfinished": sum(1 for _, c in v if c), "p50": pct_c(v, 50),
                    "p99": pct_c(v, 99)} for k, v in sorted(classes_all.items())},
            "per_class_admission_wait_ms": {k: {"p50": pct(v, 50), "p99": pct(v, 99)} for k, v in sorted(queue.items())},
            "tick_paths": args.tick_paths, "long_tick_paths": args.long_tick_paths,
            "concurrent_ticks": args.concurrent_ticks, "arena_gb": args.arena_gb,
            "denoise": "Bernoulli(0.5) per request; denoiser weights: " + weights,
            "requests_denoised": s1.requests_denoised - s0.requests_denoised, "data": "synthetic"}
    print(json.dumps(line), flush=True)


def run_precision(args, dist):
    """Precision form at scale: 200 spheres + a terrain_size^2 fBm
    heightfield, 1920x1080; 8-bit quantised BVH8 boxes, 16-bit ray/hit
    payloads, FP32 traversal, Kahan-compensated FP32 accumulation, to args.spp
    (4096) samples per pixel and on to args.ref_spp (16384).  The FP64
    oracle renders the same sample sequence to args.ref_spp on args.ref_pixels
    seeded pixels (and to args.spp, to separate Monte Carlo noise from
    arithmetic).  Reports throughput, the relative RMSE of each device image
    against the 16k-spp FP64 oracle with its per-pixel distribution, and the
    primary hit-ID agreement of the quantised BVH8 with the oracle's
    unquantised binary tree and of 16-bit with FP32 ray directions.  The
    "_offset" images use HX_RAY_OFFSET_SCALED ray origins and are compared
    with the oracle under the same policy."""
    import numpy as np
    import helios_gb300 as hx
    from oracle import binding as ob
    ctx = hx.Context(dist.local)
    t0 = time.time()
    hs = hx.HostScene(hx.SCENE_TERRAIN, terrain_size=args.terrain_size)
    scene = hx.Scene(ctx, hs)
    info = scene.info()
    t_scene = time.time() - t0
    W, H = WIDTH, HEIGHT
    f = hx.frame_desc(hs.camera(), W, H)
    spp, ref_spp = args.spp, max(args.spp, args.ref_spp)
    out = {"metric": "precision form: relative RMSE vs FP64 oracle", "mode": "precision", "n_gpus": 1,
           "scene": {"triangles": info.num_triangles, "bvh8_nodes": info.num_bvh8_nodes, "build_ms": info.build_ms,
                     "device_mb": info.device_bytes / 2**20, "setup_s": t_scene},
           "width": W, "height": H, "spp": spp, "ref_spp": ref_spp, "data": "synthetic"}
    pix = np.random.default_rng(11).choice(W * H, size=args.ref_pixels, replace=False).astype(np.uint32)
    imgs = {}
    runs = (("fp16_kahan", True, True, False), ("fp32_kahan", False, True, False), ("fp32", False, False, False),
            ("fp16_kahan_offset", True, True, True), ("fp32_kahan_offset", False, True, True))
    for name, fp16, kahan, offset in runs:
        pol = hx.policy_reference()
        pol.env_sampling = hx.ENV_SAMPLE_IMPORTANCE
        pol.payload = hx.PAYLOAD_FP16 if fp16 else hx.PAYLOAD_FP32
        pol.accumulation = hx.ACCUM_KAHAN if kahan else hx.ACCUM_RUNNING_MEAN
        pol.ray_offset = hx.RAY_OFFSET_SCALED if offset else hx.RAY_OFFSET_REFERENCE
        it = hx.PathIntegrator(ctx, scene, W, H, max_ray_bounces=DEPTH, max_samples=ref_spp, policy=pol,
                               max_paths_in_flight=W * H * 4)
        e0, e1 = hx.Event(ctx), hx.Event(ctx)
        ctx.synchronize()
        e0.record()
        it.render(f, spp)
        e1.record()
        ms = e0.elapsed_ms(e1)
        out[name + "_mpaths_per_s"] = W * H * spp / (ms / 1000.0) / 1e6
        imgs[(name, spp)] = it.read_accumulation()[:, :, :3].reshape(-1, 3).astype(np.float64)
        if name != "fp32":
            it.render(f, ref_spp - spp)
            imgs[(name, ref_spp)] = it.read_accumulation()[:, :, :3].reshape(-1, 3).astype(np.float64)
        it.close()
    # FP64 oracle (FP32-payload semantics, reference policy, the same sample
    # sequence) on the seeded pixel subset
    osc = ob.OracleScene(hs)
    d = hx.IntegratorDesc()
    d.width, d.height, d.max_ray_bounces, d.max_samples = W, H, DEPTH, 1 << 30
    d.policy = hx.policy_reference()
    d.policy.env_sampling = hx.ENV_SAMPLE_IMPORTANCE
    t1 = time.time()
    ref, cnt = osc.render(d, f, ref_spp, precision=64, pixels=pix)
    ref_lo, _ = osc.render(d, f, spp, precision=64, pixels=pix)
    # the oracle's own FP32 evaluation of the same samples: separates what FP32
    # arithmetic does to the reference's algorithm from what the device does
    ref32, _ = osc.render(d, f, spp, precision=32, pixels=pix)
    # the same three under scaled ray origins
    d.policy.ray_offset = hx.RAY_OFFSET_SCALED
    ref_off, _ = osc.render(d, f, ref_spp, precision=64, pixels=pix)
    ref_off_lo, _ = osc.render(d, f, spp, precision=64, pixels=pix)
    ref32_off, _ = osc.render(d, f, spp, precision=32, pixels=pix)
    out["oracle_s"] = time.time() - t1
    out["oracle_pixels"] = int(pix.size)
    out["oracle_threads"] = cnt.threads

    def rr(a, r=ref):
        return float(np.linalg.norm(a - r) / np.linalg.norm(r))

    def dist_of(a, r=ref):
        e = np.abs(a - r).sum(1) / max(float(np.abs(r).sum(1).mean()), 1e-30)
        q = np.percentile(e, [50, 90, 99, 99.9])
        return {"p50": float(q[0]), "p90": float(q[1]), "p99": float(q[2]), "p99.9": float(q[3]),
                "share_of_squared_error_top_1pct": float(np.sort(e ** 2)[-max(1, e.size // 100):].sum() /
                                                         max((e ** 2).sum(), 1e-300))}
    rel = {}
    for (name, n), img in imgs.items():
        if name.endswith("_offset"):
            rel["%s@%d_vs_fp64_offset@%d" % (name, n, ref_spp)] = {
                "rel_rmse": rr(img[pix], ref_off), "per_pixel_abs_err_over_mean": dist_of(img[pix], ref_off)}
        else:
            rel["%s@%d_vs_fp64@%d" % (name, n, ref_spp)] = {"rel_rmse": rr(img[pix]), "per_pixel_abs_err_over_mean":
                                                           dist_of(img[pix])}
    for name in ("fp16_kahan_offset", "fp32_kahan_offset"):
        rel["%s@%d_vs_fp64_offset@%d" % (name, spp, spp)] = {"rel_rmse": rr(imgs[(name, spp)][pix], ref_off_lo)}
    rel["oracle_fp32_offset@%d_vs_fp64_offset@%d" % (spp, spp)] = {"rel_rmse": rr(ref32_off, ref_off_lo)}
    rel["fp64_offset@%d_vs_fp64_offset@%d (noise of %d spp)" % (spp, ref_spp, spp)] = {"rel_rmse": rr(ref_off_lo, ref_off)}
    rel["fp64_offset@%d_vs_fp64@%d (what the offset changes)" % (ref_spp, ref_spp)] = {"rel_rmse": rr(ref_off)}
    # the Monte Carlo part: the FP64 oracle's own spp-sample image against its ref_spp one
    rel["fp64@%d_vs_fp64@%d (noise of %d spp)" % (spp, ref_spp, spp)] = {"rel_rmse": rr(ref_lo)}
    # the arithmetic part at spp: device vs the FP64 oracle at the same spp and sequence
    for name in ("fp16_kahan", "fp32_kahan", "fp32"):
        rel["%s@%d_vs_fp64@%d" % (name, spp, spp)] = {"rel_rmse": rr(imgs[(name, spp)][pix], ref_lo)}
    rel["oracle_fp32@%d_vs_fp64@%d (FP32 arithmetic of the algorithm itself)" % (spp, spp)] = {
        "rel_rmse": rr(ref32, ref_lo), "per_pixel_abs_err_over_mean": dist_of(ref32, ref_lo)}
    rel["fp32@%d_vs_oracle_fp32@%d (device vs FP32 oracle)" % (spp, spp)] = {
        "rel_rmse": rr(imgs[("fp32", spp)][pix], ref32)}
    out["rel_rmse"] = rel
    out["rel_rmse_fp16_vs_fp32_full_frame@%d" % spp] = float(
        np.linalg.norm(imgs[("fp16_kahan", spp)] - imgs[("fp32_kahan", spp)]) /
        np.linalg.norm(imgs[("fp32_kahan", spp)]))
    # primary hit IDs: quantised BVH8 (device) vs the oracle's unquantised
    # binary tree, FP32 rays; and 16-bit-direction rays vs FP32 rays
    d16 = hx.IntegratorDesc()
    d16.width, d16.height, d16.max_ray_bounces, d16.max_samples = W, H, 1, 1
    d16.policy = hx.policy_reference()
    d16.policy.payload = hx.PAYLOAD_FP16
    sub = np.random.default_rng(12).choice(W * H, size=65536, replace=False).astype(np.uint32)
    r32 = ob.primary_rays(d16, f, 0)[sub]
    gh = scene.trace(r32, any_hit=True)
    oh = osc.trace(r32, any_hit=True)
    out["primary_hit_agreement_quantised_bvh8_vs_unquantised"] = float((gh["prim"] == oh["prim"]).mean())
    _, h16 = osc.sample_radiance(d16, f, 0, precision=32, pixels=sub)
    out["primary_hit_agreement_fp16_vs_fp32"] = float((h16["prim"] == gh["prim"]).mean())
    osc.close()
    scene.close()
    print(json.dumps(out), flush=True)


def run_denoise(args, dist):
    """Learned denoiser: data from this tracer, training by the library's own
    tensor-core kernels, then time-to-RMSE at 1920x1080 on held-out variants
    against plain accumulation."""
    import numpy as np
    import helios_gb300 as hx
    from helios_gb300 import denoise_train as T
    ctx = hx.Context(dist.local)
    peaks = load_peaks()
    probe = hx.Denoiser(ctx)
    nparams = probe.num_params
    probe.close()
    kw = dict(quads=100000, level=6, env=(1024, 512), mask_pool=16, mask_size=256)
    out = {"mode": "denoise", "metric": "time-to-RMSE speed-up vs plain accumulation", "n_gpus": 1,
           "data": "synthetic: seeded variants of the icosphere scene (transforms, materials, lights, masks, sun "
                   "U(10,80) deg, orbit camera); 100k alpha quads, 16 masks 256^2, 1024x512 sky",
           "network": "5-level U-Net, 3x3 convs 32->128 ch, skips; BF16 weights/activations, FP32 accumulate "
                      "(tcgen05/TMEM); %d parameters" % nparams}
    spp_in = [1, 2, 4, 8, 16, 32, 64]
    seeds = list(range(1000, 1000 + args.dn_variants))
    data = T.render_pairs(ctx, seeds, 256, 256, spp_in, args.dn_target_spp, bounces=DEPTH, scene_kw=kw,
                          full_res=(WIDTH, HEIGHT))
    out["train_data"] = {"variants": len(seeds), "pairs": data.count, "crop": [256, 256],
                         "crop_of": [WIDTH, HEIGHT], "input_spp": spp_in, "target_spp": args.dn_target_spp,
                         "render_s": round(data.render_s, 1)}
    e0, e1 = hx.Event(ctx), hx.Event(ctx)
    nets, out["training"] = {}, {}
    for loss in args.dn_losses:
        dn = hx.Denoiser(ctx)
        dn.init_params(0)
        t0 = time.time()
        e0.record()
        if loss == "hybrid":
            warm = args.dn_steps // 5
            dn.set_loss(hx.DN_LOSS_L1_LOG)
            hist = T.train(dn, data, warm, batch=16, lr=1e-3, seed=1, log_every=max(1, args.dn_steps // 10))
            dn.set_loss(hx.DN_LOSS_L2_LINEAR)
            hist += [(s + warm, l) for s, l in T.train(dn, data, args.dn_steps - warm, batch=16, lr=1e-3, lr_final=1e-4,
                                                       seed=2, log_every=max(1, args.dn_steps // 10))]
        else:
            dn.set_loss(hx.DN_LOSS_L2_LINEAR if loss == "l2lin" else hx.DN_LOSS_L1_LOG)
            hist = T.train(dn, data, args.dn_steps, batch=16, lr=1e-3, lr_final=1e-4, seed=1,
                           log_every=max(1, args.dn_steps // 10))
        e1.record()
        ctx.synchronize()
        train_ms = e0.elapsed_ms(e1)
        step_flops = 3.0 * hx.denoiser_conv_flops_per_pixel() * 16 * 256 * 256
        out["training"][loss] = {"steps": args.dn_steps, "batch": 16, "adam_lr": [1e-3, 1e-4],
                                 "wall_s": round(time.time() - t0, 1), "ms_per_step": train_ms / args.dn_steps,
                                 "conv_tflops": step_flops / (train_ms / args.dn_steps * 1e-3) / 1e12,
                                 "loss": [(s, round(l, 5)) for s, l in hist]}
        nets[loss] = dn
        if args.dn_save:
            import numpy as np_
            os.makedirs(args.dn_save, exist_ok=True)
            np_.save(os.path.join(args.dn_save, "denoiser_%s.npy" % loss), dn.get_params())
    data.close()
    # held-out evaluation at 1920x1080
    W, H = WIDTH, HEIGHT
    evals = []
    feat = hx.DeviceBuffer(ctx, W * H * 48)
    den = hx.DeviceBuffer(ctx, W * H * 16)
    checkpoints = [1, 2, 4, 8, 16, 32, 64, 128, 256]
    for seed in args.dn_eval_seeds:
        hs, cam = T.variant_scene(seed, **kw)
        sc = hx.Scene(ctx, hs)
        f = hx.frame_desc(cam, W, H)
        it = hx.PathIntegrator(ctx, sc, W, H, max_ray_bounces=DEPTH, max_samples=1 << 30, policy=hx.policy_reference())
        it.render(f, args.dn_ref_spp)
        ref = it.read_accumulation()[..., 0:3].astype(np.float64)
        # plain frame time (no AOV accumulation), warm
        it.restart_bake()
        it.render(f, 4)
        e0.record()
        it.render(f, 32)
        e1.record()
        ctx.synchronize()
        frame_ms_plain = e0.elapsed_ms(e1) / 32
        it.restart_bake()
        it.set_aov_accumulation(True)
        plain, dnz, done, frame_ms = {}, {k: {} for k in nets}, 0, 0.0
        for c in checkpoints:
            e0.record()
            it.render(f, c - done)
            e1.record()
            ctx.synchronize()
            frame_ms += e0.elapsed_ms(e1)
            done = c
            img = it.read_accumulation()[..., 0:3]
            plain[c] = T.rel_rmse(img, ref)
            if c <= 64:
                for k, dn in nets.items():
                    e0.record()
                    it.features(f, feat)
                    dn.infer(feat, 1, H, W, den)
                    e1.record()
                    dn.check()
                    dn_ms = e0.elapsed_ms(e1)
                    dnz[k][c] = T.rel_rmse(den.download((H, W, 4))[..., 0:3], ref)
        frame_ms /= checkpoints[-1]
        # inference alone (features excluded), warm
        dn = next(iter(nets.values()))
        for _ in range(3):
            dn.infer(feat, 1, H, W, den)
        e0.record()
        for _ in range(10):
            dn.infer(feat, 1, H, W, den)
        e1.record()
        ctx.synchronize()
        infer_ms = e0.elapsed_ms(e1) / 10
        e256 = plain[256]
        t_plain = 256 * frame_ms_plain
        res = {"seed": seed, "ref_spp": args.dn_ref_spp, "frame_ms_plain": frame_ms_plain,
               "frame_ms_with_aov": frame_ms, "features_plus_infer_ms": dn_ms, "infer_ms": infer_ms,
               "rel_rmse_plain": plain}
        # plain spp reaching a given error: log-log interpolation of the
        # measured curve, extrapolated past 256 spp with its last slope
        cs = sorted(plain)
        lx, ly = np.log([float(c) for c in cs]), np.log(np.maximum([plain[c] for c in cs], 1e-30))

        def plain_spp_for(err):
            le = np.log(err)
            for j in range(len(cs) - 1):
                if ly[j] >= le >= ly[j + 1] and ly[j] > ly[j + 1]:
                    return float(np.exp(lx[j] + (le - ly[j]) * (lx[j + 1] - lx[j]) / (ly[j + 1] - ly[j])))
            if le > ly[0]:
                return float(cs[0])
            slope = (ly[-1] - ly[-2]) / (lx[-1] - lx[-2])
            return float(np.exp(lx[-1] + (le - ly[-1]) / slope))

        for k in nets:
            ok = [c for c in sorted(dnz[k]) if dnz[k][c] <= e256]
            s_star = ok[0] if ok else None
            t_den = (s_star * frame_ms + dn_ms) if s_star else None
            eq = {c: plain_spp_for(e) for c, e in dnz[k].items()}
            res[k] = {"rel_rmse_denoised": dnz[k], "denoised_spp_reaching_plain_256": s_star,
                      "speedup_vs_plain_256": (t_plain / t_den) if t_den else None,
                      "plain_spp_at_equal_rmse": eq,
                      "speedup_at_equal_rmse": {c: eq[c] * frame_ms_plain / (c * frame_ms + dn_ms) for c in eq}}
        evals.append(res)
        it.close()
        sc.close()
    flops = hx.denoiser_conv_flops_per_pixel() * W * ((H + 15) // 16 * 16)
    infer_ms = statistics.median(e["infer_ms"] for e in evals)
    out["eval"] = evals
    out["roofline"] = {"bound": "tensor", "kernel": "k_conv_halo (forward, all 13 layers)",
                       "achieved": flops / (infer_ms * 1e-3) / 1e12, "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                       "frac": flops / (infer_ms * 1e-3) / 1e12 / peaks["bf16_tflops"],
                       "flops_per_1080p_inference": flops, "peak_source": peaks["source"] + ", bf16 burst"}
    best = None
    for k in nets:
        speed = [e[k]["speedup_vs_plain_256"] for e in evals if e[k]["speedup_vs_plain_256"]]
        v = min(speed) if len(speed) == len(evals) else None
        out.setdefault("value_by_loss", {})[k] = v
        if v is not None and (best is None or v > best):
            best = v
    out["value"] = best
    out["unit"] = "x (plain 256-spp time / denoised time at equal or lower RMSE)"
    feat.close()
    den.close()
    for dn in nets.values():
        dn.close()
    print(json.dumps(out), flush=True)


def run_denoise_kernels(args, dist):
    """The denoiser's kernels alone, on seeded random inputs and a network from
    the library's initialiser: CUDA-event time of a 1080p inference and of a
    training step on 16 x 256^2 crops, with the convolutions' FLOP rates."""
    import numpy as np
    import helios_gb300 as hx
    ctx = hx.Context(dist.local)
    dn = hx.Denoiser(ctx)
    dn.init_params(3)
    rng = np.random.default_rng(1)
    feats = np.zeros((1, HEIGHT, WIDTH, 12), np.float32)
    feats[..., 0:3] = rng.exponential(0.5, (1, HEIGHT, WIDTH, 3))
    feats[..., 4:7] = rng.uniform(0, 1, (1, HEIGHT, WIDTH, 3))
    feats[..., 8:11] = 0.577
    fb = hx.DeviceBuffer(ctx, feats.nbytes)
    fb.upload(feats)
    ob = hx.DeviceBuffer(ctx, HEIGHT * WIDTH * 16)
    n, h, w = 16, 256, 256
    f2 = np.zeros((n, h, w, 12), np.float32)
    f2[..., 0:3] = rng.exponential(0.5, (n, h, w, 3))
    f2[..., 4:7] = 0.5
    f2[..., 8:11] = 0.577
    fb2 = hx.DeviceBuffer(ctx, f2.nbytes)
    fb2.upload(f2)
    tb2 = hx.DeviceBuffer(ctx, n * h * w * 16)
    tb2.upload(np.ones((n, h, w, 4), np.float32))
    e0, e1 = hx.Event(ctx), hx.Event(ctx)
    out = {"mode": "denoise-kernels", "n_gpus": 1, "data": "synthetic (seeded random features; random network)"}
    for name, run, flops in (
            ("inference_1080p", lambda: dn.infer(fb, 1, HEIGHT, WIDTH, ob),
             hx.denoiser_conv_flops_per_pixel() * WIDTH * ((HEIGHT + 15) // 16 * 16)),
            ("train_step_16x256x256", lambda: dn.train_step(fb2, tb2, n, h, w, 1e-4, want_loss=False),
             3 * hx.denoiser_conv_flops_per_pixel() * n * h * w)):
        for _ in range(3):
            run()
        dn.check()
        ctx.synchronize()
        e0.record()
        for _ in range(max(1, args.dn_iters)):
            run()
        e1.record()
        ms = e0.elapsed_ms(e1) / max(1, args.dn_iters)
        dn.check()
        out[name] = {"ms": ms, "conv_tflops": flops / ms / 1e9}
    print(json.dumps(out))


def main():
    args = parse()
    dist = Dist()
    try:
        if args.denoise_kernels:
            if dist.rank == 0:
                run_denoise_kernels(args, dist)
        elif args.denoise:
            if dist.rank == 0:
                run_denoise(args, dist)
        elif args.precision:
            if dist.rank == 0:
                run_precision(args, dist)
        elif args.serving:
            if dist.rank == 0:
                run_serving(args, dist)
        elif args.impl == "reference":
            run_reference(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
