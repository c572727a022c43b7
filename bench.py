#!/usr/bin/env python
"""Benchmark of the GB300 triangle rasteriser + deferred shading path.

Workload (default `soup1080`): one 1920x1080 frame of a seeded 1,000,000-face
PBR triangle soup with per-face roughness / metallic / albedo and 8 point
lamps, smoothing on, culling and clipping on, ACES tonemap -- the
"triangle-soup stress" configuration.  `sphere512` is the 512x512 Lambert UV
sphere.

A step renders one frame (Scene.render's t3_render sequence: scene upload, key
clear, rasteriser, shading) replayed from a CUDA graph, with all inputs
resident on the device.  Between steps the L2 is flushed by writing a 256 MB
buffer outside the per-step CUDA events; `value` = faces submitted per second
(Mtri/s, all ranks).  `e2e` renders a stream of the same frame through the
public API (FramePipeline: three scene replicas on three streams), every frame
copying its face arrays in from pinned host memory and scene.img back out;
`e2e.serial` does one frame at a time with a synchronise after each.

--impl reference times the CPU implementation of the same path: the reference
(Python on Taichi) cannot run here, so its restatement in oracle/ runs in its
OpenMP mode on all host cores.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mtri/s & 1080p frames/s vs Taichi-CPU; MLP-IBL vs MC-IBL fps at ΔE2000<1"
L2_FLUSH_BYTES = 256 << 20


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="soup1080", choices=["soup1080", "sphere512", "ibl1080"])
    p.add_argument("--raster", default="direct", choices=["direct", "binned"])
    p.add_argument("--e2e-steps", type=int, default=10)
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="skip every extra section (same as --extras '')")
    p.add_argument("--extras", default=",".join(EXTRAS),
                   help="comma-separated extra sections to run after the headline frame: "
                        + ", ".join(EXTRAS))
    a = p.parse_args()
    a.extras = [] if a.no_extras else [x for x in a.extras.split(",") if x]
    bad = [x for x in a.extras if x not in EXTRAS]
    if bad:
        p.error(f"unknown extra sections {bad}")
    return a


# extra sections of the JSON line, each a workload of its own with its roofline
EXTRAS = ("sphere512", "binned", "learned_ibl", "batch", "anim_grid")


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def tc_peak():
    """Dense BF16 TFLOP/s (burst: the shading kernel is timed alone)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"])
    except Exception:
        return 1900.0


def build_workload(name, seed, raster):
    import taichi_three_gb300 as tina
    if name == "soup1080":
        scene, mesh = tina.workloads.soup_scene(ntri=1_000_000, res=(1920, 1080), seed=seed,
                                                raster=raster)
        cfg = {"workload": "triangle soup 1920x1080, 1,000,000 faces, PBR per-face, 8 point lamps",
               "faces": 1_000_000, "width": 1920, "height": 1080}
    elif name == "ibl1080":
        # the soup lit by the learned IBL term; an untrained network costs the
        # same as a trained one, so this profiles the fused network shading pass
        net = tina.IBLNet(seed=seed)
        scene, mesh = tina.workloads.ibl_soup_scene(ntri=1_000_000, res=(1920, 1080), seed=seed,
                                                    mode="mlp", mlp=net, raster=raster)
        scene._bench_net = net
        cfg = {"workload": "triangle soup 1920x1080, 1,000,000 faces, PBR per-face, learned IBL "
                           "(fused tcgen05 network shading)",
               "faces": 1_000_000, "width": 1920, "height": 1080}
    else:
        scene, mesh = tina.workloads.sphere_scene(512, raster=raster)
        cfg = {"workload": "UV sphere 512x512, 3,968 faces, Lambert, 1 directional lamp",
               "faces": mesh.get_nfaces(), "width": 512, "height": 512}
    return scene, mesh, cfg


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 100 ms in the background."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return time.time()

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        rows = []
        try:
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
            os.unlink(self.path)
        except Exception:
            pass
        return rows

    @staticmethod
    def summarize(rows):
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons, "samples": len(rows)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    elif torch.cuda.is_available():
        torch.cuda.set_device(local)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x, world):
    """Max over ranks (replicas only: the sole cross-rank exchange)."""
    from taichi_three_gb300 import replicas
    return replicas.max_over_ranks(x) if world > 1 else x


def graph_of(fn):
    """fn() captured into a CUDA graph (after two eager warm-up calls)."""
    fn()
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        fn()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side):
            fn()
    torch.cuda.synchronize()
    return g


def time_graph(g, reps, flush=None):
    """Median ms of g.replay() between CUDA events (L2 flushed before each)."""
    times = []
    for i in range(reps):
        if flush is not None:
            flush.fill_(float(i))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        g.replay()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    return statistics.median(times)


def direct_launches(scene):
    """Kernels of one direct-mode t3_render: the clear; per object the vertex
    stage (grids and indexed meshes), then the raster and the large-face pass
    (one kernel for particles and lines); the shading kernel."""
    from taichi_three_gb300 import _native as N
    sc, keep = scene.describe()
    n = 1
    for o in range(sc.nobjects):
        m = sc.objects[o].mesh
        if m.kind == N.T3_MESH_PARTICLES or m.kind == N.T3_MESH_LINES or (m.flags & N.T3_MESH_WIREFRAME):
            n += 1
            continue
        if m.kind in (N.T3_MESH_GRID, N.T3_MESH_INDEXED):
            n += 1
        n += 2
    return n + 1


def stage_times(scene, reps=10, split_shade=False):
    """Median ms of the stages of t3_render_staged_n for the scene's current
    state (upload+clear | raster | shade); split_shade (learned IBL) also
    times the shading's row prepass and network kernel apart."""
    from taichi_three_gb300 import _native as N
    lib = N.load()
    scene.render()
    sc, keep = scene.describe()
    outs = N.t3_outputs(scene.image.data_ptr(), scene.face_id.data_ptr(),
                        scene.engine.depth.data_ptr(), scene.depth_f.data_ptr())
    evs = [C.c_void_p() for _ in range(5)]
    for e in evs:
        N.check(lib.t3_event_create(C.byref(e)), "t3_event_create")
    arr = (C.c_void_p * 5)(*[e.value for e in evs])
    spans = {"clear": (0, 1), "raster": (1, 2), "shade": (2, 4)}
    if split_shade:
        spans.update({"shade_rows": (2, 3), "shade_net": (3, 4)})
    st = {k: [] for k in spans}
    mode = N.T3_RASTER_DIRECT if scene.raster_mode == "direct" else N.T3_RASTER_BINNED
    for _ in range(reps):
        N.check(lib.t3_render_staged_n(C.byref(sc), mode, scene.tile, scene.bin_capacity,
                                       scene._ws.data_ptr(), scene._ws.numel(),
                                       scene._status.data_ptr(), C.byref(outs),
                                       torch.cuda.current_stream().cuda_stream, arr, 5), "staged")
        ms = C.c_float()
        for name, (a, b) in spans.items():
            N.check(lib.t3_event_elapsed_ms(evs[a], evs[b], C.byref(ms)), "elapsed")
            st[name].append(ms.value)
    for e in evs:
        lib.t3_event_destroy(e)
    return {k: statistics.median(v) for k, v in st.items()}


# FLOPs of one network evaluation counted on the real inputs and outputs:
# 2 * (386 * 64 + 64 * 64 + 64 * 64 + 64 * 9) (the 400-wide input and 16-wide
# output rows are padding for the MMA shapes)
MLP_FLOP_PER_PIXEL = 2 * (386 * 64 + 64 * 64 + 64 * 64 + 64 * 9)


def bench_learned_ibl(flush, tc_peak):
    """1080p soup lit by the procedural sky: the network frame against the
    256-sample Monte Carlo frame (fps, dE2000 against the FP64 oracle)."""
    import taichi_three_gb300 as tina
    from oracle import oracle
    sky = tina.Skybox(tina.procedural_sky(512, seed=0))
    t0 = time.time()
    net, losses = tina.train_for_skybox(sky, samples=1 << 24, spp=4096, steps=12000, batch=32768)
    torch.cuda.synchronize()
    train_s = time.time() - t0
    res = {}
    for key, mode, spp in (("mlp", "mlp", 1), ("mc256", "mc", 256)):
        scene, _ = tina.workloads.ibl_soup_scene(skybox=sky, mode=mode, spp=spp, mlp=net)
        g = graph_of(scene.render)
        ms = time_graph(g, 20 if mode == "mlp" else 5, flush)
        stages = stage_times(scene, 5, split_shade=mode == "mlp")
        res[key] = (ms, scene.img.cpu().numpy().reshape(-1, 3), scene, stages)
    scene = res["mlp"][2]
    fid = scene.face_id.cpu().numpy().ravel()
    cov = np.argwhere(fid >= 0).ravel()
    pick = np.sort(np.random.default_rng(0).choice(cov, 4000, replace=False))
    _, truth = oracle.pixels_f64(scene, pick, spp=4096, seed=12345)
    de = {k: float(tina.colour.delta_e2000(v[1][pick], truth).mean()) for k, v in res.items()}
    shade_ms = res["mlp"][3]["shade"]
    net_ms = res["mlp"][3]["shade_net"]
    flop = MLP_FLOP_PER_PIXEL * len(cov)
    return {"workload": "1920x1080 soup, 1,000,000 faces, PBR per-face, lit only by a 1024x512 "
                        "FP16 procedural sky (gradient + 12 Gaussian lobes)",
            "mlp_ms_per_frame": res["mlp"][0], "mc256_ms_per_frame": res["mc256"][0],
            "mlp_fps": 1e3 / res["mlp"][0], "mc256_fps": 1e3 / res["mc256"][0],
            "speedup": res["mc256"][0] / res["mlp"][0],
            "dE2000_mean_mlp": de["mlp"], "dE2000_mean_mc256": de["mc256"],
            "dE2000_reference": "FP64 oracle, 4096 samples/pixel, 4000 random covered pixels",
            "train_s": train_s, "train": "16M samples, 4096-sample MC targets, 12000 Adam steps of 32768",
            "mlp_shade_ms": shade_ms, "mlp_net_kernel_ms": net_ms,
            "roofline_mlp": {"bound": "tensor", "kernel": "k_mlp_net", "achieved": flop / (net_ms / 1e3) / 1e12,
                             "peak": tc_peak, "unit": "TFLOP/s",
                             "frac": flop / (net_ms / 1e3) / 1e12 / tc_peak,
                             "flop_per_pixel": MLP_FLOP_PER_PIXEL, "pixels": int(len(cov)),
                             "traffic": traffic_of("ibl1080", "mlp_net")},
            "roofline_mlp_shading": {"bound": "tensor", "kernels": "k_mlp_rows + k_mlp_net",
                                     "achieved": flop / (shade_ms / 1e3) / 1e12, "peak": tc_peak,
                                     "unit": "TFLOP/s", "frac": flop / (shade_ms / 1e3) / 1e12 / tc_peak},
            "stages_ms": {k: v[3] for k, v in res.items()}}, sky, net


def traffic_of(section, kernel):
    """ncu DRAM bytes (read + write) per launch of `kernel` in `section`, from
    profiles/traffic.json (null when not captured)."""
    try:
        return json.load(open(os.path.join(ROOT, "profiles", "traffic.json"))).get(section, {}).get(kernel)
    except Exception:
        return None


def hbm_roofline(alg_bytes, ms, peak, peak_kind, what, traffic=None):
    achieved = alg_bytes / (ms / 1e3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "alg_bytes": alg_bytes, "of": what, "peak_source": peak_kind}


def bench_sphere(flush, peak):
    """512x512 Lambert UV sphere (3,968 faces): launch-bound, a few microseconds."""
    import taichi_three_gb300 as tina
    scene, mesh = tina.workloads.sphere_scene(512)
    ms = time_graph(graph_of(scene.render), 50, flush)
    stages = stage_times(scene, 20)
    T, P = mesh.get_nfaces(), 512 * 512
    alg = 72 * T + 36 * P
    return {"workload": "UV sphere 512x512 (64 lon x 32 lat: 3,968 faces), Diffuse(0.8), 1 directional lamp",
            "faces": T, "ms_per_frame": ms, "fps": 1e3 / ms, "mtri_s": T / ms / 1e3,
            "mpix_s": P / ms / 1e3, "stage_ms": stages,
            "roofline": hbm_roofline(alg, ms, peak[0], peak[1], "whole frame: 72 B/face + 36 B/px")}


def bench_binned(flush, peak):
    """The headline soup frame through the binned tile rasteriser (tile 16,
    automatic bin capacity): upload, bin, tile (raster + shade in shared memory)."""
    import taichi_three_gb300 as tina
    scene, mesh = tina.workloads.soup_scene(ntri=1_000_000, res=(1920, 1080), seed=0, raster="binned")
    scene.render()  # settles the bin capacity (re-renders once if a bin overflowed)
    scene.check_bins = False
    ms = time_graph(graph_of(scene.render), 20, flush)
    stages = stage_times(scene, 10)
    stages = dict(zip(("upload", "bin", "tile"), (stages["clear"], stages["raster"], stages["shade"])))
    T, P = 1_000_000, 1920 * 1080
    fid = scene.face_id
    visible = int(torch.unique(fid[fid >= 0]).numel())
    alg_bin, alg_tile = 36 * T, 24 * P + visible * (36 + 36 + 20)
    frame = 92 * T + 20 * P
    return {"workload": "triangle soup 1920x1080, 1,000,000 faces, PBR per-face, 8 point lamps; binned, tile 16",
            "bin_capacity": scene.bin_capacity, "ms_per_frame": ms, "mtri_s": T / ms / 1e3,
            "stage_ms": stages,
            "roofline": hbm_roofline(alg_tile, stages["tile"], peak[0], peak[1],
                                     "k_tile: 24 B/px outputs + 92 B per visible face",
                                     traffic_of("binned", "tile")),
            "roofline_bin": hbm_roofline(alg_bin, stages["bin"], peak[0], peak[1], "k_bin: 36 B/face",
                                         traffic_of("binned", "bin")),
            "frame_roofline": hbm_roofline(frame, ms, peak[0], peak[1],
                                           "whole frame: 92 B/face + 20 B/px (keys stay on chip)")}


def bench_batch(flush, peak):
    """64 views (1e3..2e6 faces, 256..1024 px square, Classic + 8 lamps) in two
    launches over all views (the autotuner's pick of the direct work-item
    sizes and the binned tile size / threads / bin capacity), against the same
    frames rendered one scene at a time (both captured as CUDA graphs)."""
    import taichi_three_gb300 as tina
    from taichi_three_gb300.autotune import Autotuner
    scenes = tina.workloads.batch_scenes(64, seed=0)
    faces = sum(list(s.objects)[0].get_nfaces() for s in scenes)
    pix = sum(s.res[0] * s.res[1] for s in scenes)

    def seq():
        for s in scenes:
            s.render()
    ms_seq = time_graph(graph_of(seq), 5, flush)
    b = tina.BatchRenderer(scenes)
    tuner = Autotuner(timer=lambda fn: time_graph(graph_of(fn), 3))
    cfg, _ = b.autotune(tuner=tuner, repeats=1)
    ms = time_graph(graph_of(lambda: b.render(cfg, check_bins=False)), 10, flush)
    status = b.status()
    # every candidate the tuner timed (binned ones whose bins overflowed are not)
    sweep = {"/".join(f"{k}={v}" for k, v in c.items()): round(t, 4) for c, t in tuner.log}
    # positions + normals read once, the 3 albedo channels Classic reads, 36 B/px
    alg = (72 + 12) * faces + 36 * pix
    return {"workload": "64 views: soups of round(exp(U[ln 1e3, ln 2e6])) faces, square "
                        "256/512/768/1024 px, cameras on the radius-3 sphere, Classic, 8 lamps",
            "faces": faces, "pixels": pix, "ms_per_batch": ms, "mtri_s": faces / ms / 1e3,
            "mpix_s": pix / ms / 1e3, "views_per_s": 64e3 / ms, "per_scene_graph_ms": ms_seq,
            "speedup_vs_per_scene": ms_seq / ms, "autotuned": cfg, "status": status, "sweep_ms": sweep,
            "roofline": hbm_roofline(alg, ms, peak[0], peak[1],
                                     "whole batch: 84 B/face + 36 B/px summed over the views",
                                     {k: traffic_of("batch", k) for k in ("raster", "shade")})}


def bench_anim_grid(sky, net, flush, peak, tcp):
    """3840x2160, MeshGrid(2048) displaced per frame, PBR + learned IBL + 2
    lamps, 120 frames in one CUDA graph.  Without a trained network (the
    section run alone) an untrained one of the same shape stands in: the
    work per frame is the same."""
    import taichi_three_gb300 as tina
    if net is None:
        sky = tina.Skybox(tina.procedural_sky(512, seed=0))
        net = tina.IBLNet(seed=0)
    scene, grid = tina.workloads.wave_grid_scene(skybox=sky, mlp=net)
    fg = tina.FrameGraph(scene, 120, update=lambda k: grid.displace_wave(k / 30.0)).capture()
    ms = time_graph(fg.graph, 3, flush)
    # the same frames through the binned tiles (16-pixel tiles; bins sized by a
    # first eager frame), for the raster-mode comparison
    bscene, bgrid = tina.workloads.wave_grid_scene(skybox=sky, mlp=net, raster="binned", tile=16)
    bscene.render()
    bfg = tina.FrameGraph(bscene, 120, update=lambda k: bgrid.displace_wave(k / 30.0)).capture()
    binned_ms = time_graph(bfg.graph, 3, flush)
    binned_status = bscene.status()
    del bfg, bscene, bgrid
    T = grid.get_nfaces()
    V, P = grid.res[0] * grid.res[1], scene.res[0] * scene.res[1]
    cov = float((scene.face_id >= 0).float().mean())
    frame_ms = ms / 120
    alg = 48 * V + 36 * P                     # vertex stage out + back in, 36 B/px
    flop = MLP_FLOP_PER_PIXEL * cov * P       # the network on every covered pixel
    hbm = hbm_roofline(alg, frame_ms, peak[0], peak[1], "per frame: 48 B/vertex + 36 B/px")
    tc = {"bound": "tensor", "achieved": flop / (frame_ms / 1e3) / 1e12, "peak": tcp,
          "unit": "TFLOP/s", "flop": flop}
    tc["frac"] = tc["achieved"] / tcp
    return {"workload": "3840x2160, MeshGrid(2048) (8,380,418 faces), z = 0.1 sin(8x+t) cos(8y+1.3t) "
                        "per frame, PBR + learned IBL + 2 point lamps, 120 frames in one CUDA graph",
            "ms_per_120_frames": ms, "ms_per_frame": frame_ms, "fps": 120e3 / ms,
            "binned_ms_per_frame": binned_ms / 120, "binned_status": binned_status,
            "mtri_s": T * 120 / ms / 1e3, "coverage": cov, "status": scene.status(),
            "roofline": hbm if hbm["frac"] >= tc["frac"] else tc, "roofline_hbm": hbm,
            "roofline_tensor": tc,
            "traffic": {k: traffic_of("anim_grid", k) for k in ("grid_wave", "grid_normals", "vertex_ndc")}}


def cpu_baseline(scene, faces, seconds, label):
    """The oracle's OpenMP mode on all host threads over whole frames."""
    from oracle import oracle
    oracle.load()
    sc, keep = scene.describe("cpu")
    threads = os.cpu_count() or 1
    oracle.render_desc(sc, mode=1, nthreads=threads, want_depth_f=False)  # warm
    times = []
    t_end = time.time() + seconds
    while True:
        t0 = time.perf_counter()
        oracle.render_desc(sc, mode=1, nthreads=threads, want_depth_f=False)
        times.append(time.perf_counter() - t0)
        if time.time() > t_end or len(times) >= 50:
            break
    t = statistics.median(times)
    return {"value": faces / t / 1e6, "unit": "Mtri/s", "cores": threads, "kind": "port",
            "sample": f"{len(times)} whole frames of the {label} (median frame {t * 1e3:.1f} ms)",
            "fps": 1.0 / t}


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import taichi_three_gb300 as tina  # noqa: F401  (scene construction only)
    scene, mesh, cfg = build_workload(args.workload, 0, "direct")
    faces = cfg["faces"]
    from oracle import oracle
    oracle.load()
    sc, keep = scene.describe("cpu")
    threads = os.cpu_count() or 1
    for _ in range(max(1, min(args.warmup, 3))):
        oracle.render_desc(sc, mode=1, nthreads=threads, want_depth_f=False)
    times = []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.render_desc(sc, mode=1, nthreads=threads, want_depth_f=False)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_all > args.cpu_seconds * 2:
            break
    t = sum(times) / len(times)
    value = faces / t / 1e6
    line = {"metric": METRIC, "impl": "reference", "value": value, "unit": "Mtri/s",
            "n_gpus": args.gpus, "steps": len(times), "warmup": args.warmup,
            "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "config": cfg,
            "setup": {"parallelism": "replicas only (rank 0 runs)", "l2": "n/a (CPU)",
                      "threads": threads},
            "fps": 1.0 / t,
            "cpu_baseline": {"value": value, "unit": "Mtri/s", "cores": threads, "kind": "port",
                             "sample": f"{len(times)} whole frames; the reference's Taichi CPU "
                                       "backend is not installable here, so its C++ restatement "
                                       "(oracle/, OpenMP) runs in its place"},
            "e2e": {"value": value, "unit": "Mtri/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    world, rank, local = dist_setup(args)
    import taichi_three_gb300 as tina
    from taichi_three_gb300 import _native as N
    lib = N.load()
    dev = torch.device("cuda", local)
    scene, mesh, cfg = build_workload(args.workload, rank, args.raster)
    faces = cfg["faces"]
    W, H = scene.res

    # one eager frame allocates the outputs and workspace
    scene.render()
    torch.cuda.synchronize()
    sc, keep = scene.describe(dev)
    mode = N.T3_RASTER_DIRECT if args.raster == "direct" else N.T3_RASTER_BINNED
    outs = N.t3_outputs(scene.image.data_ptr(), scene.face_id.data_ptr(),
                        scene.engine.depth.data_ptr(), scene.depth_f.data_ptr())
    ws, status = scene._ws, scene._status

    def frame(stream, events=None):
        if events is None:
            rc = lib.t3_render(C.byref(sc), mode, scene.tile, scene.bin_capacity, ws.data_ptr(),
                               ws.numel(), status.data_ptr(), C.byref(outs), stream)
        else:
            rc = lib.t3_render_staged(C.byref(sc), mode, scene.tile, scene.bin_capacity,
                                      ws.data_ptr(), ws.numel(), status.data_ptr(), C.byref(outs),
                                      stream, events)
        N.check(rc, "t3_render")

    # capture the frame into a CUDA graph
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        frame(side.cuda_stream)
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    with torch.cuda.graph(graph):
        frame(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    if args.raster == "direct":
        kernels_per_frame = direct_launches(scene)
        stage_names = ("clear", "raster", "shade")
    else:                        # upload, bin x objects, tile (raster + shade)
        kernels_per_frame = 1 + len(scene.objects) + 1
        stage_names = ("upload", "bin", "tile")

    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    for i in range(args.warmup):
        flush.fill_(float(i))
        graph.replay()
    torch.cuda.synchronize()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.25)
    barrier(world)
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    for i in range(args.steps):
        flush.fill_(float(i))
        starts[i].record()
        graph.replay()
        ends[i].record()
    torch.cuda.synchronize()
    barrier(world)
    wall = time.perf_counter() - t_wall
    if wall < 1.0:  # keep sampling under the same load for at least a second
        t_soak = time.perf_counter()
        while time.perf_counter() - t_soak < 1.0 - wall:
            for _ in range(50):
                flush.fill_(0.0)
                graph.replay()
            torch.cuda.synchronize()
    rows = sampler.stop()
    clocks = ClockSampler.summarize(rows)
    clocks["window"] = "timed steps" + (" + 1 s soak of the same frames" if wall < 1.0 else "")
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = allmax(sum(step_ms), world)
    ms_per_step = total_ms / args.steps
    value = world * faces * args.steps / (total_ms / 1e3) / 1e6

    # per-stage timing of eager frames (events between the stages on the launch stream)
    evs = [C.c_void_p() for _ in range(4)]
    for e in evs:
        N.check(lib.t3_event_create(C.byref(e)), "t3_event_create")
    ev_arr = (C.c_void_p * 4)(*[e.value for e in evs])
    stage = {k: [] for k in stage_names}
    stream = torch.cuda.current_stream().cuda_stream
    for i in range(20):
        flush.fill_(float(i))
        frame(stream, ev_arr)
        ms = C.c_float()
        for name, (a, b) in zip(stage, ((0, 1), (1, 2), (2, 3))):
            N.check(lib.t3_event_elapsed_ms(evs[a], evs[b], C.byref(ms)), "elapsed")
            stage[name].append(ms.value)
    stage_ms = {k: statistics.median(v) for k, v in stage.items()}
    for e in evs:
        lib.t3_event_destroy(e)

    # algorithmic bytes per launch: every input byte the stage must read and
    # every output byte it must write once, nothing for re-reads
    P = W * H
    fid = scene.face_id
    visible = int(torch.unique(fid[fid >= 0]).numel())
    attr_b = 4 * (mesh.face_attr.shape[1] if mesh.face_attr is not None else 0)
    out_b = (12 + 4 + 4 + 4) * P  # rgb, face id, depth, depth_f written once
    alg = {
        "clear": 8 * P,
        "raster": 36 * faces,
        "shade": 8 * P + out_b + visible * (36 + 36 + attr_b),
        "upload": 0,
        "bin": 36 * faces,
        "tile": out_b + visible * (36 + 36 + attr_b),
    }
    dominant = max(stage_ms, key=lambda k: stage_ms[k])
    peak, peak_kind = peaks()
    achieved = alg[dominant] / (stage_ms[dominant] / 1e3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get(args.workload, {}).get(dominant)
        except Exception:
            traffic = None
    frame_bytes = (72 + attr_b) * faces + 36 * P
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "kernel": dominant,
                "peak_source": peak_kind, "stage_ms": stage_ms, "alg_bytes": alg[dominant],
                "frame_alg_bytes": frame_bytes,
                "frame_frac": frame_bytes / (ms_per_step / 1e3) / 1e9 / peak}

    # atomic work: depth reductions per frame against the measured u64
    # atomicMin rate on distinct L2-resident addresses
    atomics = None
    if args.raster == "direct":
        nfrag = C.c_int64()
        N.check(lib.t3_raster_fragments(C.byref(sc), ws.data_ptr(), ws.numel(), C.byref(nfrag),
                                        torch.cuda.current_stream().cuda_stream), "t3_raster_fragments")
        probe_n, rounds = 1 << 22, 16  # 32 MB of keys, L2 resident
        probe = torch.empty(probe_n, dtype=torch.int64, device=dev)
        rates = []
        for i in range(6):
            probe.fill_(-1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            N.check(lib.t3_red_min_rate(probe.data_ptr(), probe_n, rounds,
                                        torch.cuda.current_stream().cuda_stream), "t3_red_min_rate")
            e1.record()
            torch.cuda.synchronize()
            if i:
                rates.append(probe_n * rounds / (e0.elapsed_time(e1) / 1e3) / 1e9)
        peak_red = max(rates)
        frag_rate = nfrag.value / (stage_ms["raster"] / 1e3) / 1e9
        atomics = {"fragments_per_frame": nfrag.value, "rate": frag_rate, "peak": peak_red,
                   "unit": "G reductions/s", "frac": frag_rate / peak_red,
                   "probe": f"u64 atomicMin, {probe_n} distinct L2-resident addresses x {rounds} rounds, "
                            "best of 5 (CUDA events)"}
        del probe

    # end to end through the public API: pinned host arrays in, scene.img out
    verts_h = mesh.verts.cpu().pin_memory()
    norms_h = mesh.norms.cpu().pin_memory()
    attrs_h = mesh.face_attr.cpu().pin_memory() if mesh.face_attr is not None else None
    img_h = torch.empty((W, H, 3), dtype=torch.float32).pin_memory()
    h2d = verts_h.numel() * 4 + norms_h.numel() * 4 + (attrs_h.numel() * 4 if attrs_h is not None else 0)
    d2h = img_h.numel() * 4

    def upload(m):
        m.set_face_verts(verts_h)
        m.set_face_norms(norms_h)
        if attrs_h is not None:
            m.set_face_attrs(attrs_h)

    # one frame at a time: upload, render, read back, synchronise
    e2e_times = []
    for i in range(args.e2e_steps + 2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        upload(mesh)
        scene.render()
        img_h.copy_(scene.img, non_blocking=True)
        torch.cuda.synchronize()
        if i >= 2:
            e2e_times.append(time.perf_counter() - t0)
    serial_t = allmax(statistics.median(e2e_times), world)
    # a stream of frames through FramePipeline: three scene replicas on three
    # streams, each frame's inputs copied in and its image copied out, frame
    # k+1's upload overlapping frame k's render and read-back
    replicas = [(scene, mesh)] + [build_workload(args.workload, rank, args.raster)[:2] for _ in range(2)]
    meshes = {id(s): m for s, m in replicas}
    pipe = tina.FramePipeline([s for s, _ in replicas])
    for i in range(6):
        pipe.submit(lambda sc: upload(meshes[id(sc)]))
    pipe.synchronize()
    nframes = max(4 * args.e2e_steps, 12)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(nframes):
        pipe.submit(lambda sc: upload(meshes[id(sc)]))
    pipe.synchronize()
    pipe_t = allmax((time.perf_counter() - t0) / nframes, world)
    del pipe, replicas, meshes
    e2e = {"value": world * faces / pipe_t / 1e6, "unit": "Mtri/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "ms_per_step": pipe_t * 1e3,
           "method": f"FramePipeline, 3 scene replicas on 3 streams, {nframes} frames, host clock "
                     "around the whole run; every frame uploads its face arrays from pinned host "
                     "memory and reads scene.img back",
           "serial": {"value": world * faces / serial_t / 1e6, "ms_per_step": serial_t * 1e3,
                      "method": "one frame at a time, synchronised (median of steps)"}}

    line = {"metric": METRIC, "value": value, "unit": "Mtri/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": cfg,
            "setup": {"raster": args.raster, "parallelism": f"replicas x{world}",
                      "l2": "flushed between steps (256 MB write outside the per-step events)",
                      "graph": "one CUDA graph per frame"},
            "fps": world * 1e3 / ms_per_step, "mpix_s": world * P / (ms_per_step / 1e3) / 1e6,
            "gpu_launches": kernels_per_frame * args.steps, "e2e": e2e, "roofline": roofline,
            "atomics": atomics,
            "clocks": clocks, "wall_s_timed": wall}
    if rank == 0 and not args.no_cpu_baseline and args.workload != "ibl1080":
        line["cpu_baseline"] = cpu_baseline(scene, faces, args.cpu_seconds, cfg["workload"])
    if rank == 0 and world == 1 and args.extras:
        del scene, mesh, ws, status
        pk = peaks()
        sky = net = None
        for name in EXTRAS:
            if name not in args.extras:
                continue
            torch.cuda.empty_cache()
            if name == "sphere512":
                line["sphere512"] = bench_sphere(flush, pk)
            elif name == "binned":
                line["binned"] = bench_binned(flush, pk)
            elif name == "learned_ibl":
                line["learned_ibl"], sky, net = bench_learned_ibl(flush, tc_peak())
            elif name == "batch":
                line["batch"] = bench_batch(flush, pk)
            elif name == "anim_grid":
                line["anim_grid"] = bench_anim_grid(sky, net, flush, pk, tc_peak())
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
