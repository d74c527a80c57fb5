#!/usr/bin/env python
"""Benchmark: path segments/s of the GB300 path tracer at 1920x1080.

One step = one full frame of the default-quality workload (c2_default:
1920x1080, 1024 samples per pixel, at most 12 bounces, 64 spheres + 16 cubes
+ the ground cube, brute-force closest hit), rendered from a cleared
accumulator with a fresh seed.  A segment is one trace_ray call of the
reference (src/renderer/cpu.rs:257); the kernel counts them exactly.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`ours` prints one JSON line: `value` is segments/s with the scene and
accumulator resident on the device (the timed region is bracketed by
barrier + synchronize; the 256 MiB L2-flush write between steps is inside
it), `e2e` is the same metric through the C ABI from host buffers (scene
upload, reset, render, 8-bit read-back every step), `roofline` relates the
render kernel's CUDA-event time to the FP32 issue rate measured in the same
run, and `cpu_baseline` times the CPU oracle (single thread, like the
reference's serial pixel loop) on a bounded sample of the same workload.

`reference` times the CPU restatement of the reference renderer on all host
threads (the reference is Rust and cannot be built here), one 1-spp frame of
the same workload per step.

With N > 1 (torchrun), every rank renders the full workload with its own
seeds on its own GPU ("replicas", weak scaling); value = all ranks' segments
/ the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "path segments/s @1080p"
UNIT = "segments/s"


def _args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--spp", type=int, default=0, help="samples per pixel per step (default: the workload's 1024)")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU-baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-batch", action="store_true", help="skip the batched (config 3) measurement")
    p.add_argument("--batch-only", action="store_true", help="only the batched (config 3) measurement")
    p.add_argument("--no-large", action="store_true", help="skip the LBVH (config 5) measurement")
    p.add_argument("--large-only", default="", metavar="WxHxSPP",
                   help="only the LBVH (config 5) measurement, at WxHxSPP (e.g. 480x270x32; 0 = full size)")
    p.add_argument("--form", choices=("auto", "megakernel", "wavefront"), default="auto",
                   help="rdc_render's form in the LBVH measurement (rdc_set_render_form; default: auto)")
    p.add_argument("--no-adjoint", action="store_true", help="skip the adjoint (config 4) measurement")
    p.add_argument("--adjoint-only", action="store_true", help="only the adjoint (config 4) measurement")
    p.add_argument("--no-wavefront", action="store_true", help="skip the megakernel / wavefront A/B")
    p.add_argument("--no-refscene", action="store_true", help="skip the reference's benchmark.rscn at 3840x2160")
    p.add_argument("--no-progressive", action="store_true", help="skip the editor-style render_sample loop")
    p.add_argument("--wavefront-only", action="store_true", help="only the megakernel / wavefront A/B")
    p.add_argument("--inverse", action="store_true",
                   help="only the config 5 inverse-rendering run (200 Adam steps on 1000 albedos)")
    p.add_argument("--no-inverse", action="store_true", help="skip the config 5 inverse-rendering run")
    p.add_argument("--batch-spp-div", type=int, default=1, help="divide every batch item's spp (small profiling case)")
    return p.parse_args()


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def combine_replicas(dist, elapsed_s: float, segments: float, device: str):
    """Replicas only: every rank renders its own frames, with no exchange on
    the data path.  Whole-job figures are the slowest rank's time and the sum
    of all ranks' segments.  dist = None on one rank."""
    if dist is None:
        return float(elapsed_s), float(segments)
    import torch
    t = torch.tensor([float(elapsed_s)], dtype=torch.float64, device=device)
    s = torch.tensor([float(segments)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(s, op=dist.ReduceOp.SUM)
    return float(t.item()), float(s.item())


def _workload():
    from raydar_gb300 import scenegen
    return scenegen.c2_default()


def _config(w, spp):
    n = len(w.scene.objects)
    return {
        "workload": f"c2_default: {w.scene.width}x{w.scene.height}, {spp} spp per step, "
                    f"max {w.max_bounces} bounces, {n} objects (64 spheres + 16 cubes + ground), brute force",
        "resolution": [w.scene.width, w.scene.height],
        "spp_per_step": spp,
        "max_bounces": w.max_bounces,
        "objects": n,
        "scene_seed": 2,
        "l2": "scene and accumulator fit in L2; a 256 MiB buffer is written before every timed step to flush it",
    }


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str):
        self.gpu_id = gpu_id
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", self.gpu_id, f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self._t.join(timeout=2)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "power_w_max": max(power),
                "samples": len(sm), "reasons": sorted(reasons)}


# ------------------------------------------------------------ CPU baseline --
def cpu_baseline(w, seconds: float, gpu=None):
    """The oracle on one host thread over a random pixel sample of the same
    1080p workload (1 spp, 12 bounces), sized to about `seconds` of work.
    With `gpu` (a CudaRenderer holding the same scene), the last sample's
    pixels are compared with the GPU's render of the same seed and sample:
    the images are matched when they are bit-identical (RMSE 0)."""
    import numpy as np

    import oracle
    sc = w.scene.to_c()
    npix = w.scene.width * w.scene.height
    rng = np.random.default_rng(0)
    n = 2000
    seed = 7
    total_seg, total_t, total_px = 0, 0.0, 0
    while True:
        px = rng.choice(npix, n, replace=False).astype(np.uint32)
        t0 = time.perf_counter()
        acc, seg = oracle.render_pixels(sc, px, 0, 1, w.max_bounces, seed)
        dt = time.perf_counter() - t0
        total_seg += seg
        total_t += dt
        total_px += n
        if total_t >= seconds:
            break
        rate = max(n / max(dt, 1e-6), 1.0)
        n = int(min(npix, max(500, rate * (seconds - total_t) * 1.05)))
    out = {"value": total_seg / total_t, "unit": UNIT, "cores": 1, "kind": "port",
           "sample": f"{total_px} random pixels of the 1920x1080 c2_default frame, 1 spp, "
                     f"{w.max_bounces} bounces, {total_seg} segments in {total_t:.1f} s "
                     f"(CPU oracle, -O3 -ffp-contract=off, one thread)"}
    if gpu is not None:
        gpu.seed = seed
        gpu._check(gpu.lib.rdc_reset(gpu.ctx), "rdc_reset")
        gpu.render_range(0, 1)
        g = gpu.accumulator(w.scene).reshape(-1, 4)[px]
        rgb_g, rgb_c = g[:, :3].astype(np.float64), acc[:, :3].astype(np.float64)
        out["image_check"] = {
            "pixels": int(len(px)),
            "bit_identical": bool(g.tobytes() == acc.tobytes()),
            "rmse_gpu_vs_cpu": float(np.sqrt(((rgb_g - rgb_c) ** 2).mean())),
            "what": "the CPU sample's last batch of pixels against the GPU render of the same seed and sample",
        }
    return out


# --------------------------------------------------------------- reference --
def reference_workload():
    """The headline workload built without loading the CUDA library: the
    camera matrices come from the oracle's restatement of
    Camera::update_matrices (bit-identical to the library's), so the CPU arm's
    process runs the reference's path only."""
    import oracle
    from raydar_gb300.scene import camera_matrices_from
    with camera_matrices_from(oracle.camera_matrices):
        return _workload()


def run_reference(args):
    rank, world, _ = _dist()
    if rank != 0:
        return
    import oracle
    w = reference_workload()
    sc = w.scene.to_c()
    try:
        threads = len(os.sched_getaffinity(0))
    except AttributeError:
        threads = os.cpu_count() or 1
    for i in range(args.warmup):
        oracle.render(sc, 0, 1, w.max_bounces, 500 + i, threads=threads)
    segs = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        _, s = oracle.render(sc, 0, 1, w.max_bounces, 1000 + k, threads=threads)
        segs += s
    dt = time.perf_counter() - t0
    v = segs / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded c2_default scene (64 spheres, 16 cubes, ground), fresh seed per step",
        "config": _config(w, w.spp),
        "sample_per_step": f"1 of the workload's {w.spp} samples of every pixel (segments/s is a rate)",
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"each step: the full 1920x1080 frame at 1 spp, {w.max_bounces} bounces, on "
                                   f"{threads} host threads ({segs} segments in {dt:.2f} s over {args.steps} steps); "
                                   "the CPU restatement of src/renderer/cpu.rs, -O3 -ffp-contract=off (the Rust "
                                   "reference cannot be built here)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# -------------------------------------------------------------------- ours --
def _traffic_per_launch():
    """DRAM bytes of one 1080p render launch from the committed ncu summary
    (per pixel, independent of spp)."""
    f = ROOT / "profiles" / "render_kernel_traffic.json"
    if not f.exists():
        return None
    try:
        d = json.loads(f.read_text())
        return float(d["dram_bytes_per_launch"])
    except (ValueError, KeyError):
        return None


def batch_bench(local: int, steps: int, spp_div: int = 1):
    """Config 3: the 64 seeded scenes of c3_batch in one persistent launch (CUDA
    graph, launch shape from the autotuner) vs one render launch per scene
    (each scene resident in its own context, launched back to back)."""
    from raydar_gb300 import CudaRenderer, RendererConfig, scenegen
    from raydar_gb300.batch import BatchRenderer

    ws = scenegen.c3_batch()
    items = [(w.scene, max(1, w.spp // spp_div), w.max_bounces, 3000 + i) for i, w in enumerate(ws)]
    br = BatchRenderer(items, device=local)
    tune = br.autotune()
    br.render()
    br.stats()
    segs, dev_ms = 0, 0.0
    t0 = time.perf_counter()
    for _ in range(steps):
        br.render()
        st = br.stats()  # synchronises
        segs += st.segments
        dev_ms += st.device_ms
    batch_s = (time.perf_counter() - t0) / steps
    paths = br.stats().paths
    br.close()

    rs = []
    for sc, spp, b, seed in items:
        r = CudaRenderer(RendererConfig(max_sample_count=spp, max_bounces=b), device=local, seed=seed)
        r.upload(sc)
        rs.append(r)
    for r, (sc, spp, b, seed) in zip(rs, items):  # warm-up
        r._check(r.lib.rdc_reset(r.ctx), "rdc_reset")
        r.render_range(0, spp)
        r.stats()
    ps_segs = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        for r, (sc, spp, b, seed) in zip(rs, items):
            r._check(r.lib.rdc_reset(r.ctx), "rdc_reset")
            r.render_range(0, spp)
            ps_segs += r.stats().segments  # synchronises: one scene at a time
    per_scene_s = (time.perf_counter() - t0) / steps
    for r in rs:
        r.close()
    n = len(items)
    return {
        "workload": f"c3_batch: {n} scenes, width 128..1024, 16:9 or 1:1, spp 16..512 log-uniform, "
                    f"4..12 bounces, 4..200 spheres + 0..20 cubes; {paths / 1e9:.2f} G paths per batch",
        "scenes_per_s": n / batch_s,
        "segments_per_s": segs / steps / batch_s,
        "kernel_ms_per_batch": dev_ms / steps,
        "per_scene_scenes_per_s": n / per_scene_s,
        "per_scene_segments_per_s": ps_segs / steps / per_scene_s,
        "speedup_vs_per_scene": per_scene_s / batch_s,
        "launch_config": {k: tune[k] for k in ("block_size", "blocks_per_sm", "refill_min_idle")},
        "steps": steps,
    }


def lbvh_bench(local: int, steps: int, peak_tflops: float, width: int = 1920, height: int = 1080, spp: int = 0,
               form: str = "auto"):
    """Config 5 forward: 100k spheres + 10k cubes, device-built LBVH, one
    1920x1080 frame of 256 spp / 12 bounces per step (width, height, spp:
    a smaller case of the same scene).  Ops/segment follow the LBVH model
    30 * node visits + 24 * object tests + 100, with the visit and test counts
    measured by the kernel in the same launches."""
    from raydar_gb300 import CudaRenderer, RendererConfig, native, scenegen

    w = scenegen.c5_large(width=width, height=height)
    if spp:
        w.spp = spp
    r = CudaRenderer(RendererConfig(max_sample_count=w.spp, max_bounces=w.max_bounces), device=local, seed=0)
    forms = {"auto": native.FORM_AUTO, "megakernel": native.FORM_MEGAKERNEL, "wavefront": native.FORM_WAVEFRONT}
    r._check(r.lib.rdc_set_render_form(r.ctx, forms[form]), "rdc_set_render_form")
    t0 = time.perf_counter()
    r.upload(w.scene)
    build_s = time.perf_counter() - t0
    st = r.stats()
    depth = st.bvh_depth
    r._check(r.lib.rdc_reset(r.ctx), "rdc_reset")
    r.render_range(0, w.spp)  # warm-up frame
    r.stats()
    segs = visits = tests = launches = 0
    dev_ms = 0.0
    t0 = time.perf_counter()
    for k in range(steps):
        r.seed = 7000 + k
        r._check(r.lib.rdc_reset(r.ctx), "rdc_reset")
        r.render_range(0, w.spp)
        st = r.stats()
        segs += st.segments
        visits += st.node_visits
        tests += st.prim_tests
        dev_ms += st.device_ms
        launches += st.kernel_launches
    wall = time.perf_counter() - t0
    r.close()
    v_per = visits / segs
    t_per = tests / segs
    ops = 30 * v_per + 24 * t_per + 100
    achieved = ops * segs / (dev_ms / 1e3) / 1e12
    return {
        "workload": "c5_large: 100k spheres r in [0.01,0.2] + 10k cubes edge in [0.02,0.3] in a 40x10x40 box, "
                    f"{width}x{height}, {w.spp} spp, 12 bounces, device-built LBVH",
        "segments_per_s": segs / wall,
        "kernel_ms_per_frame": dev_ms / steps,
        "node_visits_per_segment": v_per,
        "object_tests_per_segment": t_per,
        "ops_per_segment": ops,
        "achieved_tflops": achieved,
        "frac_of_peak": achieved / peak_tflops if peak_tflops else None,
        "bvh_build_s": build_s,
        "bvh_depth": depth,
        # rdc_render's form (RDC_FORM_AUTO): the wavefront once a wave holds 4 or more samples of every pixel
        "form": "wavefront" if launches > steps else "megakernel",
        "kernel_launches_per_frame": launches / steps,
        "steps": steps,
    }


def adjoint_bench(local: int, steps: int, fd_spp: int = 4096):
    """Config 4: 512x512, 128 spp, 6 bounces, 32 spheres + 2 emissive spheres
    + ground.  Loss = L2 distance to a target rendered from the same scene with
    every parameter perturbed by N(0, 0.05) and clamped (albedo and roughness
    to [0, 1], emission >= 0).  Per step: rdc_forward, then rdc_backward with
    dL/dimage = 2 (image - target); device times of both kernels and their
    ratio.  Then central differences with common random numbers (same seed,
    eps 1e-3, fd_spp samples) for two albedo channels and one emission,
    against the adjoint at the same spp."""
    import copy

    import numpy as np

    from raydar_gb300 import CudaRenderer, RendererConfig, scenegen

    w = scenegen.c4_diff()
    scene = w.scene
    rng = np.random.default_rng(40)
    target_scene = copy.deepcopy(scene)
    for o in target_scene.objects:
        m = o.material
        m.albedo = np.clip(m.albedo + rng.normal(0, 0.05, 3), 0, 1).astype(np.float32)
        m.roughness = float(np.float32(np.clip(m.roughness + rng.normal(0, 0.05), 0, 1)))
        if m.emission_strength > 0:
            m.emission_strength = float(np.float32(max(m.emission_strength + rng.normal(0, 0.05), 0.0)))
    r = CudaRenderer(RendererConfig(max_bounces=w.max_bounces), device=local, seed=11)
    target = r.forward(target_scene, w.spp)
    r.forward(scene, w.spp)  # warm-up
    fwd_ms, bwd_ms, fwd_segs, bwd_segs = [], [], 0, 0
    t0 = time.perf_counter()
    for k in range(steps):
        r.seed = 500 + k
        img = r.forward(scene, w.spp)
        st = r.stats()
        fwd_ms.append(st.device_ms)
        fwd_segs += st.segments
        dl = 2.0 * (img - target)
        ga, gr, ge = r.backward(scene, dl)
        st = r.stats()
        bwd_ms.append(st.device_ms)
        bwd_segs += st.segments
    wall = time.perf_counter() - t0

    # central differences with common random numbers at fd_spp
    r.seed = 77
    img = r.forward(scene, fd_spp)
    dl = 2.0 * (img - target)
    ga, gr, ge = r.backward(scene, dl)

    def loss(s):
        r.seed = 77
        im = r.forward(s, fd_spp)
        return float(((im.astype(np.float64) - target) ** 2).sum())

    checks = []
    diffuse = next(i for i, o in enumerate(scene.objects) if i > 0 and o.material.roughness == 1.0
                   and o.material.emission_strength == 0)
    for j, c in ((0, 1), (diffuse, 0)):
        lo, hi = copy.deepcopy(scene), copy.deepcopy(scene)
        lo.objects[j].material.albedo = lo.objects[j].material.albedo.copy()
        hi.objects[j].material.albedo = hi.objects[j].material.albedo.copy()
        a = float(scene.objects[j].material.albedo[c])
        lo.objects[j].material.albedo[c] = np.float32(a - 1e-3)
        hi.objects[j].material.albedo[c] = np.float32(a + 1e-3)
        den = float(hi.objects[j].material.albedo[c]) - float(lo.objects[j].material.albedo[c])
        fd = (loss(hi) - loss(lo)) / den
        checks.append({"param": f"albedo[{j}][{c}]", "adjoint": float(ga[j, c]), "central_difference": fd,
                       "rel_gap": float(abs(fd - ga[j, c]) / max(abs(fd), 1e-30))})
    j = len(scene.objects) - 1
    lo, hi = copy.deepcopy(scene), copy.deepcopy(scene)
    s0 = scene.objects[j].material.emission_strength
    lo.objects[j].material.emission_strength = float(np.float32(s0 - 1e-3))
    hi.objects[j].material.emission_strength = float(np.float32(s0 + 1e-3))
    den = hi.objects[j].material.emission_strength - lo.objects[j].material.emission_strength
    fd = float((loss(hi) - loss(lo)) / den)
    adj = float((ge[j] * np.asarray(scene.objects[j].material.emission_color, np.float32)).sum())
    checks.append({"param": f"emission_strength[{j}]", "adjoint": adj, "central_difference": fd,
                   "rel_gap": abs(fd - adj) / max(abs(fd), 1e-30)})
    # roughness on this cluttered scene: the difference quotient also holds the
    # paths whose hit object changes within the step (silhouette crossings, a
    # boundary term the estimator leaves out), so this entry states the gap
    metals = [i for i, o in enumerate(scene.objects) if o.material.metallic == 1.0 and o.material.roughness > 0.1]
    j = max(metals, key=lambda i: abs(gr[i]))
    lo, hi = copy.deepcopy(scene), copy.deepcopy(scene)
    r0 = scene.objects[j].material.roughness
    lo.objects[j].material.roughness = float(np.float32(r0 - 1e-3))
    hi.objects[j].material.roughness = float(np.float32(r0 + 1e-3))
    den = hi.objects[j].material.roughness - lo.objects[j].material.roughness
    fd = float((loss(hi) - loss(lo)) / den)
    checks.append({"param": f"roughness[{j}]", "adjoint": float(gr[j]), "central_difference": fd,
                   "rel_gap": abs(fd - float(gr[j])) / max(abs(fd), 1e-30),
                   "note": "c4 scene: the difference includes silhouette crossings the estimator omits"})
    r.close()
    rough_checks = roughness_fd_checks(local)
    f_ms, b_ms = sum(fwd_ms) / steps, sum(bwd_ms) / steps
    return {
        "workload": "c4_diff: 512x512, 128 spp, 6 bounces, 32 spheres + 2 emissive + ground; L2 loss to a "
                    "perturbed-parameter target",
        "forward_ms": f_ms, "backward_ms": b_ms, "adjoint_over_forward": b_ms / f_ms,
        "forward_segments_per_s": fwd_segs / (sum(fwd_ms) / 1e3),
        "backward_replayed_segments_per_s": bwd_segs / (sum(bwd_ms) / 1e3),
        "steps": steps, "wall_s": wall,
        "fd_check": {"spp": fd_spp, "eps": 1e-3, "common_random_numbers": True, "params": checks},
        "roughness_fd_check": rough_checks,
    }


def roughness_fd_checks(local: int, eps: float = 1e-2):
    """The roughness gradient against central differences (common random
    numbers) on the three scenes where they are well defined
    (tests/roughness_scenes.py): a lone rough metal sphere (pathwise part), a
    lone Specular-class sphere (+ the diffuse/specular coin) and a rough metal
    sphere over a glass floor (+ the Fresnel coin)."""
    import copy

    import numpy as np

    from raydar_gb300 import CudaRenderer, RendererConfig
    from tests import roughness_scenes as RS

    out = []
    for name, size, spp in (("lone_metal", 96, 256), ("lone_specular", 512, 4096), ("glass_floor", 512, 4096)):
        scene, j, bounces = getattr(RS, name)(size)
        dl = RS.pixel_weights(name, scene)
        r = CudaRenderer(RendererConfig(max_bounces=bounces), seed=1, device=local)
        r.forward(scene, spp)
        _, gr, _ = r.backward(scene, dl)

        def loss(rho):
            s = copy.deepcopy(scene)
            s.objects[j].material.roughness = rho
            return float((r.forward(s, spp).astype(np.float64) * dl).sum())

        r0 = scene.objects[j].material.roughness
        lo, hi = float(np.float32(r0 - eps)), float(np.float32(r0 + eps))
        fd = (loss(hi) - loss(lo)) / (hi - lo)
        r.close()
        out.append({"scene": name, "size": size, "spp": spp, "eps": eps, "roughness": r0,
                    "adjoint": float(gr[j]), "central_difference": fd,
                    "rel_gap": abs(fd - float(gr[j])) / max(abs(fd), 1e-30)})
    return out


def reference_scene_bench(local: int, steps: int, spp: int = 16, bounces: int = 12):
    """The reference's own benchmark scene (scenes/benchmark.rscn: 3840x2160,
    70 spheres + 113 cubes, committed as tests/golden/benchmark.rscn), rendered
    at full resolution, `spp` samples per frame, the default 12 bounces."""
    from raydar_gb300 import CudaRenderer, RendererConfig
    from raydar_gb300.roofline import ops_per_segment
    from raydar_gb300.scene import Scene

    scene = Scene.load(ROOT / "tests" / "golden" / "benchmark.rscn")
    r = CudaRenderer(RendererConfig(max_sample_count=spp, max_bounces=bounces), device=local, seed=0)
    r.upload(scene)
    r._check(r.lib.rdc_reset(r.ctx), "rdc_reset")
    r.render_range(0, spp)  # warm-up
    r.stats()
    ms, segs = 0.0, 0
    for k in range(steps):
        r.seed = 300 + k
        r._check(r.lib.rdc_reset(r.ctx), "rdc_reset")
        r.render_range(0, spp)
        st = r.stats()
        ms += st.device_ms
        segs += st.segments
    r.close()
    n = len(scene.objects)
    return {
        "workload": f"scenes/benchmark.rscn: {scene.width}x{scene.height}, {n} objects (70 spheres + 113 cubes), "
                    f"{spp} spp per frame, {bounces} bounces, brute force",
        "segments_per_s": segs / (ms / 1e3), "kernel_ms_per_frame": ms / steps,
        "ops_per_segment": ops_per_segment(n), "steps": steps,
    }


def progressive_bench(local: int, samples: int = 256, size: int = 584, bounces: int = 12):
    """The editor's live view (f1, src/renderer/cpu.rs:142-158 through the
    reference's render_sample): Scene::default in a 584x584 viewport (the size
    of the reference's own editor screenshot), one sample per call with the
    tone-mapped RGBA8 image read back each time, as the editor redraws.  Wall
    clock per call through the public API (upload check, render, sync,
    tone map, copy), and the kernel time inside it."""
    from raydar_gb300 import CudaRenderer, RendererConfig
    from raydar_gb300.scene import default_scene, resized

    scene = resized(default_scene(), size, size)
    r = CudaRenderer(RendererConfig(max_sample_count=samples, max_bounces=bounces), device=local, seed=0)
    r.new_frame(scene)
    for _ in range(8):  # warm-up: first uploads and launches
        r.render_sample(scene)
    r.new_frame(scene)
    dev_ms, n = 0.0, 0
    t0 = time.perf_counter()
    while True:
        img = r.render_sample(scene)
        if img is None:
            break
        dev_ms += r.stats().device_ms
        n += 1
    wall = time.perf_counter() - t0
    r.close()
    return {
        "workload": f"Scene::default at {size}x{size}, {bounces} bounces, {n} calls of render_sample "
                    f"(1 spp each, RGBA8 read back per call)",
        "samples_per_s": n / wall, "ms_per_sample_wall": wall / n * 1e3, "kernel_ms_per_sample": dev_ms / n,
        "d2h_bytes_per_sample": size * size * 4,
    }


def _mk_vs_wf(local, w, spp, steps, accel=None):
    from raydar_gb300 import CudaRenderer, RendererConfig, native
    out = {}
    for fn in ("rdc_render", "rdc_render_wavefront"):
        r = CudaRenderer(RendererConfig(max_bounces=w.max_bounces), device=local, seed=0)
        # the megakernel arm: rdc_render held to its megakernel form
        r._check(r.lib.rdc_set_render_form(r.ctx, native.FORM_MEGAKERNEL), "rdc_set_render_form")
        if accel is not None:
            r._check(r.lib.rdc_set_accel(r.ctx, accel), "rdc_set_accel")
        r.upload(w.scene)
        f = getattr(r.lib, fn)
        r._check(r.lib.rdc_reset(r.ctx), "rdc_reset")
        r._check(f(r.ctx, 0, spp, w.max_bounces, 1), fn)  # warm-up
        r.stats()
        ms, segs = 0.0, 0
        for k in range(steps):
            r._check(r.lib.rdc_reset(r.ctx), "rdc_reset")
            r._check(f(r.ctx, 0, spp, w.max_bounces, 100 + k), fn)
            st = r.stats()
            ms += st.device_ms
            segs += st.segments
        r.close()
        out[fn] = {"ms_per_frame": ms / steps, "segments_per_s": segs / (ms / 1e3)}
    return out["rdc_render"], out["rdc_render_wavefront"]


def wavefront_bench(local: int, steps: int, spp: int = 64, lbvh_spp: int = 16):
    """Megakernel vs wavefront A/B on the headline scene (c2_default 1920x1080,
    12 bounces) at `spp` samples per frame, and on the config-5 LBVH scene
    (1920x1080, 12 bounces) at `lbvh_spp`: the same paths, the same
    accumulator bit for bit; device time of each form."""
    from raydar_gb300 import native, scenegen

    mk, wf = _mk_vs_wf(local, scenegen.c2_default(), spp, steps)
    lmk, lwf = _mk_vs_wf(local, scenegen.c5_large(), lbvh_spp, steps, accel=native.ACCEL_LBVH)
    return {
        "workload": f"c2_default 1920x1080, {spp} spp per frame, 12 bounces, 81 objects",
        "megakernel": mk, "wavefront": wf,
        "wavefront_over_megakernel_time": wf["ms_per_frame"] / mk["ms_per_frame"],
        "lbvh": {
            "workload": f"c5_large 1920x1080, {lbvh_spp} spp per frame, 12 bounces, 110k objects, device LBVH",
            "megakernel": lmk, "wavefront": lwf,
            "wavefront_over_megakernel_time": lwf["ms_per_frame"] / lmk["ms_per_frame"],
        },
        "steps": steps,
    }


def inverse_bench(local: int, steps: int = 200, lr: float = 1e-2, spp: int = 64):
    """Config 5, inverse: recover the albedos of the 1,000 spheres nearest the
    camera in the 100k-sphere / 10k-cube scene (device LBVH) from a 512x512,
    64 spp target.  Start from albedo 0.5 for those spheres; each step renders
    (rdc_forward, fresh seed), takes the L2 loss to the target, runs
    rdc_backward and applies Adam (lr 1e-2) to their albedos, clamped to
    [0, 1], written back with rdc_update_materials (no geometry upload, no
    LBVH rebuild).  Reports the recovered-parameter RMSE before and after."""
    import numpy as np

    from raydar_gb300 import CudaRenderer, RendererConfig, scenegen
    from raydar_gb300.scene import material_records

    w = scenegen.c5_large(width=512, height=512)
    scene = w.scene
    rec = scene.packed
    cam = np.asarray(scene.camera.position, np.float64)
    spheres = np.where(rec["geometry"] == 0)[0]
    dist = np.linalg.norm(rec["center"][spheres].astype(np.float64) - cam, axis=1)
    chosen = spheres[np.argsort(dist)[:1000]]
    truth = rec["albedo"][chosen].astype(np.float64)

    r = CudaRenderer(RendererConfig(max_bounces=w.max_bounces), device=local, seed=1)
    t0 = time.perf_counter()
    r.upload(scene)
    r.seed = 900
    target = r.forward(None, 4 * spp)  # a cleaner target than one step's estimate
    mats = material_records(scene)
    est = np.full_like(truth, 0.5)
    mats["albedo"][chosen] = est.astype(np.float32)
    r.update_materials(mats)
    rmse0 = float(np.sqrt(((est - truth) ** 2).mean()))
    m1 = np.zeros_like(est)
    m2 = np.zeros_like(est)
    b1, b2, eps = 0.9, 0.999, 1e-8
    fwd_ms = bwd_ms = 0.0
    losses = []
    for k in range(steps):
        r.seed = 1000 + k
        img = r.forward(None, spp)
        fwd_ms += r.stats().device_ms
        diff = img.astype(np.float64) - target
        losses.append(float((diff ** 2).sum()))
        ga, _, _ = r.backward(None, (2.0 * diff).astype(np.float32))
        bwd_ms += r.stats().device_ms
        g = ga[chosen].astype(np.float64)
        m1 = b1 * m1 + (1 - b1) * g
        m2 = b2 * m2 + (1 - b2) * g * g
        mh = m1 / (1 - b1 ** (k + 1))
        vh = m2 / (1 - b2 ** (k + 1))
        est = np.clip(est - lr * mh / (np.sqrt(vh) + eps), 0.0, 1.0)
        mats["albedo"][chosen] = est.astype(np.float32)
        r.update_materials(mats)
    wall = time.perf_counter() - t0
    st = r.stats()
    r.close()
    seen = np.abs(est - 0.5).sum(axis=1) > 0  # spheres whose albedo moved (seen by some path)
    return {
        "workload": "c5_large at 512x512: 100k spheres + 10k cubes, device LBVH; albedos of the 1000 spheres "
                    f"nearest the camera from a {4 * spp} spp target, {spp} spp per step",
        "steps": steps, "lr": lr, "optimizer": "Adam(0.9, 0.999)",
        "rmse_initial": rmse0, "rmse_final": float(np.sqrt(((est - truth) ** 2).mean())),
        "rmse_final_spheres_moved": float(np.sqrt(((est[seen] - truth[seen]) ** 2).mean())) if seen.any() else None,
        "spheres_moved": int(seen.sum()),
        "loss_first": losses[0], "loss_last": losses[-1],
        "forward_ms_per_step": fwd_ms / steps, "backward_ms_per_step": bwd_ms / steps,
        "wall_s": wall, "accel": int(st.accel),
    }


def run_ours(args):
    import numpy as np
    import torch

    from raydar_gb300 import CudaRenderer, RendererConfig, native
    from raydar_gb300.roofline import ops_per_segment

    rank, world, local = _dist()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    w = _workload()
    spp = args.spp or w.spp
    r = CudaRenderer(RendererConfig(max_sample_count=spp, max_bounces=w.max_bounces), device=local, seed=0)
    lib, ctx = r.lib, r.ctx
    r.upload(w.scene)
    sptr = C.c_void_p()
    r._check(lib.rdc_get_stream(ctx, C.byref(sptr)), "rdc_get_stream")
    stream = torch.cuda.ExternalStream(sptr.value, device=torch.device("cuda", local))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def render(seed):
        r._check(lib.rdc_reset(ctx), "rdc_reset")
        r._check(lib.rdc_render(ctx, 0, spp, w.max_bounces, seed), "rdc_render")

    seed_base = 1000 + 100000 * rank
    for i in range(args.warmup):
        with torch.cuda.stream(stream):
            flush.zero_()
        render(seed_base + 50000 + i)
    r._check(lib.rdc_synchronize(ctx), "sync")
    # FP32 issue-rate probe with the GPU warm (the roofline denominator).
    ops_s = C.c_double(0)
    mhz = C.c_double(0)
    r._check(lib.rdc_measure_fp32_issue(ctx, C.byref(ops_s), C.byref(mhz)), "rdc_measure_fp32_issue")
    n_sms = torch.cuda.get_device_properties(local).multi_processor_count

    props = torch.cuda.get_device_properties(local)
    gpu_id = str(getattr(props, "uuid", "") or "")
    gpu_id = f"GPU-{gpu_id}" if gpu_id and not gpu_id.startswith("GPU-") else (gpu_id or str(local))
    clocks = ClockSampler(gpu_id)

    evs = []
    segs = []
    launches = 0
    barrier()
    clocks.start()
    time.sleep(0.4)
    barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        r._check(lib.rdc_reset(ctx), "rdc_reset")
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r._check(lib.rdc_render(ctx, 0, spp, w.max_bounces, seed_base + k), "rdc_render")
        e1.record(stream)
        st = r.stats()  # synchronises the context stream
        segs.append(st.segments)
        launches += st.kernel_launches
        evs.append((e0, e1))
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    barrier()
    clk = clocks.stop()
    elapsed = t1 - t0
    kernel_ms = [a.elapsed_time(b) for a, b in evs]
    my_segments = sum(segs)

    elapsed, total_segments = combine_replicas(dist, elapsed, my_segments, f"cuda:{local}")

    # ---- e2e through the C ABI from host buffers --------------------------
    img = np.empty((w.scene.height, w.scene.width, 4), np.uint8)
    sc = w.scene.to_c()
    st0 = r.stats()
    e2e_segs = 0
    barrier()
    te0 = time.perf_counter()
    for k in range(args.steps):
        r._check(lib.rdc_scene_upload(ctx, sc.ref()), "rdc_scene_upload")
        r._check(lib.rdc_reset(ctx), "rdc_reset")
        r._check(lib.rdc_render(ctx, 0, spp, w.max_bounces, seed_base + 20000 + k), "rdc_render")
        r._check(lib.rdc_read_rgba8(ctx, spp, native.u8ptr(img), img.size), "rdc_read_rgba8")
        e2e_segs += r.stats().segments
    te1 = time.perf_counter()
    st1 = r.stats()
    e2e_time, e2e_total = combine_replicas(dist, te1 - te0, e2e_segs, f"cuda:{local}")

    batched = None
    if rank == 0 and not args.no_batch:
        batched = batch_bench(local, max(1, min(args.steps, 3)), args.batch_spp_div)

    large = None
    if rank == 0 and not args.no_large:
        pk = max(ops_s.value / 1e12, n_sms * 128 * (clk.get("sm_mhz") or 0.0) * 1e6 / 1e12)
        large = lbvh_bench(local, max(1, min(args.steps, 2)), pk, form=args.form)

    adjoint = None
    if rank == 0 and not args.no_adjoint:
        adjoint = adjoint_bench(local, max(1, min(args.steps, 3)))

    wavefront = None
    if rank == 0 and not args.no_wavefront:
        wavefront = wavefront_bench(local, max(1, min(args.steps, 3)))

    refscene = None
    if rank == 0 and not args.no_refscene:
        refscene = reference_scene_bench(local, max(1, min(args.steps, 3)))

    progressive = None
    if rank == 0 and not args.no_progressive:
        progressive = progressive_bench(local)

    inverse = None
    if rank == 0 and not args.no_inverse:
        inverse = inverse_bench(local)

    base = None
    if rank == 0 and not args.no_cpu_baseline:
        base = cpu_baseline(w, args.cpu_seconds, gpu=r)

    r.close()
    if dist is not None:
        dist.destroy_process_group()
    if rank != 0:
        return

    n_obj = len(w.scene.objects)
    ops = ops_per_segment(n_obj)
    mean_kernel_s = sum(kernel_ms) / len(kernel_ms) / 1e3
    seg_per_launch = my_segments / len(segs)
    achieved = ops * seg_per_launch / mean_kernel_s / 1e12
    # Peak: the larger of the probe and SMs x 128 lanes x the median SM clock
    # sampled during the timed region (conservative: a larger peak, a smaller fraction).
    peak_probe = ops_s.value / 1e12
    peak_clock = n_sms * 128 * clk["sm_mhz"] * 1e6 / 1e12 if clk.get("sm_mhz") else 0.0
    peak = max(peak_probe, peak_clock)
    traffic = _traffic_per_launch()
    line = {
        "metric": METRIC, "value": total_segments / elapsed, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded c2_default scene (64 spheres, 16 cubes, ground), fresh seed per step",
        "config": _config(w, spp),
        "segments_per_step": seg_per_launch,
        "paths_per_step": w.scene.width * w.scene.height * spp,
        "kernel_ms_per_step": sum(kernel_ms) / len(kernel_ms),
        "roofline": {
            "bound": "fp32", "kernel": "render_kernel", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak if peak > 0 else None,
            "traffic": traffic,
            "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one 1080p render_kernel launch from "
                              "the committed ncu capture (profiles/render_kernel_traffic.json), not measured in this "
                              "run; per pixel, independent of spp",
            "ops_per_segment": ops,
            "peak_source": f"max of the FFMA issue rate measured in this run ({peak_probe:.2f} T lane-ops/s, "
                           f"= {mhz.value:.0f} MHz x {n_sms} SMs x 128) and {n_sms} SMs x 128 x the median "
                           f"sampled SM clock ({peak_clock:.2f} T); one FP32 op per lane per clock",
        },
        "e2e": {"value": e2e_total / e2e_time, "unit": UNIT,
                "h2d_bytes_per_step": (st1.h2d_bytes - st0.h2d_bytes) / args.steps,
                "d2h_bytes_per_step": (st1.d2h_bytes - st0.d2h_bytes) / args.steps},
        "gpu_launches": launches,
        "clocks": clk,
        "cpu_baseline": base,
        "batched": batched,
        "large_scene": large,
        "adjoint": adjoint,
        "wavefront_ab": wavefront,
        "reference_benchmark_scene": refscene,
        "progressive": progressive,
        "inverse": inverse,
    }
    print(json.dumps(line), flush=True)


def main():
    args = _args()
    if args.batch_only:
        import torch
        torch.cuda.set_device(_dist()[2])
        print(json.dumps({"batched": batch_bench(_dist()[2], max(1, min(args.steps, 3)), args.batch_spp_div)}))
        return
    if args.large_only:
        import torch
        torch.cuda.set_device(_dist()[2])
        wh = [int(x) for x in args.large_only.split("x")] if args.large_only != "0" else [1920, 1080, 0]
        print(json.dumps({"large_scene": lbvh_bench(_dist()[2], max(1, min(args.steps, 2)), 0.0, *wh, form=args.form)}))
        return
    if args.wavefront_only:
        import torch
        torch.cuda.set_device(_dist()[2])
        print(json.dumps({"wavefront_ab": wavefront_bench(_dist()[2], max(1, min(args.steps, 3)))}))
        return
    if args.inverse:
        import torch
        torch.cuda.set_device(_dist()[2])
        print(json.dumps({"inverse": inverse_bench(_dist()[2])}))
        return
    if args.adjoint_only:
        import torch
        torch.cuda.set_device(_dist()[2])
        print(json.dumps({"adjoint": adjoint_bench(_dist()[2], max(1, min(args.steps, 3)))}))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
