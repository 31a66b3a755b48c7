"""Benchmark: Mrays/s of the GB300 path tracer on the 256-icosphere scene.

Workload (one step = one frame): 256 level-4 icospheres (1.31 M triangles; the
identical geometries share one BLAS, + TLAS), 1 directional + 4 point + 2 spot lights, constant background
0.1, 1920x1080, 8 samples per pixel, path depth 8, Russian roulette from bounce
4 (kuafu's defaults). Rays = primary + extension + shadow traversals actually
issued; BVH build is outside the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

The line also carries "time_to_relmse": the Cornell box at 1920x1080, the learned
denoiser (trained first on this renderer's own low/high-spp pairs) against plain
accumulation, both measured until relMSE <= 1e-3 against a 40960-spp FP64
reference (kuafu_gb300/denoise_eval.py; --no-denoise skips it; N = 1 only). The
two networks shipped with the package (Cornell; Cornell and icosphere scenes) are
evaluated on the same frames, and all three networks on the 1080p icosphere scene
against plain accumulation there.

Under torchrun (N > 1) every rank renders its own replica of the workload (the
path has no cross-GPU exchange); value = rays of all ranks / max time over ranks.
--impl reference times the CPU implementation (the oracle port of kuafu's
shaders) on the host cores over a bounded crop of the same workload, with the
scene flattened on the oracle side: that arm maps no library of this package.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
# denoiser network shipped with the package (trained by kuafu_gb300.denoise_eval.train_network)
SHIPPED_WEIGHTS = ROOT / "kuafu_gb300" / "weights" / "unet_cornell_2000x256.kfw"
# 1200 Cornell windows and 300 windows of seeded 256-icosphere scenes, same inputs and targets
MIXED_WEIGHTS = ROOT / "kuafu_gb300" / "weights" / "unet_mixed_1500x256.kfw"
sys.path.insert(0, str(ROOT))

WORKLOAD = dict(width=1920, height=1080, spp=8, depth=8, count=256, level=4, seed=0)


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def aggregate_over_ranks(t_ms: float, rays: float, ws: int, device="cpu"):
    """The job's timed region and work under torchrun: the slowest rank's time (MAX) and
    the rays of all ranks (SUM), each rank rendering its own replica. One rank: as given."""
    if ws <= 1:
        return float(t_ms), float(rays)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(t_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    rr = torch.tensor([float(rays)], dtype=torch.float64, device=device)
    dist.all_reduce(rr, op=dist.ReduceOp.SUM)
    return float(t.item()), float(rr.item())


def _finish_ranks(ws: int):
    """All ranks leave together: rank 0 prints after its extra passes while the others wait."""
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()


def mrays_per_s(rays_all: float, t_ms: float) -> float:
    """Whole-job throughput: all ranks' rays over the slowest rank's time."""
    return rays_all / (t_ms / 1e3) / 1e6


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"kf_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        try:
            self.path.unlink()
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_scene(device: int, profile=False, debug=False):
    from kuafu_gb300 import api, scenes

    cfg = scenes.icosphere_config(spp=WORKLOAD["spp"], depth=WORKLOAD["depth"], seed=WORKLOAD["seed"],
                                  count=WORKLOAD["count"])
    cfg._c.device = device
    cfg.setProfile(profile)
    cfg.setDebugOutputs(debug)
    if "traversal" in WORKLOAD:
        cfg.setTraversal(WORKLOAD["traversal"])
    if "bvh_builder" in WORKLOAD:
        cfg.setBvhBuilder(WORKLOAD["bvh_builder"])
    if "blas_leaf_size" in WORKLOAD:
        cfg.setBlasLeafSize(WORKLOAD["blas_leaf_size"])
    if "blas_share" in WORKLOAD:
        cfg.setBlasShare(WORKLOAD["blas_share"])
    if "dyn_refill_below" in WORKLOAD or "dyn_steps" in WORKLOAD:
        cfg.setDynamicFetch(WORKLOAD.get("dyn_refill_below", 16), WORKLOAD.get("dyn_steps", 32))
    r = api.Kuafu(cfg)
    cam = scenes.icospheres(r, WORKLOAD["width"], WORKLOAD["height"], count=WORKLOAD["count"],
                            level=WORKLOAD["level"], seed=WORKLOAD["seed"])
    return r, cam


def _per_ray(sc, closest: bool) -> dict:
    """Node visits, triangle tests and instance entries per ray of one traversal kind
    (counting variant of the kernels)."""
    if closest:
        n = max(sc.rays_primary + sc.rays_extension, 1)
        return {"node_visits": sc.node_visits / n, "tri_tests": sc.tri_tests / n, "inst_entries": sc.inst_visits / n}
    n = max(sc.rays_shadow, 1)
    return {"node_visits": sc.shadow_node_visits / n, "tri_tests": sc.shadow_tri_tests / n,
            "inst_entries": sc.shadow_inst_visits / n}


def separate_blas_summary(device: int, steps: int = 5) -> dict:
    """The same frame with blas_share = 0: every icosphere geometry keeps its own copy of
    the BLAS nodes and triangles (256 copies, ~150 MB against the 129 MB L2) instead of the
    default one shared copy. Same hits and radiance; CUDA-event frame times after an L2
    flush, as for the headline."""
    import torch

    WORKLOAD["blas_share"] = 0
    try:
        r, _ = build_scene(device)
    finally:
        del WORKLOAD["blas_share"]
    stream = torch.cuda.ExternalStream(r.stream(), device=torch.device("cuda", device))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{device}")
    for _ in range(2):
        r.run()
    r.synchronize()
    nodes = r.stats().blas_nodes
    r.resetStats()
    ms = []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        r.run()
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    st = r.stats()
    rays = st.rays_primary + st.rays_extension + st.rays_shadow
    r.close()
    return {"mrays_s": rays / (sum(ms) / 1e3) / 1e6, "ms_per_step": statistics.median(ms), "blas_nodes": nodes}


def cpu_baseline_sample(seconds_target=12.0, threads=0):
    """The oracle on the host cores over a centred crop, sized for ~10-30 s of work. The
    scene is flattened on the oracle side (oracle/scenes.py): this leg maps no product
    library."""
    from oracle import oracle as O
    from oracle import scenes as OS

    W, H = WORKLOAD["width"], WORKLOAD["height"]
    fs = OS.icospheres(W, H, count=WORKLOAD["count"], level=WORKLOAD["level"], seed=WORKLOAD["seed"])
    pc = O.push_constants(WORKLOAD["spp"], WORKLOAD["depth"], clear=fs.clear, rr=True, rr_min=4)
    nthreads = threads or os.cpu_count() or 1
    side = 32
    while True:
        x0, y0 = (W - side) // 2, (H - side) // 2
        t0 = time.perf_counter()
        res = O.render(fs.flat, fs.camera, W, H, pc, seed=WORKLOAD["seed"], frame=0, camera_index=1, use_bvh=True,
                       threads=nthreads, crop=(x0, y0, side, side), want_paths=False, want_hits=False)
        dt = time.perf_counter() - t0
        rays = sum(res["rays"])
        if dt >= seconds_target / 4 or side >= 512:
            break
        side = min(512, int(side * max(1.5, (seconds_target / 4 / max(dt, 1e-3)) ** 0.5)))
    return {"value": rays / dt / 1e6, "unit": "Mrays/s", "cores": nthreads, "kind": "port",
            "sample": f"{side}x{side} centre crop of the 1920x1080 frame, {WORKLOAD['spp']} spp, depth "
                      f"{WORKLOAD['depth']}, {rays} rays in {dt:.2f} s"}


def cpu_baseline_cornell(threads=0) -> dict:
    """The oracle on the host cores over the whole Cornell configuration (256x256, 64 spp,
    depth 5, no Russian roulette). The scene is built and flattened by this package's host
    code (a host-only renderer: no device work), so this leg runs in the GPU arm only."""
    from kuafu_gb300 import api, scenes
    from oracle import oracle as O

    cfg = scenes.cornell_config(spp=64, depth=5)
    cfg.setHostOnly(True)
    r = api.Kuafu(cfg)
    try:
        cam = scenes.cornell(r, 256, 256)
        flat = r.getScene().export()
        pc = O.push_constants(64, 5, clear=(0.0, 0.0, 0.0, 1.0))
        nthreads = threads or os.cpu_count() or 1
        t0 = time.perf_counter()
        res = O.render(flat, cam.ubo(), 256, 256, pc, seed=0, frame=0, camera_index=1, use_bvh=True,
                       threads=nthreads, want_paths=False, want_hits=False)
        dt = time.perf_counter() - t0
    finally:
        r.close()
    rays = sum(res["rays"])
    return {"value": rays / dt / 1e6, "unit": "Mrays/s", "cores": nthreads, "kind": "port",
            "sample": f"Cornell 256x256, 64 spp, depth 5 in full: {rays} rays in {dt:.2f} s"}


def time_to_relmse_summary() -> dict:
    """Second half of the metric: time to relMSE <= 1e-3 at 1920x1080 (Cornell box, depth 5),
    learned denoiser vs plain accumulation, one GPU (kuafu_gb300.denoise_eval). Both arms
    are measured (no extrapolation) against a 40960-spp FP64 reference."""
    import tempfile

    from kuafu_gb300 import denoise_eval

    log = lambda m: print(m, file=sys.stderr, flush=True)  # noqa: E731
    t0 = time.perf_counter()
    shipped = SHIPPED_WEIGHTS if SHIPPED_WEIGHTS.exists() else None
    try:
        with tempfile.TemporaryDirectory() as tmp:
            in_run = str(Path(tmp) / "in_run.kfw")
            more = {"mixed": str(MIXED_WEIGHTS)} if MIXED_WEIGHTS.exists() else None
            res = denoise_eval.run(shipped=shipped, save_trained=in_run, more_networks=more, log=log)
            nets = {"in_run": in_run}
            if shipped:
                nets["shipped"] = str(shipped)
            nets.update(more or {})
            ico = denoise_eval.icosphere_eval(nets, log=log)
    except Exception as e:  # reported in the line, the Mrays/s result stands
        return {"error": f"{type(e).__name__}: {e}"}
    peak_tf = None
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peak_tf = json.loads(pk.read_text()).get("bf16_tflops")
    head = next(r for r in res["time_to_relmse"] if r["tau"] == 1e-3)
    tf = [d["denoise_tflops"] for d in res["denoised"]]
    ach = statistics.median(tf)
    return {
        "scene": f"cornell {res['width']}x{res['height']} depth {res['depth']}",
        "relmse": "mean (x - ref)^2 / (ref^2 + 1e-2) over pixels and rgb, FP64 on the GPU",
        "reference": res["reference"],
        "headline_tau": 1e-3,
        "headline": head["relmse"],
        "headline_debiased": head["relmse_debiased"],
        "thresholds": res["time_to_relmse"],
        "plain": res["plain"],
        "plain_ms_per_spp": res["plain_fit"]["ms_per_spp"],
        "denoised": [{k: d[k] for k in ("spp", "ms", "render_ms", "denoise_ms", "relmse", "relmse_debiased")}
                     for d in res["denoised"]],
        "training": {k: v for k, v in res["training"].items() if k != "loss_curve"},
        "loss_first_last": [res["training"]["loss_curve"][0], res["training"]["loss_curve"][-1]],
        "note_4096spp_reference": res["note_4096spp_reference"],
        "shipped_network": ({"weights": SHIPPED_WEIGHTS.name,
                             "training": "2000 Cornell variations through 256x256 windows of the 1920x1080 view, "
                                         "4-spp inputs plus one input of 1..1024 spp each, 4096-spp FP64 targets "
                                         "(kuafu_gb300.denoise_eval.train_network)",
                             "headline": next(r for r in res["shipped"]["time_to_relmse"]
                                              if r["tau"] == 1e-3)["relmse"],
                             "denoised": [{k: d[k] for k in ("spp", "ms", "relmse_noisy", "relmse")}
                                          for d in res["shipped"]["denoised"]]}
                            if "shipped" in res else None),
        "mixed_network": ({"weights": MIXED_WEIGHTS.name,
                           "training": "1200 Cornell variations and 300 seeded 256-icosphere scenes (depth 8, RR) "
                                       "through 256x256 windows of their 1920x1080 views, inputs and targets as "
                                       "the shipped network's, 8000 Adam steps",
                           "headline": next(r for r in res["networks"]["mixed"]["time_to_relmse"]
                                            if r["tau"] == 1e-3)["relmse"],
                           "denoised": [{k: d[k] for k in ("spp", "ms", "relmse_noisy", "relmse")}
                                        for d in res["networks"]["mixed"]["denoised"]]}
                          if "mixed" in res.get("networks", {}) else None),
        "icosphere_scene": ico,
        # relMSE 1e-3 on the icosphere scene, per network: plain accumulation against one frame
        # plus one inference, both measured against the same 8192-spp reference
        "icosphere_headline": {n: next(r for r in ico[n + "_time_to_relmse"] if r["tau"] == 1e-3)["relmse"]
                               for n in nets if n + "_time_to_relmse" in ico},
        "denoiser_roofline": {"bound": "tensor", "achieved": ach, "peak": peak_tf, "unit": "TFLOP/s",
                              "frac": (ach / peak_tf) if peak_tf else None,
                              "flops_per_frame": res["denoiser_flops_per_frame"],
                              "peak_source": "measured (bf16 burst)" if peak_tf else None},
        "seconds": time.perf_counter() - t0,
    }


def batched_summary(device: int, steps: int = 3) -> dict:
    """The batched workload (64 Cornell rooms with 2..400 level-4 icospheres, 128 views of
    128^2..1024^2 at 1..32 spp, depth 5) traced as one wavefront per frame: Mrays/s with the
    renderer's default launch configuration, then after kf_renderer_autotune (tuned on every
    8th view at <= 4 spp) on the full batch."""
    import torch

    from kuafu_gb300 import api, scenes

    t0 = time.perf_counter()
    try:
        r = api.Kuafu(scenes.batch_config())
        items = scenes.batch_views(r)
        stream = torch.cuda.ExternalStream(r.stream(), device=torch.device("cuda", device))

        def measure():
            r.runBatch(items)  # warm-up: pools, graph capture
            r.synchronize()
            r.resetStats()
            ms = []
            for _ in range(steps):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                r.runBatch(items)
                e1.record(stream)
                e1.synchronize()
                ms.append(e0.elapsed_time(e1))
            st = r.stats()
            rays = st.rays_primary + st.rays_extension + st.rays_shadow
            return {"ms_per_batch": statistics.median(ms), "mrays_s": rays / (sum(ms) / 1e3) / 1e6,
                    "rays_per_batch": rays / steps}

        default = measure()
        tune_items = [(s, c, min(spp, 4)) for (s, c, spp) in items[::8]]
        res = r.autotune(tune_items, reps=2)
        tuned = measure()
        out = {
            "workload": "64 Cornell rooms x 2..400 level-4 icospheres, 128 views 128^2..1024^2, 1..32 spp, depth 5",
            "views": len(items),
            "scenes": len({id(s) for s, _, _ in items}),
            "paths_per_batch": int(sum(c._size()[0] * c._size()[1] * spp for _, c, spp in items)),
            "default": default,
            "autotuned": tuned,
            "autotune": {"traversal": res.traversal, "blas_leaf_size": res.blas_leaf_size,
                         "max_paths_in_flight": res.max_paths_in_flight, "grid_extend": res.grid_extend,
                         "grid_shade": res.grid_shade, "dyn_refill_below": res.dyn_refill_below,
                         "dyn_steps": res.dyn_steps, "candidates": res.candidates,
                         "tune_set_ms_before": res.start_ms, "tune_set_ms_after": res.best_ms},
            "graph": "one CUDA graph per batch layout, replayed every batch",
            "seconds": time.perf_counter() - t0,
        }
        r.close()
        return out
    except Exception as e:  # reported in the line, the Mrays/s result stands
        return {"error": f"{type(e).__name__}: {e}"}


def active_light_summary(device: int, steps: int = 3) -> dict:
    """Active light sensing: the icosphere scene trimmed to 64 instances, a 1280x720 dot
    pattern (5 %) projected for two 848x480 IR cameras 55 mm apart, plus a 1280x720 RGB
    camera; 16 spp, depth 6; the three views in one batch; the shipped denoiser network on
    the RGB view."""
    import torch

    from kuafu_gb300 import api, scenes

    t0 = time.perf_counter()
    try:
        r = api.Kuafu(scenes.icosphere_config(spp=16, depth=6, count=64))
        rig = scenes.active_light_rig(r, count=64)
        (irs, left), (_, right) = rig["ir"]
        rgbs, rgb = rig["rgb"]
        items = [(irs, left, 16), (irs, right, 16), (rgbs, rgb, 16)]
        stream = torch.cuda.ExternalStream(r.stream(), device=torch.device("cuda", device))
        r.runBatch(items)
        r.synchronize()
        r.resetStats()
        ms = []
        for _ in range(steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r.runBatch(items)
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        st = r.stats()
        rays = st.rays_primary + st.rays_extension + st.rays_shadow
        d = api.Denoiser(r, seed=0)
        if SHIPPED_WEIGHTS.exists():
            d.load(str(SHIPPED_WEIGHTS))
        d.apply(rgb)
        r.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        d.apply(rgb)
        e1.record(stream)
        e1.synchronize()
        dn_ms = e0.elapsed_time(e1)
        ir = r.downloadAov(left, 0)[..., 0]
        out = {"workload": "64 icospheres, 1280x720 dot projector (5 %), IR 2x 848x480 (55 mm), RGB 1280x720, "
                           "16 spp, depth 6, one batch",
               "ms_per_batch": statistics.median(ms), "mrays_s": rays / (sum(ms) / 1e3) / 1e6,
               "rgb_denoise_ms": dn_ms,
               "rgb_denoiser_weights": SHIPPED_WEIGHTS.name if SHIPPED_WEIGHTS.exists() else "untrained",
               "ir_lit_fraction": float((ir > 0).mean()),
               "seconds": time.perf_counter() - t0}
        d.close()
        r.close()
        return out
    except Exception as e:
        return {"error": f"{type(e).__name__}: {e}"}


def run_denoiser_profile(reps: int) -> int:
    """Profiling entry: `reps` 1920x1080 denoiser inferences (untrained weights: the time does
    not depend on them) on a 1-spp Cornell frame; prints the CUDA-event time of each."""
    import torch

    from kuafu_gb300 import api, scenes

    with api.Kuafu(scenes.cornell_config(spp=1, depth=5)) as r:
        cam = scenes.cornell(r, 1920, 1080)
        r.run()
        r.synchronize()
        d = api.Denoiser(r, seed=0)
        stream = torch.cuda.ExternalStream(r.stream())
        ms = []
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            d.apply(cam)
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        from kuafu_gb300.denoise_eval import unet_flops
        print(json.dumps({"denoiser_inference_ms": ms, "flops_per_frame": unet_flops(1080, 1920)}), flush=True)
        d.close()
    return 0


def run_reference(args):
    ws, rank, local = _dist()
    if rank != 0:
        return 0
    samples = []
    base = None
    for step in range(args.warmup + args.steps):
        b = cpu_baseline_sample(seconds_target=8.0 if step < args.warmup else 10.0)
        if step >= args.warmup:
            samples.append(b["value"])
            base = b
    v = statistics.median(samples)
    line = {"impl": "reference", "metric": "Mrays/s", "value": v, "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "icospheres-256 1920x1080 8spp depth8", **WORKLOAD},
            "cpu_baseline": {**base, "value": v},
            "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import ctypes as C

    import torch

    from kuafu_gb300 import _native as N

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    device = local
    r, cam = build_scene(device)
    stream = torch.cuda.ExternalStream(r.stream(), device=torch.device("cuda", device))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{device}")

    # warm-up (also builds BLAS / TLAS and captures the frame graph)
    for _ in range(max(args.warmup, 1)):
        r.run()
    r.synchronize()
    first_build_ms = r.stats().bvh_build_ms
    r.resetStats()

    def barrier():
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()

    clocks = ClockSampler(device)
    times = []
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)  # L2 flush between steps, outside the timed events
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        r.run()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier()
    st = r.stats()
    rays = st.rays_primary + st.rays_extension + st.rays_shadow
    t_ms, rays_all = aggregate_over_ranks(sum(times), rays, ws, device=f"cuda:{device}")
    value = mrays_per_s(rays_all, t_ms)
    rays_per_frame = rays / args.steps
    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": "Mrays/s", "value": value, "unit": "Mrays/s", "quick": True,
                              "ms_per_step": t_ms / args.steps, "config": dict(WORKLOAD), "clocks": clk,
                              "bvh_build_ms": first_build_ms}), flush=True)
        r.close()
        _finish_ranks(ws)
        return 0

    # e2e: the public API with host buffers: run + download of the BGRA frame per step
    host = torch.empty((WORKLOAD["height"], WORKLOAD["width"], 4), dtype=torch.uint8).pin_memory()
    r.resetStats()
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r.run()
        N.check(N.load().kf_renderer_download_latest_frame(r._h, cam._h, host.data_ptr(), host.numel()))
    e2e_s = time.perf_counter() - t0
    st2 = r.stats()
    e2e_rays = st2.rays_primary + st2.rays_extension + st2.rays_shadow
    e2e_ms, e2e_rays_all = aggregate_over_ranks(e2e_s * 1e3, e2e_rays, ws, device=f"cuda:{device}")
    e2e_val = mrays_per_s(e2e_rays_all, e2e_ms)
    h2d = C.sizeof(N.kf_camera_ubo) + C.sizeof(N.kf_push_constants) + 32 + C.sizeof(N.kf_dir_light_ubo) + \
        C.sizeof(N.kf_point_lights_ubo) + C.sizeof(N.kf_active_lights_ubo)

    result = None
    if rank == 0:
        # per-kernel durations (CUDA events around each launch) and algorithmic bytes (counting pass)
        r.close()
        rp, _ = build_scene(device, profile=True)
        rp.run()
        build_ms = rp.stats().bvh_build_ms  # default builder, first frame of a fresh scene
        rp.resetStats()
        rp.run()
        sp = rp.stats()
        rp.countTraversal(True)
        rp.resetStats()
        rp.run()
        sc = rp.stats()
        # the traversal's roofline denominator: achievable L2 read bandwidth of this GPU
        l2_peak = rp.measureL2Read()
        rp.close()
        gpu_build_ms = {}
        if WORKLOAD.get("bvh_builder", 1) == 1:
            for b in (0, 2):  # GPU LBVH, GPU PLOC
                WORKLOAD["bvh_builder"] = b
                rl, _ = build_scene(device, profile=True)
                rl.run()
                gpu_build_ms[b] = rl.stats().bvh_build_ms
                rl.close()
            del WORKLOAD["bvh_builder"]
        launches = WORKLOAD["depth"] + 1
        node_b, tri_b, inst_b = 128, 48, 64
        ext_bytes = sc.node_visits * node_b + sc.tri_tests * tri_b + sc.inst_visits * inst_b
        sh_bytes = sc.shadow_node_visits * node_b + sc.shadow_tri_tests * tri_b + sc.shadow_inst_visits * inst_b
        peak, peak_kind = _peaks()
        dom_ext = sp.extend_ms >= sp.shadow_ms
        k_bytes, k_ms = (ext_bytes, sp.extend_ms) if dom_ext else (sh_bytes, sp.shadow_ms)
        achieved = k_bytes / launches / (k_ms / launches / 1e3) / 1e9 if k_ms > 0 else None
        if WORKLOAD.get("traversal", 1) == 1:
            kname = "k_trace_dyn<closest-hit>" if dom_ext else "k_trace_dyn<shadow>"
        else:
            kname = "k_extend" if dom_ext else "k_shadow"
        traffic = None
        tf = ROOT / "profiles" / "traffic.json"
        if tf.exists():
            try:
                traffic = json.loads(tf.read_text()).get(kname + " dram_bytes_per_launch")
            except Exception:
                traffic = None
        shared_nodes = sp.blas_nodes
        separate = separate_blas_summary(device)
        cpu = cpu_baseline_sample()
        try:
            cpu["cornell_256_64spp"] = cpu_baseline_cornell()
        except Exception as e:  # reported in the line, the main baseline stands
            cpu["cornell_256_64spp"] = {"error": f"{type(e).__name__}: {e}"}
        # single-GPU experiments: run once, at N = 1 (under torchrun the other ranks would idle)
        ttr = None if (args.no_denoise or ws > 1) else time_to_relmse_summary()
        batched = None if (args.no_batch or ws > 1) else batched_summary(device)
        active = None if (args.no_batch or ws > 1) else active_light_summary(device)
        result = {
            "metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "icospheres-256 1920x1080 8spp depth8", **WORKLOAD,
                       "triangles": WORKLOAD["count"] * 20 * 4 ** WORKLOAD["level"],
                       "rays_per_frame": rays_per_frame, "l2": "flushed (512 MiB write) before every timed step",
                       "parallelism": f"replicas x{ws}"},
            "roofline": {"bound": "l2", "kernel": kname,
                         "achieved": achieved, "peak": l2_peak, "unit": "GB/s",
                         "frac": (achieved / l2_peak) if achieved else None, "traffic": traffic,
                         "peak_source": "measured in this run: 32 MiB L2-resident buffer read 64 times through L2 "
                                        "(ld.global.cg, full occupancy), best of 5 (kf_renderer_measure_l2_read)",
                         "achieved_basis": "algorithmic bytes (node 128 B, triangle 48 B, instance 64 B per visit, "
                                           "counted) per launch / CUDA-event time per launch",
                         "hbm_equivalent": {"peak": peak, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                                            "frac": (achieved / peak) if achieved else None},
                         "bytes_per_ray": (k_bytes / ((sc.rays_primary + sc.rays_extension) if dom_ext else
                                                      max(sc.rays_shadow, 1))),
                         "per_ray": _per_ray(sc, dom_ext),
                         "kernel_ms_per_frame": {"extend": sp.extend_ms, "shade": sp.shade_ms,
                                                 "shadow": sp.shadow_ms, "frame": sp.frame_ms}},
            "blas": {"shared": {"blas_nodes": shared_nodes,
                                "note": "the 256 geometries have identical positions and indices (one material "
                                        "each) and share one BLAS copy (blas_share = 1, the default)"},
                     "separate": separate},
            "bvh_build_ms": {"default (host SAH, 256 BLAS + TLAS)": build_ms,
                             "gpu_lbvh (256 BLAS + TLAS)": gpu_build_ms.get(0),
                             "gpu_ploc (256 BLAS + TLAS)": gpu_build_ms.get(2),
                             "note": "the first frame's scene update (geometry upload, BLAS and TLAS builds) between "
                                     "CUDA events on the renderer's stream, host build time included; the 256 "
                                     "identical geometries share one BLAS build"},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_val, "unit": "Mrays/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": WORKLOAD["width"] * WORKLOAD["height"] * 4},
            "clocks": clk,
            # per frame: raygen; per bounce closest-hit traversal, k_miss, k_shade, k_nee,
            # shadow traversal, k_gather; resolve and sRGB
            "gpu_launches": args.steps * (1 + 6 * (WORKLOAD["depth"] + 1) + 2),
        }
        if ttr is not None:
            result["time_to_relmse"] = ttr
        if batched is not None:
            result["batched"] = batched
        if active is not None:
            result["active_light"] = active
        print(json.dumps(result), flush=True)
    else:
        r.close()
    _finish_ranks(ws)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--width", type=int, default=None, help="profiling: smaller frame of the same scene")
    ap.add_argument("--height", type=int, default=None)
    ap.add_argument("--quick", action="store_true",
                    help="profiling: timed steps only (no e2e, counting or CPU-baseline passes)")
    ap.add_argument("--traversal", type=int, default=None, help="0: thread per ray, 1: dynamic fetch (default)")
    ap.add_argument("--no-denoise", action="store_true",
                    help="skip the time-to-relMSE experiment (denoiser training and 1080p evaluation)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched 128-view workload")
    ap.add_argument("--bvh-builder", type=int, default=None, help="0: GPU LBVH, 1: host SAH (default), 2: GPU PLOC")
    ap.add_argument("--leaf", type=int, default=None, help="BLAS leaf size")
    ap.add_argument("--blas-share", type=int, default=None, help="1: identical geometries share one BLAS (default)")
    ap.add_argument("--dyn", type=int, nargs=2, default=None, metavar=("REFILL_BELOW", "STEPS"),
                    help="persistent traversal scheduling")
    ap.add_argument("--profile-denoiser", type=int, default=0, metavar="N",
                    help="profiling: only N 1080p denoiser inferences")
    args = ap.parse_args()
    if args.traversal is not None:
        WORKLOAD["traversal"] = args.traversal
    if args.bvh_builder is not None:
        WORKLOAD["bvh_builder"] = args.bvh_builder
    if args.leaf is not None:
        WORKLOAD["blas_leaf_size"] = args.leaf
    if args.blas_share is not None:
        WORKLOAD["blas_share"] = args.blas_share
    if args.dyn is not None:
        WORKLOAD["dyn_refill_below"], WORKLOAD["dyn_steps"] = args.dyn
    if args.warmup < 3:
        args.warmup = 3
    if args.width:
        WORKLOAD["width"] = args.width
    if args.height:
        WORKLOAD["height"] = args.height
    from kuafu_gb300 import build

    build.build_oracle()
    if args.impl == "reference":
        return run_reference(args)
    build.build_libkf()
    if args.profile_denoiser:
        return run_denoiser_profile(args.profile_denoiser)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
