"""Time-to-relMSE of the learned denoiser against plain accumulation.

The scene is the Cornell box (kuafu's example scene, built procedurally) rendered
at 1920x1080, path depth 5, no Russian roulette. The experiment, all on one GPU:

1. Reference: two independent FP64 accumulations (seeds A and B) of ref_spp / 2
   samples each; ref = their mean. relMSE(A, B) / 4 estimates the reference's own
   noise floor (the expected relMSE of a noise-free image against this reference),
   reported as `ref_floor`; the default 40960 spp put it near 4.6e-4, well below
   the 1e-3 target, so raw relMSE against the reference can be measured down to it.
2. Plain accumulation (an independent seed) into the FP64 sum: frames of
   `plain_frame_spp` samples, checkpoints at powers of two to 1024 spp and every
   `plain_checkpoint_step` samples after that, until the raw relMSE reaches the
   smallest threshold (or `plain_max_spp`); cumulative GPU time of the frames
   from CUDA events (the checkpoints' relMSE evaluations are not counted).
3. Learned denoiser: trained in the run on this renderer's own pairs (Cornell
   variations seen through 256x256 windows of the 1920x1080 view, inputs cycling
   1..1024 spp, targets at 4096 spp), then applied to single frames of k spp of the
   held-out scene; time = render + denoise (CUDA events). With `shipped` set, the
   network shipped with the package (train_network: 2000 windows, 4-spp inputs plus
   one more input per window, 4096-spp targets) is evaluated on the same frames, and
   so is each network of `more_networks` (name -> parameter file).
4. For each threshold tau: the measured time plain accumulation needs to reach raw
   relMSE <= tau and the time the denoised form needs (smallest k whose denoised
   frame reaches tau), and their ratio. "Debiased" values (raw minus ref_floor)
   are reported beside them.

relMSE = mean over pixels and channels of (x - ref)^2 / (ref^2 + 1e-2), reduced
in FP64 on the GPU (kf_relmse).

  python -m kuafu_gb300.denoise_eval [--small] [--json out.json]
  python -m kuafu_gb300.denoise_eval --train-network kuafu_gb300/weights/unet_cornell_2000x256.kfw
  python -m kuafu_gb300.denoise_eval --train-network kuafu_gb300/weights/unet_mixed_1500x256.kfw \
      --views 1200 --icosphere-views 300 --train-iters 8000
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from . import _native as N
from . import api, scenes

EPS = 1e-2

# (cin, cout) of the U-Net convolutions (kf_denoise.cu) and their resolution level
_LAYERS = [(32, 32, 0), (32, 32, 0), (32, 64, 1), (64, 64, 1), (64, 96, 2), (96, 96, 2), (96, 128, 3),
           (128, 128, 3), (128, 160, 4), (160, 160, 4), (288, 128, 3), (128, 128, 3), (224, 96, 2), (96, 96, 2),
           (160, 64, 1), (64, 64, 1), (96, 32, 0), (32, 32, 0), (32, 3, 0)]


def unet_flops(h: int, w: int) -> float:
    """Dense multiply-add FLOPs one inference executes (2 * H_l * W_l * Cin * Cout * 9 summed
    over convs). Frames at least 96 wide feed the first convolution 16 input channels (the
    11 features and 5 zeros) instead of 32."""
    hp, wp = (h + 15) // 16 * 16, (w + 15) // 16 * 16
    layers = [(16, 32, 0)] + _LAYERS[1:] if wp >= 96 else _LAYERS
    return float(sum(2.0 * (hp >> l) * (wp >> l) * ci * co * 9 for ci, co, l in layers))


class _Timer:
    """CUDA events on the renderer's stream."""

    def __init__(self, r: api.Kuafu):
        import torch

        self.torch = torch
        self.stream = torch.cuda.ExternalStream(r.stream())

    def __enter__(self):
        t = self.torch
        self.e0 = t.cuda.Event(enable_timing=True)
        self.e1 = t.cuda.Event(enable_timing=True)
        self.e0.record(self.stream)
        return self

    def __exit__(self, *a):
        self.e1.record(self.stream)
        self.e1.synchronize()
        self.ms = self.e0.elapsed_time(self.e1)


def _gpu_relmse(r: api.Kuafu, x: np.ndarray, ref: np.ndarray) -> float:
    """kf_relmse over float4 images (host arrays uploaded to the device)."""
    import ctypes as C

    import torch

    a = torch.from_numpy(np.ascontiguousarray(x, np.float32).reshape(-1, 4)).cuda()
    b = torch.from_numpy(np.ascontiguousarray(ref, np.float32).reshape(-1, 4)).cuda()
    torch.cuda.synchronize()
    out = C.c_double()
    N.check(N.load().kf_relmse(r._h, a.data_ptr(), b.data_ptr(), a.shape[0], EPS, C.byref(out)))
    return out.value


def _fp64_mean(r: api.Kuafu, cam: api.Camera) -> np.ndarray:
    s = r.downloadAov(cam, N.KF_AOV_SUM_F64)
    out = np.ones(s.shape, np.float64)
    out[..., :3] = s[..., :3] / s[..., 3:4]
    return out


def _accumulate(r, cfg, cam, seed, spp_total, frame_spp):
    cfg.setSeed(seed)
    cfg.setPerPixelSampleRate(frame_spp)
    cfg.setAccumulatingFrames(True)
    cfg.setUseDenoiser(False)
    r.applyConfig()
    r.resetFrame()
    for _ in range(spp_total // frame_spp):
        r.run()
    r.synchronize()
    return _fp64_mean(r, cam)


def window_camera(cam: api.Camera, size: int, full_w: int, full_h: int, x0: int, y0: int, fov_deg=40.0):
    """Makes cam a size x size camera that sees pixels [x0, x0 + size) x [y0, y0 + size) of
    the full_w x full_h pinhole view of the same pose: same focal length, principal point
    moved by the window's origin (kuafu's projection, src/core/camera.cpp:111-124, puts
    pixel u at fx * X / -Z + cx). Training crops are then rendered at the scale of the
    1080p frames the network denoises, for the cost of the crop."""
    fy = (full_h / 2.0) / math.tan(math.radians(fov_deg) / 2.0)
    cam.setFullPerspective(size, size, fy, fy, full_w / 2.0 - x0, full_h / 2.0 - y0, 0.0)


def add_training_views(r: api.Kuafu, cfg: api.Config, d: api.Denoiser, count: int, size: int, full_w: int,
                       full_h: int, inputs_of, high_spp: int, high_frames: int, first: int = 0, log=None) -> float:
    """Adds `count` training views: seeded Cornell variations (scenes.cornell variation
    1000 + v), each seen through a size x size window at a seeded place of the full_w x
    full_h view, with inputs of inputs_of(v) spp and one target of high_frames x high_spp
    samples (FP64 accumulation). Each view's scene is removed once its pairs are stored.
    Returns the seconds taken."""
    rng = scenes.SplitMix64(0x5EED0000 + first)
    t0 = time.perf_counter()
    for v in range(first, first + count):
        s = r.createScene()
        c = scenes.cornell(r, size, size, scene=s, variation=1000 + v)
        x0 = min(full_w - size, int(rng.uniform() * (full_w - size + 1)))
        y0 = min(full_h - size, int(rng.uniform() * (full_h - size + 1)))
        window_camera(c, size, full_w, full_h, x0, y0)
        cfg.setSeed(50000 + v)
        r.applyConfig()
        d.addViewInputs(s, c, inputs_of(v), high_spp, high_frames)
        r.removeScene(s)
        if log and (v - first + 1) % 200 == 0:
            log(f"training views: {v - first + 1} of {count} ({time.perf_counter() - t0:.0f} s)")
    return time.perf_counter() - t0


def add_icosphere_views(r: api.Kuafu, cfg: api.Config, d: api.Denoiser, count: int, size: int, full_w: int,
                        full_h: int, inputs_of, high_spp: int, high_frames: int, spheres: int = 256, log=None) -> float:
    """Adds `count` training views of icosphere scenes (scenes.icospheres with `spheres`
    level-4 spheres, seed 20000 + v: placements, materials and lights vary) through
    size x size windows of their full_w x full_h 60-degree view, rendered at depth 8 with
    Russian roulette as the icosphere workload is, then restores cfg's depth and roulette;
    each scene is removed once its pairs are stored. The renderer's geometry and instance
    limits must admit `spheres` of each (train_network sets 264). Returns the seconds taken."""
    rng = scenes.SplitMix64(0x1C05F00D)
    t0 = time.perf_counter()
    depth_before, rr_before = cfg.getPathDepth(), cfg.getRussianRoulette()
    cfg.setPathDepth(8)
    cfg.setRussianRoulette(True)
    try:
        for v in range(count):
            s = r.createScene()
            c = scenes.icospheres(r, size, size, count=spheres, level=4, seed=20000 + v, scene=s)
            x0 = min(full_w - size, int(rng.uniform() * (full_w - size + 1)))
            y0 = min(full_h - size, int(rng.uniform() * (full_h - size + 1)))
            window_camera(c, size, full_w, full_h, x0, y0, fov_deg=60.0)
            cfg.setSeed(70000 + v)
            r.applyConfig()
            d.addViewInputs(s, c, inputs_of(v), high_spp, high_frames)
            r.removeScene(s)
            if log and (v + 1) % 100 == 0:
                log(f"icosphere views: {v + 1} of {count} ({time.perf_counter() - t0:.0f} s)")
    finally:
        cfg.setPathDepth(depth_before)
        cfg.setRussianRoulette(rr_before)
        r.applyConfig()
    return time.perf_counter() - t0


def _train(r: api.Kuafu, d: api.Denoiser, iters: int, batch: int, crop: int, lr: float) -> list:
    """Adam over random crops; lr x 0.1 for the last 20 % of the steps. Mean loss per tenth."""
    losses, done, chunk = [], 0, max(1, iters // 10)
    while done < iters:
        k = min(chunk, iters - done)
        losses.append(d.train(k, batch, crop, lr * (0.1 if done >= 0.8 * iters else 1.0)))
        done += k
    r.synchronize()
    return losses


def _denoised_frames(r, cfg, cam, d, spps, ref, floor, timer, flops, log, seed=9):
    """Single frames of k spp of the current scene, denoised by d: times and relMSE."""
    den = []
    for k in spps:
        cfg.setSeed(seed)
        cfg.setPerPixelSampleRate(k)
        cfg.setAccumulatingFrames(False)
        r.applyConfig()
        r.resetFrame()
        r.run()  # capture
        d.apply(cam)
        r.synchronize()
        with timer:
            r.run()
        t_render = timer.ms
        noisy = r.downloadAov(cam, N.KF_AOV_RADIANCE_F32)
        with timer:
            d.apply(cam)
        t_dn = timer.ms
        out = r.downloadAov(cam, N.KF_AOV_DENOISED_F32)
        e_n = _gpu_relmse(r, noisy, ref)
        e_d = _gpu_relmse(r, out, ref)
        den.append({"spp": k, "render_ms": t_render, "denoise_ms": t_dn, "ms": t_render + t_dn,
                    "relmse_noisy": e_n, "relmse": e_d, "relmse_debiased": e_d - floor,
                    "denoise_tflops": flops / (t_dn / 1e3) / 1e12})
        log(f"denoised {k} spp: noisy {e_n:.3e} -> {e_d:.3e} ({t_render:.1f} + {t_dn:.1f} ms)")
    return den


def _plain_curve(r, cfg, cam, ref, floor, timer, frame_spp, checkpoint_step, max_spp, tau_min, seed=7):
    """Plain accumulation of frame_spp-sample frames into the FP64 sum (seed `seed`): the
    cumulative CUDA-event time of the frames and the relMSE of the running mean against
    ref at powers of two up to 1024 spp, then every checkpoint_step spp, until the relMSE
    is at most tau_min or max_spp is reached (the evaluations are not timed). Returns
    (checkpoints, samples accumulated)."""
    cfg.setSeed(seed)
    cfg.setPerPixelSampleRate(frame_spp)
    cfg.setAccumulatingFrames(True)
    cfg.setUseDenoiser(False)
    r.applyConfig()
    r.run()  # graph capture outside the timed frames; the reset below discards this frame
    r.synchronize()
    r.resetFrame()
    plain = []
    t_ms, spp = 0.0, 0
    next_cp = frame_spp
    while spp < max_spp:
        with timer:
            r.run()
        t_ms += timer.ms
        spp += frame_spp
        if spp >= next_cp:
            e = _gpu_relmse(r, _fp64_mean(r, cam), ref)
            plain.append({"spp": spp, "ms": t_ms, "relmse": e, "relmse_debiased": e - floor})
            next_cp = next_cp * 2 if next_cp < 1024 else next_cp + checkpoint_step
            if e <= tau_min:
                break
    return plain, spp


def _time_to(plain, den, thresholds):
    """For each threshold: measured plain time, denoised time, ratio (raw and debiased relMSE)."""
    ttr = []
    for tau in thresholds:
        row = {"tau": tau}
        for key in ("relmse", "relmse_debiased"):
            hit = next((p for p in plain if p[key] <= tau), None)
            pt, how = (hit["ms"], "measured") if hit is not None else (None, "not reached")
            dh = [p for p in den if p[key] <= tau]
            dt = min(p["ms"] for p in dh) if dh else None
            dk = min((p for p in dh), key=lambda p: p["ms"])["spp"] if dh else None
            row[key] = {"plain_ms": pt, "plain": how, "plain_spp": hit["spp"] if hit else None, "denoised_ms": dt,
                        "denoised_input_spp": dk, "speedup": (pt / dt) if (pt and dt) else None}
        ttr.append(row)
    return ttr


def run(width=1920, height=1080, ref_spp=40960, ref_frame_spp=256, plain_frame_spp=8, plain_checkpoint_step=2048,
        plain_max_spp=65536, train_views=66, train_size=256, train_high_spp=64,
        train_high_frames=64, train_iters=6000, train_batch=12, train_crop=128, lr=1e-3,
        denoise_spps=(1, 2, 4, 8, 16, 32, 64, 128, 256, 512, 1024), thresholds=(1e-1, 3e-2, 1e-2, 3e-3, 1e-3),
        depth=5, shipped=None, save_trained=None, more_networks=None, log=print) -> dict:
    cfg = scenes.cornell_config(spp=ref_frame_spp, depth=depth)
    res = {"scene": "cornell", "width": width, "height": height, "depth": depth, "eps": EPS}
    with api.Kuafu(cfg) as r:
        scene = r.getScene()
        cam = scenes.cornell(r, width, height, scene=scene)
        # 1. reference halves
        t0 = time.perf_counter()
        a = _accumulate(r, cfg, cam, 1001, ref_spp // 2, ref_frame_spp)
        b = _accumulate(r, cfg, cam, 1002, ref_spp // 2, ref_frame_spp)
        ref = 0.5 * (a + b)
        floor = _gpu_relmse(r, a, b) / 4.0
        res["reference"] = {"spp": ref_spp, "accumulation": "fp64", "halves_relmse": 4.0 * floor,
                            "ref_floor": floor, "seconds": time.perf_counter() - t0}
        log(f"reference {ref_spp} spp: floor {floor:.4e} ({time.perf_counter() - t0:.1f} s)")
        del a, b

        # 2. plain accumulation (FP64 sum of equal frames), measured until the smallest
        #    threshold is reached
        timer = _Timer(r)
        plain, spp = _plain_curve(r, cfg, cam, ref, floor, timer, plain_frame_spp, plain_checkpoint_step,
                                  plain_max_spp, min(thresholds))
        s64 = r.downloadAov(cam, N.KF_AOV_SUM_F64)
        res["plain"] = plain
        res["plain_check"] = {"frames_in_fp64_sum": float(s64[..., 3].max()), "spp": spp}
        log("plain: " + ", ".join(f"{p['spp']}spp {p['relmse']:.3e}" for p in plain))
        ms_per_spp = plain[-1]["ms"] / plain[-1]["spp"]
        res["plain_fit"] = {"ms_per_spp": ms_per_spp}

        # 3. denoiser training on Cornell variations seen through train_size windows of
        #    the width x height view
        d = api.Denoiser(r, seed=0)
        t_data = add_training_views(r, cfg, d, train_views, train_size, width, height,
                                    lambda v: [denoise_spps[v % len(denoise_spps)],
                                               denoise_spps[(v + 5) % len(denoise_spps)]], train_high_spp,
                                    train_high_frames)
        t0 = time.perf_counter()
        losses = _train(r, d, train_iters, train_batch, train_crop, lr)
        t_train = time.perf_counter() - t0
        res["training"] = {"views": train_views, "size": train_size, "windows_of": [width, height],
                           "input_spp": list(denoise_spps), "target_spp": train_high_spp * train_high_frames,
                           "iters": train_iters, "batch": train_batch, "crop": train_crop, "lr": lr,
                           "loss_curve": losses, "data_seconds": t_data, "train_seconds": t_train}
        log(f"training: data {t_data:.1f} s, {train_iters} iters {t_train:.1f} s, loss {losses[0]:.4f} -> "
            f"{losses[-1]:.4f}")
        if save_trained:
            d.save(save_trained)

        # 4. denoised single frames of the held-out scene
        r.setScene(scene)
        flops = unet_flops(height, width)
        den = _denoised_frames(r, cfg, cam, d, denoise_spps, ref, floor, timer, flops, log)
        res["denoised"] = den
        res["denoiser_flops_per_frame"] = flops
        d.close()
        # the network shipped with the package (trained by train_network), same frames
        if shipped:
            d2 = api.Denoiser(r, seed=0)
            d2.load(shipped)
            log("shipped network:")
            den2 = _denoised_frames(r, cfg, cam, d2, denoise_spps, ref, floor, timer, flops, log)
            res["shipped"] = {"weights": str(shipped), "denoised": den2,
                              "time_to_relmse": _time_to(plain, den2, thresholds)}
            d2.close()
        for name, path in (more_networks or {}).items():
            d3 = api.Denoiser(r, seed=0)
            d3.load(path)
            log(f"{name} network:")
            den3 = _denoised_frames(r, cfg, cam, d3, denoise_spps, ref, floor, timer, flops, log)
            res.setdefault("networks", {})[name] = {"weights": str(path), "denoised": den3,
                                                    "time_to_relmse": _time_to(plain, den3, thresholds)}
            d3.close()

    # 5. time to each threshold: measured on both arms, raw relMSE (debiased beside it)
    res["time_to_relmse"] = _time_to(plain, den, thresholds)
    floor_4096 = floor * ref_spp / 4096.0  # the floor falls as 1 / spp
    res["note_4096spp_reference"] = (
        f"against a 4096-spp reference the floor would be about {floor_4096:.2e} (the relMSE of an independent "
        f"estimate includes the reference's own noise), so nothing could be measured below 1e-3 against it; the "
        f"reference here has {ref_spp} spp")
    return res


def train_network(path, views=2000, size=256, full_w=1920, full_h=1080, base_spp=4,
                  extra_spps=(1, 2, 8, 16, 32, 64, 128, 256, 512, 1024), high_spp=256, high_frames=16, iters=10000,
                  batch=16, crop=128, lr=1e-3, depth=5, seed=0, icosphere_views=0, log=print) -> dict:
    """Trains the network shipped with the package and saves it to `path`.

    Training set: `views` Cornell variations, each a size x size window of the
    full_w x full_h view (window_camera), with two inputs — one frame of `base_spp`
    samples and one of extra_spps[v % len] — sharing one target of high_frames x
    high_spp samples from the FP64 accumulation (defaults: 2000 crops of 256x256,
    4-spp inputs, 4096-spp targets; the second input covers the 1..1024-spp frames the
    time-to-relMSE experiment denoises). `icosphere_views` > 0 adds that many windows of
    seeded icosphere scenes (add_icosphere_views) with the same inputs and targets.
    Adam over random crop x crop crops."""
    cfg = scenes.cornell_config(spp=high_spp, depth=depth)
    if icosphere_views:
        cfg.setGeometryLimit(264)
        cfg.setGeometryInstanceLimit(264)
    with api.Kuafu(cfg) as r:
        d = api.Denoiser(r, seed=seed)
        t_data = add_training_views(r, cfg, d, views, size, full_w, full_h,
                                    lambda v: [base_spp, extra_spps[v % len(extra_spps)]], high_spp, high_frames,
                                    log=log)
        if icosphere_views:
            t_data += add_icosphere_views(r, cfg, d, icosphere_views, size, full_w, full_h,
                                          lambda v: [base_spp, extra_spps[v % len(extra_spps)]], high_spp,
                                          high_frames, log=log)
        log(f"{d.numViews()} training pairs from {views + icosphere_views} views in {t_data:.0f} s")
        t0 = time.perf_counter()
        losses = _train(r, d, iters, batch, crop, lr)
        t_train = time.perf_counter() - t0
        log(f"{iters} Adam steps in {t_train:.0f} s, loss {losses[0]:.4f} -> {losses[-1]:.4f}")
        d.save(path)
        d.close()
    return {"views": views, "icosphere_views": icosphere_views, "pairs": 2 * (views + icosphere_views), "size": size,
            "windows_of": [full_w, full_h],
            "input_spp": [base_spp] + list(extra_spps), "target_spp": high_spp * high_frames, "iters": iters,
            "batch": batch, "crop": crop, "lr": lr, "loss_curve": losses, "data_seconds": t_data,
            "train_seconds": t_train}


def icosphere_eval(networks: dict, width=1920, height=1080, ref_spp=8192, ref_frame_spp=32, plain_frame_spp=8,
                   plain_checkpoint_step=512, plain_max_spp=16384, spps=(1, 4, 8, 32, 128),
                   thresholds=(1e-1, 3e-2, 1e-2, 3e-3, 1e-3), log=print) -> dict:
    """The networks (name -> parameter file) on the 256-icosphere scene of seed 0 (glossy,
    metallic and transmissive spheres, 7 lights, RR, depth 8) at width x height: content the
    Cornell-trained networks never saw; a network trained with add_icosphere_views saw
    scenes of other seeds. Reference: two FP64 accumulations of ref_spp / 2 (floor as in
    run()). Plain accumulation of 8-spp frames (seed 7) is measured against the same
    reference until its relMSE reaches the smallest threshold (as in run()), and each
    network's denoised frames give a time to each threshold."""
    cfg = scenes.icosphere_config(spp=ref_frame_spp, depth=8)
    cfg.setRussianRoulette(True)
    out = {"scene": f"256 icospheres {width}x{height} depth 8", "reference_spp": ref_spp}
    with api.Kuafu(cfg) as r:
        cam = scenes.icospheres(r, width, height)
        a = _accumulate(r, cfg, cam, 2001, ref_spp // 2, ref_frame_spp)
        b = _accumulate(r, cfg, cam, 2002, ref_spp // 2, ref_frame_spp)
        ref = 0.5 * (a + b)
        floor = _gpu_relmse(r, a, b) / 4.0
        out["ref_floor"] = floor
        log(f"icosphere reference {ref_spp} spp: floor {floor:.3e}")
        del a, b
        timer = _Timer(r)
        plain, _ = _plain_curve(r, cfg, cam, ref, floor, timer, plain_frame_spp, plain_checkpoint_step,
                                plain_max_spp, min(thresholds))
        out["plain"] = plain
        log("icosphere plain: " + ", ".join(f"{p['spp']}spp {p['relmse']:.3e}" for p in plain))
        flops = unet_flops(height, width)
        for name, path in networks.items():
            d = api.Denoiser(r, seed=0)
            d.load(path)
            log(f"{name} network on the icosphere scene:")
            den = _denoised_frames(r, cfg, cam, d, spps, ref, floor, timer, flops, log)
            out[name] = [{k: p[k] for k in ("spp", "ms", "relmse_noisy", "relmse", "relmse_debiased")} for p in den]
            out[name + "_time_to_relmse"] = _time_to(plain, den, thresholds)
            d.close()
    return out


SMALL = dict(width=480, height=272, ref_spp=4096, plain_max_spp=8192, plain_checkpoint_step=512, train_views=18, train_iters=300,
             train_crop=96, train_high_frames=16)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--small", action="store_true", help="a reduced run (480x272, shorter training)")
    ap.add_argument("--json", default=None)
    ap.add_argument("--train-iters", type=int, default=None)
    ap.add_argument("--ref-spp", type=int, default=None)
    ap.add_argument("--train-network", metavar="PATH", default=None,
                    help="train the shipped network (2000 windows of 256x256, 4-spp inputs, 4096-spp targets) "
                         "and save it to PATH instead of running the experiment")
    ap.add_argument("--views", type=int, default=2000, help="training views of --train-network")
    ap.add_argument("--icosphere-views", type=int, default=0,
                    help="training views of icosphere scenes added to --train-network's Cornell views")
    a = ap.parse_args(argv)
    if a.train_network:
        kw = {"views": a.views, "icosphere_views": a.icosphere_views}
        if a.train_iters:
            kw["iters"] = a.train_iters
        res = train_network(a.train_network, **kw)
        s = json.dumps(res)
        if a.json:
            with open(a.json, "w") as f:
                f.write(s)
        print(s)
        return
    kw = dict(SMALL) if a.small else {}
    if a.train_iters:
        kw["train_iters"] = a.train_iters
    if a.ref_spp:
        kw["ref_spp"] = a.ref_spp
    res = run(**kw)
    s = json.dumps(res)
    if a.json:
        with open(a.json, "w") as f:
            f.write(s)
    print(s)


if __name__ == "__main__":
    main()
