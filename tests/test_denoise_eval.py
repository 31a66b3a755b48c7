"""Host-side arithmetic of the time-to-relMSE experiment (kuafu_gb300.denoise_eval)."""
import pytest

from kuafu_gb300 import denoise_eval as E


def test_time_to_threshold_takes_the_first_measured_plain_point_and_the_fastest_denoised_frame():
    plain = [{"spp": 8, "ms": 10.0, "relmse": 0.5, "relmse_debiased": 0.4},
             {"spp": 16, "ms": 20.0, "relmse": 0.2, "relmse_debiased": 0.1},
             {"spp": 32, "ms": 40.0, "relmse": 0.09, "relmse_debiased": 0.05}]
    den = [{"spp": 1, "ms": 2.0, "relmse": 0.3, "relmse_debiased": 0.25},
           {"spp": 2, "ms": 3.0, "relmse": 0.08, "relmse_debiased": 0.06},
           {"spp": 4, "ms": 5.0, "relmse": 0.05, "relmse_debiased": 0.03}]
    rows = E._time_to(plain, den, (0.1, 0.06, 0.01))
    r = rows[0]["relmse"]
    assert (r["plain_ms"], r["plain_spp"], r["denoised_ms"], r["denoised_input_spp"]) == (40.0, 32, 3.0, 2)
    assert r["speedup"] == pytest.approx(40.0 / 3.0) and r["plain"] == "measured"
    d = rows[0]["relmse_debiased"]  # debiased: 16 spp already reaches 0.1
    assert (d["plain_ms"], d["plain_spp"]) == (20.0, 16)
    r = rows[1]["relmse"]  # 0.06: no plain point reaches it, the 4-spp frame does
    assert r["plain"] == "not reached" and r["plain_ms"] is None and r["speedup"] is None
    assert r["denoised_input_spp"] == 4
    r = rows[2]["relmse"]  # 0.01: neither arm
    assert r["denoised_ms"] is None and r["speedup"] is None


def test_unet_flops_counts_the_executed_layers():
    # 1080p: padded to 1088 x 1920, the first convolution takes 16 input channels
    full = E.unet_flops(1080, 1920)
    per_px = sum(2 * ci * co * 9 / 4 ** lv for ci, co, lv in E._LAYERS)
    first_32 = 2 * 32 * 32 * 9
    first_16 = 2 * 16 * 32 * 9
    assert full == pytest.approx(1088 * 1920 * (per_px - first_32 + first_16))
    # narrow frames (below 96 padded pixels) keep the 32-channel first layer
    assert E.unet_flops(64, 80) == pytest.approx(64 * 80 * per_px)


def test_plain_curve_checkpoints_and_stops_at_the_threshold(monkeypatch):
    """Plain accumulation checkpoints at powers of two up to 1024 spp, then every
    checkpoint_step spp; it stops at the first checkpoint at or below tau_min, and the
    time is the sum of the timed frames (evaluations untimed)."""

    class FakeRenderer:
        frames = 0

        def applyConfig(self):
            pass

        def run(self):
            self.frames += 1

        def synchronize(self):
            pass

        def resetFrame(self):
            self.frames = 0

    class FakeConfig:
        def __getattr__(self, name):
            return lambda *a: None

    class FakeTimer:
        ms = 2.0

        def __enter__(self):
            return self

        def __exit__(self, *a):
            pass

    r = FakeRenderer()
    # relMSE of the running mean falls as 8 / spp
    monkeypatch.setattr(E, "_fp64_mean", lambda rr, cam: rr.frames * 8)
    monkeypatch.setattr(E, "_gpu_relmse", lambda rr, spp, ref: 8.0 / spp)
    plain, spp = E._plain_curve(r, FakeConfig(), None, None, 1e-3, FakeTimer(), 8, 512, 65536, 8.0 / 2560)
    assert [p["spp"] for p in plain] == [8, 16, 32, 64, 128, 256, 512, 1024, 1536, 2048, 2560]
    assert spp == 2560 and plain[-1]["ms"] == 2.0 * 2560 / 8
    assert plain[-1]["relmse_debiased"] == 8.0 / 2560 - 1e-3
    # never reached: stops at max_spp
    plain, spp = E._plain_curve(r, FakeConfig(), None, None, 0.0, FakeTimer(), 8, 512, 256, 1e-9)
    assert spp == 256 and plain[-1]["spp"] == 256
