"""tcgen05 tensor-core kernels of the denoiser against PyTorch FP32 references.

The kernels take BF16 operands and accumulate in FP32; the reference evaluates the
same BF16-rounded operands in FP32. Tolerances: GEMM (FP32 output) 1e-4 of the
output scale; convolution (BF16 output) 1e-2 of the output scale (BF16 keeps 8
significant bits).
"""
import ctypes as C

import pytest

from kuafu_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _tc_error():
    e = C.c_uint32()
    N.check(N.load().kf_tc_error(C.byref(e)))
    return e.value


@pytest.mark.parametrize("n,h,w,cin,cout,rows,relu,cstride,coff", [
    # narrow images: one CTA per 128-pixel tile, 9 tap-shifted boxes per chunk
    (2, 20, 24, 64, 40, 48, True, 40, 0),
    (3, 8, 8, 96, 160, 160, True, 160, 0),
    (1, 33, 17, 32, 288, 288, False, 288, 0),
    # images at least 128 wide: the persistent halo kernel (rows per tile R, channel
    # chunk CK, resident or streamed weights, ragged last tile in x and y, channel slices,
    # 1 to 3 output rows per MMA)
    (1, 9, 150, 32, 32, 32, False, 96, 32),     # R 4, CK 32, resident weights
    (2, 7, 200, 96, 32, 32, True, 32, 0),       # 3 streamed chunks of 32
    (1, 10, 131, 64, 64, 64, True, 160, 96),    # CK 16, 4 chunks
    (1, 5, 256, 160, 160, 160, True, 160, 0),   # R 1, n 160, one row per MMA
    (1, 6, 130, 32, 80, 80, True, 80, 0),       # R 2, n 80: three output rows per MMA (N 240)
    (1, 9, 140, 16, 32, 32, True, 32, 0),       # 16 input channels (the inference input layer)
    (1, 6, 140, 32, 288, 288, False, 288, 0),   # three 128-row slices of the weights
    (2, 3, 128, 64, 40, 48, False, 40, 0),      # N 48, output channels not a multiple of 8
    (1, 13, 384, 96, 224, 224, True, 224, 0),   # no halo shape fits: falls back to the tile kernel
])
def test_conv3x3_matches_torch(n, h, w, cin, cout, rows, relu, cstride, coff):
    import torch

    lib = N.load()
    g = torch.Generator(device="cuda").manual_seed(n * 1000 + h)
    x = torch.randn((n, h, w, cin), device="cuda", generator=g).to(torch.bfloat16)
    wt = (torch.randn((9, rows, cin), device="cuda", generator=g) * 0.1).to(torch.bfloat16)
    bias = torch.randn((rows,), device="cuda", generator=g, dtype=torch.float32)
    y = torch.zeros((n, h, w, cstride), device="cuda", dtype=torch.bfloat16)
    torch.cuda.synchronize()
    N.check(lib.kf_conv3x3_bf16(x.data_ptr(), n, h, w, cin, wt.data_ptr(), rows, bias.data_ptr(), cout, int(relu),
                                y.data_ptr(), cstride, coff, torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert _tc_error() == 0
    # reference: tap = ky * 3 + kx reads x[y + ky - 1, x + kx - 1]  (cross-correlation, padding 1)
    wr = wt.float()[:, :cout, :].permute(1, 2, 0).reshape(cout, cin, 3, 3)
    ref = torch.nn.functional.conv2d(x.float().permute(0, 3, 1, 2), wr, bias[:cout], padding=1)
    if relu:
        ref = torch.relu(ref)
    ref = ref.permute(0, 2, 3, 1)
    got = y[..., coff:coff + cout].float()
    scale = ref.abs().max().item() + 1e-6
    err = (got - ref).abs().max().item() / scale
    assert err < 1e-2, f"max error {err:.3e} of scale {scale:.3e}"
    # channels outside the slice are untouched
    if cstride > cout:
        rest = torch.cat([y[..., :coff], y[..., coff + cout:]], dim=-1)
        assert (rest == 0).all()


@pytest.mark.parametrize("m,n,k,splits", [(200, 96, 4096, 4), (128, 32, 64, 1), (77, 160, 1000, 3)])
def test_gemm_tn_matches_torch(m, n, k, splits):
    import torch

    lib = N.load()
    g = torch.Generator(device="cuda").manual_seed(m + n + k)
    a = torch.randn((m, k), device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn((n, k), device="cuda", generator=g).to(torch.bfloat16)
    d = torch.zeros((m, n), device="cuda", dtype=torch.float32)
    torch.cuda.synchronize()
    N.check(lib.kf_gemm_bf16_tn(a.data_ptr(), m, b.data_ptr(), n, k, d.data_ptr(), n, splits,
                                torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert _tc_error() == 0
    ref = a.float() @ b.float().T
    err = (d - ref).abs().max().item() / (ref.abs().max().item() + 1e-6)
    assert err < 1e-4, f"max error {err:.3e}"


def test_bounded_wait_gives_up_reports_and_leaves_the_context_usable():
    """The tensor-core kernels' bounded wait, made to run out: a kernel waits on an mbarrier
    that nothing arrives on with a budget of 2e6 SM cycles (about 1 ms). It gives up, and
    the error word reads 99 once, then 0. The context stays usable: a convolution run after
    it matches the PyTorch reference."""
    import torch

    lib = N.load()
    _tc_error()  # start from a clear error word
    N.check(lib.kf_tc_wait_probe(2_000_000, torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert _tc_error() == 99
    assert _tc_error() == 0
    test_conv3x3_matches_torch(1, 6, 130, 32, 80, 80, True, 80, 0)
