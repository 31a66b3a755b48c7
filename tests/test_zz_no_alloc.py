"""kf_relmse_noalloc: the relative-MSE reduction for callers that cannot allocate.

Some embedders cannot call cudaMalloc: their device memory belongs to their own
pool allocator, or their frame loop cannot afford the device-wide
synchronisation that cudaMalloc / cudaFree imply. kf_relmse_noalloc keeps its
scratch in a static device array instead. This test calls it through the C-ABI
twice in a row, on different data, and checks each result against kf_relmse
(which uses allocated scratch) at the FP64 tolerance the reduction tests use.
The file is named to be collected last, and it works alone in a fresh process.
"""
import ctypes as C

import pytest

from kuafu_gb300 import _native as N
from kuafu_gb300 import api, scenes

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12  # two FP64 reductions of the same terms in a different order


def test_noalloc_relmse_matches_allocating_entry_point():
    import torch

    lib = N.load()
    cfg = scenes.cornell_config()
    with api.Kuafu(cfg) as r:
        r.synchronize()
        stream = torch.cuda.current_stream()
        gen = torch.Generator(device="cuda").manual_seed(7)
        for n, eps in ((1920 * 1080, 1e-2), (300_001, 1e-3)):
            x = torch.rand((n, 4), device="cuda", generator=gen, dtype=torch.float32) * 4.0
            ref = torch.rand((n, 4), device="cuda", generator=gen, dtype=torch.float32) * 4.0
            torch.cuda.synchronize()
            want = C.c_double()
            N.check(lib.kf_relmse(r._h, x.data_ptr(), ref.data_ptr(), n, eps, C.byref(want)))
            got = C.c_double()
            N.check(lib.kf_relmse_noalloc(x.data_ptr(), ref.data_ptr(), n, eps, stream.cuda_stream, C.byref(got)))
            assert got.value == pytest.approx(want.value, rel=REL_TOL)
            # against an independent FP64 evaluation as well
            d = (x[:, :3].double() - ref[:, :3].double()) ** 2 / (ref[:, :3].double() ** 2 + eps)
            assert got.value == pytest.approx(d.mean().item(), rel=1e-9)


def test_noalloc_relmse_rejects_sizes_beyond_its_scratch():
    lib = N.load()
    got = C.c_double()
    rc = lib.kf_relmse_noalloc(C.c_void_p(16), C.c_void_p(16), 4096 * 65536 + 1, 1e-2, None, C.byref(got))
    assert rc == 3  # KF_ERR_LIMIT, before anything touches the device
    assert b"static scratch" in lib.kf_last_error()
