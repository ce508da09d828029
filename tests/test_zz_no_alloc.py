"""The allocation-free render entry point against rt_render_device (gpu).

rt_render_device_noalloc renders out of one fixed device array instead of
allocating.  It runs the same kernels with the same per-pixel summation order
as rt_render_device, so the tolerance is zero: every float of the film must
match.  Two calls in a row reuse the array with different crops, seeds and
integrators, so state left over from the previous call would show.  The file
name makes pytest collect it last; it also passes alone in a fresh process.
A call after the first also leaves the device's free memory and the library's
count of device allocations unchanged: it allocates nothing.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from radiantium_gb300 import native as N
from radiantium_gb300 import procedural
from radiantium_gb300.device import Device

pytestmark = pytest.mark.gpu

TOLERANCE_ULP = 0   # bit-identical films


def _device_allocations(dev):
    """The library's process-wide count of device allocations (a test hook)."""
    n = C.c_ulonglong()
    f = dev.lib.rt_debug_device_allocations
    f.argtypes = [C.POINTER(C.c_ulonglong)]
    f.restype = C.c_int
    assert f(C.byref(n)) == 0
    return n.value


def _film(fn, settings, w, h):
    out = torch.full((w * h * 3,), float("nan"), dtype=torch.float32, device="cuda:0")
    torch.cuda.synchronize()
    fn(settings, out.data_ptr())
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _assert_same(a, b):
    assert np.isfinite(a).all()
    diff = np.abs(a.view(np.int32).astype(np.int64) - b.view(np.int32).astype(np.int64))
    assert diff.max() <= TOLERANCE_ULP, f"{np.count_nonzero(diff)} floats differ, max {diff.max()} ulp"


@pytest.fixture(scope="module")
def scenes():
    cb, cb_st = procedural.cornell_box(96, 80)
    vb, vb_st = procedural.volume_box(40, 40)
    d_cb, d_vb = Device(0), Device(0)
    d_cb.upload(cb)
    d_vb.upload(vb)
    yield (d_cb, cb_st), (d_vb, vb_st)
    d_cb.close()
    d_vb.close()


def test_noalloc_matches_render_device_on_consecutive_calls(scenes):
    (d_cb, cb_st), (d_vb, vb_st) = scenes
    calls = [
        (d_cb, cb_st.replace(spp=6, seed=11, x0=8, y0=4, width=80, height=70), 80, 70),
        (d_cb, cb_st.replace(spp=3, seed=12, x0=0, y0=0, width=32, height=24, method=N.METHOD_NEE), 32, 24),
        (d_vb, vb_st.replace(spp=4, seed=5), 40, 40),
    ]
    for d, st, w, h in calls:
        want = _film(d.render_device, st, w, h)
        got = _film(d.render_device_noalloc, st, w, h)
        _assert_same(got, want)
        again = _film(d.render_device_noalloc, st, w, h)
        _assert_same(again, want)


def test_noalloc_second_call_allocates_nothing(scenes):
    """The property the entry point exists for: once the scratch array is set
    up, a call takes no device memory (cudaMemGetInfo) and makes no allocation."""
    (d_cb, cb_st), _ = scenes
    st = cb_st.replace(spp=5, seed=3, x0=4, y0=2, width=64, height=60)
    out = torch.empty(64 * 60 * 3, dtype=torch.float32, device="cuda:0")
    d_cb.render_device_noalloc(st, out.data_ptr())              # sets the scratch array up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    n0 = _device_allocations(d_cb)
    for seed in (4, 5):
        d_cb.render_device_noalloc(st.replace(seed=seed), out.data_ptr())
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert _device_allocations(d_cb) == n0
    assert free1 == free0, (free0, free1)
    assert torch.isfinite(out).all()


def test_noalloc_rejects_crop_over_scratch(scenes):
    (d_cb, cb_st), _ = scenes
    big = procedural.cornell_box(2048, 1024)[0]
    d = Device(0)
    try:
        d.upload(big)
        out = torch.empty(3, dtype=torch.float32, device="cuda:0")
        with pytest.raises(N.RTError) as e:
            d.render_device_noalloc(cb_st.replace(spp=1), out.data_ptr())
        assert e.value.code == N.RT_ERR_INVALID_ARG
        assert "scratch" in str(e.value)
        # a crop that fits still renders on the same context
        st = cb_st.replace(spp=1, x0=100, y0=200, width=64, height=64)
        want = _film(d.render_device, st, 64, 64)
        got = _film(d.render_device_noalloc, st, 64, 64)
        _assert_same(got, want)
    finally:
        d.close()
