"""The allocation-free CFL entry point (cans_cfl_m3_2d_noalloc).

It serves callers that cannot allocate device memory: they already hold the
state in device memory and the library must take nothing from the device
allocator, so its reduction scratch is a fixed array in device memory shared
by every call.  These tests call it through the C ABI and compare it with the
ordinary cans_cfl_m3_2d on the same data, on two calls in a row (a large grid
first, then a small one, so the second call runs over scratch the first one
left behind).  This file is collected last so that a failure here stops a
-x run only after every other test has run.
"""
import numpy as np
import pytest

from utrip_gb300 import capi, setups

pytestmark = pytest.mark.gpu


def _device_copy(torch, a):
    # the caller's own device memory, column-major like the host arrays
    return torch.from_numpy(np.ascontiguousarray(np.ravel(a, order="F"))).cuda()


@pytest.mark.parametrize("exact", [True, False])
def test_noalloc_cfl_matches_cfl_m3_on_two_calls(gpu, exact):
    torch = pytest.importorskip("torch")
    gpu.set_exact(exact)
    try:
        for s in (setups.random_state(300, 260, seed=31), setups.orszag_tang(64)):
            st = s["state"]
            ref_dt, ref_merr = gpu.cfl_m3(0.4, 1e-10, s["gm"], *st[:8], s["dx"], s["dy"])
            dev = [_device_copy(torch, a) for a in st[:8]]
            ddx, ddy = _device_copy(torch, s["dx"]), _device_copy(torch, s["dy"])
            torch.cuda.synchronize()
            dt, merr = gpu.cfl_m3_noalloc(0.4, 1e-10, s["gm"], [t.data_ptr() for t in dev],
                                          ddx.data_ptr(), ddy.data_ptr(), *st[0].shape)
            # exact policy: the same operations, so the same bits; fast
            # policy: the compiler may contract differently in the two
            # kernels, so within a relative 1e-13 (well inside the 1e-10 the
            # fast policy is held to)
            assert merr == ref_merr == 0
            if exact:
                assert dt == ref_dt
            else:
                assert abs(dt - ref_dt) <= 1e-13 * ref_dt
            _, merr = gpu.cfl_m3_noalloc(0.4, 1.0, s["gm"], [t.data_ptr() for t in dev],
                                         ddx.data_ptr(), ddy.data_ptr(), *st[0].shape)
            assert merr == 9001
    finally:
        gpu.set_exact(False)


@pytest.mark.parametrize("exact", [True, False])
def test_noalloc_cfl_at_and_past_one_fold_block(gpu, exact):
    """Grids whose partials the final fold walks in strides of 1024: one at
    the scratch limit (1024 x 1024 cells, 4096 partials) and one just over
    1024 partials (600 x 440 cells, 1032), each against cans_cfl_m3_2d, on
    two calls in a row."""
    torch = pytest.importorskip("torch")
    gpu.set_exact(exact)
    try:
        for ix, jx in ((1024, 1024), (600, 440)):
            s = setups.random_state(ix, jx, seed=ix + jx)
            st = s["state"]
            ref_dt, ref_merr = gpu.cfl_m3(0.4, 1e-10, s["gm"], *st[:8], s["dx"], s["dy"])
            dev = [_device_copy(torch, a) for a in st[:8]]
            ddx, ddy = _device_copy(torch, s["dx"]), _device_copy(torch, s["dy"])
            torch.cuda.synchronize()
            dt, merr = gpu.cfl_m3_noalloc(0.4, 1e-10, s["gm"], [t.data_ptr() for t in dev],
                                          ddx.data_ptr(), ddy.data_ptr(), ix, jx)
            assert merr == ref_merr == 0
            if exact:
                assert dt == ref_dt
            else:
                assert abs(dt - ref_dt) <= 1e-13 * ref_dt
    finally:
        gpu.set_exact(False)


def test_noalloc_rejects_grids_beyond_its_scratch(gpu):
    # 1025 x 1025 cells exceed the fixed scratch (1,048,576 cells); the call
    # is refused on the host before any device work
    with pytest.raises(capi.CansError) as e:
        gpu.cfl_m3_noalloc(0.4, 1e-10, 5.0 / 3.0, [8] * 8, 8, 8, 1025, 1025)
    assert e.value.code == capi.CANS_ERR_ARG
