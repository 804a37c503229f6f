"""The allocation-free step-size entry point, through the C ABI.

uppe_step_size_noalloc serves callers that may not allocate device memory once they run, such as
a host program that reserves all GPU memory at start-up.  It must give the same step size as
the handle's adaptive RK4 step, which reduces over work buffers it allocated itself.  This file sorts
last so that a run stopping at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

import replay

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from searay_gb300 import _native, build
    build.build()
    return _native.lib()


def _setup(name):
    from searay_gb300 import grid, ionization, uppe
    vd, _ = replay.load_case(name)
    g = grid.VolumeGrid(vd)
    rates = ionization.RateCoefficients(vd["ionizer"]) if vd.get("ionizer") else None
    dev = uppe.DeviceGrid(g, vd, rates, "mixed")
    chi = vd["dispersion inside"].chi(g.w).astype(np.cdouble)
    mat = uppe.Material(dev, g, vd["wave coordinates"], None, chi, vd.get("chi3", 0.0), vd["density reference"],
                        vd.get("window speed", 1.0), vd["density lambda"])
    return vd, g, dev, mat


@pytest.mark.parametrize("name", ["cart_ion", "cyl_kerr"])
def test_noalloc_step_size_matches_handle(lib, name):
    import torch
    from searay_gb300 import _native
    vd, g, dev, mat = _setup(name)
    z = 777.0
    L = 5.0e5  # long subcycle: the estimate stays below L, so neither path clamps
    mat.UpdateMaterial(z)
    a = torch.from_numpy(vd["incoming wave"](g.w, g.x1, g.x2).astype(np.complex64)).cuda()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):  # two calls in a row share the scratch array
        dev.load_field(a)
        q = dev.empty_field()
        dev.get_field(q)
        S = dev.empty_field()
        dev.eval_rhs(q, z, S)
        dz_dev = torch.full((1,), -1.0, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        free0, alloc0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
        rc = lib.uppe_step_size_noalloc(ctypes.c_void_p(q.data_ptr()), ctypes.c_void_p(S.data_ptr()),
                                        q.numel(), L, 0.4, 1e-2, ctypes.c_void_p(dz_dev.data_ptr()), stream)
        assert rc == 0, lib.uppe_last_error(None)
        torch.cuda.synchronize()
        if call > 0:  # after the first call on the device (which loads the module), nothing is allocated
            assert torch.cuda.mem_get_info()[0] == free0
            assert torch.cuda.memory_allocated() == alloc0
        dz_noalloc = float(dz_dev.item())
        # the handle path: adaptive RK4 step from the same q at the same z (dzmin 0, no clamp hit)
        dz_handle = dev.rk4_step(z, L, 0.0, 0.0)
        assert 0.0 < dz_noalloc < L
        assert dz_noalloc == pytest.approx(dz_handle, rel=1e-6), (call, dz_noalloc, dz_handle)
    dev.close()


def test_noalloc_reports_nonfinite_field(lib):
    import torch
    q = torch.ones(3 * 8192 + 5, dtype=torch.complex64, device="cuda")
    S = torch.full_like(q, 0.5 + 0.25j)
    out = torch.zeros(1, dtype=torch.float32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def call():
        rc = lib.uppe_step_size_noalloc(ctypes.c_void_p(q.data_ptr()), ctypes.c_void_p(S.data_ptr()), q.numel(),
                                        10.0, 0.4, 1e-2, ctypes.c_void_p(out.data_ptr()), stream)
        assert rc == 0, lib.uppe_last_error(None)
        return float(out.item())

    assert np.isfinite(call())
    S[2 * 8192 + 3] = float("nan")
    assert np.isnan(call())
    S[2 * 8192 + 3] = 0.5
    q[7] = float("inf")
    assert np.isnan(call())
    q[7] = 1.0
    assert np.isfinite(call())


def test_noalloc_rejects_oversize_and_bad_arguments(lib):
    import torch
    from searay_gb300 import _native
    buf = torch.zeros(4, dtype=torch.complex64, device="cuda")
    out = torch.zeros(1, dtype=torch.float32, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    o = ctypes.c_void_p(out.data_ptr())
    rc = lib.uppe_step_size_noalloc(p, p, _native.NOALLOC_MAX_POINTS + 1, 1.0, 0.4, 1e-2, o, None)
    assert rc == _native.UPPE_E_RANGE
    assert b"scratch limit" in lib.uppe_last_error(None)
    assert lib.uppe_step_size_noalloc(p, p, 0, 1.0, 0.4, 1e-2, o, None) == _native.UPPE_E_ARG
    assert lib.uppe_step_size_noalloc(None, p, 4, 1.0, 0.4, 1e-2, o, None) == _native.UPPE_E_ARG
