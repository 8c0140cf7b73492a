"""asg_flux_columns_device: the Burgers column step on device buffers with no
allocation of its own, checked against asg_flux_columns (host buffers, which
allocates per call) through the C ABI.

Collected last so it also runs after every other GPU test in the session."""
import ctypes as C

import numpy as np
import pytest

import scenarios as S
from gpu_helpers import rel

pytestmark = pytest.mark.gpu

N_COEF = 3.5 / (2 * 1540.0 ** 3 * 1000.0)
CASES = [  # (flux, extra keyword arguments)
    ("RUSANOV", {}),
    ("RUSANOV_TVD", {"beta_tvd": 1.7}),
    ("KT", {}),
    ("KT_MINMOD", {}),
    ("KT", {"cfl_target": 0.3}),
]


def _columns(ncols, nT):
    return np.stack([S.seeded_column(nT, s) * a for s, a in
                     zip(range(ncols), np.linspace(0.3, 6.0, ncols))]).astype(np.float32)


def _device_call(lib, d_in, d_out, ncols, nT, flux, dz, dt, beta_tvd=1.0, cfl_target=0.0,
                 max_subcycles=1024, stream=None):
    return lib.asg_flux_columns_device(
        C.c_void_p(d_in.data_ptr()), C.c_void_p(d_out.data_ptr()), ncols, nT, flux, N_COEF, dz,
        dt, beta_tvd, cfl_target, max_subcycles, C.c_void_p(stream))


@pytest.mark.parametrize("nT", [3, 65, 256, 801, 2048])
def test_device_entry_matches_host_entry_twice(nT):
    import torch
    from angularspectrum_heterogeneous_gb300 import _lib
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    lib = _lib.load()
    ncols = 37
    cols = _columns(ncols, nT)
    dz, dt = 4e-4, 1e-8
    stream = torch.cuda.current_stream()
    d_in = torch.from_numpy(cols).cuda()
    for name, extra in CASES:
        flux = getattr(_lib, "FLUX_" + name)
        ref = _lib.flux_columns(cols, flux, N_COEF, dz, dt, **extra)
        for call in range(2):  # two calls in a row reuse the same scratch
            d_out = torch.full_like(d_in, float("nan"))
            _lib.check(_device_call(lib, d_in, d_out, ncols, nT, flux, dz, dt,
                                    stream=stream.cuda_stream, **extra))
            stream.synchronize()
            out = d_out.cpu().numpy()
            assert np.isfinite(out).all(), (name, call)
            assert rel(out, ref) < 1e-6, (name, extra, call, rel(out, ref))
    assert torch.equal(d_in.cpu(), torch.from_numpy(cols)), "input buffer was modified"


def test_device_entry_rejects_long_columns():
    import torch
    from angularspectrum_heterogeneous_gb300 import _lib
    lib = _lib.load()
    d = torch.zeros(2 * 4096, device="cuda")
    code = _device_call(lib, d, d, 2, 4096, _lib.FLUX_KT, 1e-4, 1e-8)
    assert code == -2  # ASG_ERR_SHAPE
    assert b"2048" in lib.asg_last_error()


def test_device_entry_rejects_overlapping_buffers():
    import torch
    from angularspectrum_heterogeneous_gb300 import _lib
    lib = _lib.load()
    nT, ncols = 256, 8
    d = torch.zeros(ncols * nT + nT, device="cuda")
    assert _device_call(lib, d, d, ncols, nT, _lib.FLUX_KT, 1e-4, 1e-8) == -1  # same buffer
    assert _device_call(lib, d, d[nT:], ncols, nT, _lib.FLUX_KT, 1e-4, 1e-8) == -1  # shifted
    assert b"overlap" in lib.asg_last_error()


def test_device_entry_reports_capped_subcycles():
    """Columns that need more sub-cycles than the cap are counted in the fixed
    scratch; the count is read after the stream completes, and the next call
    starts again from zero."""
    import torch
    from angularspectrum_heterogeneous_gb300 import _lib
    lib = _lib.load()
    nT, ncols = 256, 16
    cols = _columns(ncols, nT)
    stream = torch.cuda.current_stream()
    d_in = torch.from_numpy(cols).cuda()
    d_out = torch.empty_like(d_in)
    n, need = C.c_uint(0), C.c_uint(0)
    for cap, expect_capped in [(2, True), (4096, False)]:
        _lib.check(_device_call(lib, d_in, d_out, ncols, nT, _lib.FLUX_KT, 4e-4, 1e-8,
                                cfl_target=1e-3, max_subcycles=cap, stream=stream.cuda_stream))
        _lib.check(lib.asg_flux_columns_device_clamped(C.c_void_p(stream.cuda_stream),
                                                       C.byref(n), C.byref(need)))
        if expect_capped:
            assert n.value > 0 and need.value > cap, (n.value, need.value)
        else:
            assert n.value == 0, n.value


def test_device_entry_records_into_a_cuda_graph():
    """Global-mode stream capture rejects cudaMalloc, cudaFree and synchronising
    calls: after one direct call (which loads the kernels), a call recorded into
    a CUDA graph runs nothing while capturing, and the replay gives the direct
    call's result."""
    import torch
    from angularspectrum_heterogeneous_gb300 import _lib
    lib = _lib.load()
    ncols, nT = 37, 256
    cols = _columns(ncols, nT)
    dz, dt = 4e-4, 1e-8
    flux = _lib.FLUX_KT
    ref = _lib.flux_columns(cols, flux, N_COEF, dz, dt, cfl_target=0.3)
    s = torch.cuda.Stream()
    d_in = torch.from_numpy(cols).cuda()
    d_out = torch.full_like(d_in, float("nan"))
    torch.cuda.synchronize()
    _lib.check(_device_call(lib, d_in, d_out, ncols, nT, flux, dz, dt, cfl_target=0.3,
                            stream=s.cuda_stream))
    s.synchronize()
    direct = d_out.clone()
    d_out.fill_(float("nan"))
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        rc = _device_call(lib, d_in, d_out, ncols, nT, flux, dz, dt, cfl_target=0.3,
                          stream=s.cuda_stream)
    _lib.check(rc)
    torch.cuda.synchronize()
    assert torch.isnan(d_out).all(), "the captured call ran during capture"
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(d_out, direct)
    assert rel(d_out.cpu().numpy(), ref) < 1e-6
