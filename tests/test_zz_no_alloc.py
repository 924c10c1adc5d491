"""The allocation-free DFT entry point, called through the C ABI.

fit_dft_noalloc serves callers that cannot allocate device memory when they need a
spectrum (all of HBM handed to their own pool, or no device-wide synchronisation
allowed while solver kernels run).  It must give the results of fit_dft, which
allocates its scratch, on two calls in a row: the second call sees the first call's
leftovers in the shared scratch array and must not depend on them.  This file runs
last so that a failure here does not hide the other tests; it passes alone too.
"""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from wakis_gb300 import _native
    return _native.load()


def _signals(seed, nsig, length):
    rng = np.random.default_rng(seed)
    t = np.arange(length)
    base = np.exp(-((t - length / 3) ** 2) / (2 * (length / 10) ** 2))
    return np.stack([base * (1 + 0.1 * s) + 0.01 * rng.standard_normal(length) for s in range(nsig)])


def test_noalloc_dft_matches_allocating_dft_twice(lib):
    from wakis_gb300 import _native
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    cases = [(11, 3, 5000, 221221, 0, 999), (12, 4, 3000, 103103, 5, 640)]
    for seed, nsig, length, n, b0, nb in cases:
        x = _signals(seed, nsig, length)
        ref = _native.dft(x, n, b0, nb)  # allocating entry point (host in / host out)
        xd = torch.as_tensor(x, device=dev).contiguous()
        out = torch.full((nsig, nb, 2), float("nan"), dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev)
        rc = lib.fit_dft_noalloc(ctypes.c_void_p(xd.data_ptr()), nsig, length, n, b0, nb,
                                 ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, _native.last_error(None)
        torch.cuda.synchronize(dev)
        got = out[..., 0].cpu().numpy() + 1j * out[..., 1].cpu().numpy()
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < 1e-12, err
        # and against numpy's FFT of the zero-padded signal
        npf = np.fft.fft(x, n=n, axis=1)[:, b0:b0 + nb]
        assert np.linalg.norm(got - npf) / np.linalg.norm(npf) < 1e-10


def test_noalloc_dft_rejects_sizes_beyond_its_scratch(lib):
    from wakis_gb300 import _native
    dev = torch.device("cuda", 0)
    xd = torch.zeros(8, 16, dtype=torch.float64, device=dev)
    out = torch.zeros(8, 40000, 2, dtype=torch.float64, device=dev)
    rc = lib.fit_dft_noalloc(ctypes.c_void_p(xd.data_ptr()), 8, 16, 100000, 0, 40000,
                             ctypes.c_void_p(out.data_ptr()), None)
    assert rc == -1
    assert "exceeds the fixed scratch" in _native.last_error(None)


def test_noalloc_dft_at_the_scratch_limit_matches(lib):
    """nsig*nb = 2^18 partial sums fill the fixed scratch exactly: a long signal (which
    would otherwise be split 32 ways along time) is then summed in one slice.  Two calls in
    a row agree with the allocating entry point and with numpy."""
    from wakis_gb300 import _native
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    nsig, length, n, b0, nb = 4, 65536, 1 << 18, 0, 1 << 16
    for seed in (21, 22):
        x = _signals(seed, nsig, length)
        ref = _native.dft(x, n, b0, nb)
        xd = torch.as_tensor(x, device=dev).contiguous()
        out = torch.full((nsig, nb, 2), float("nan"), dtype=torch.float64, device=dev)
        rc = lib.fit_dft_noalloc(ctypes.c_void_p(xd.data_ptr()), nsig, length, n, b0, nb,
                                 ctypes.c_void_p(out.data_ptr()), None)
        assert rc == 0, _native.last_error(None)
        torch.cuda.synchronize(dev)
        got = out[..., 0].cpu().numpy() + 1j * out[..., 1].cpu().numpy()
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-12
        npf = np.fft.fft(x, n=n, axis=1)[:, b0:b0 + nb]
        assert np.linalg.norm(got - npf) / np.linalg.norm(npf) < 1e-10


def test_noalloc_dft_refuses_host_pointers_and_too_many_signals(lib):
    """Arguments the kernels cannot use are refused on the host before any launch: host
    memory for x or out, and more signals than a launch grid holds."""
    from wakis_gb300 import _native
    dev = torch.device("cuda", 0)
    xh = np.zeros((2, 64))
    xd = torch.zeros(2, 64, dtype=torch.float64, device=dev)
    outd = torch.zeros(2, 8, 2, dtype=torch.float64, device=dev)
    outh = np.zeros((2, 8, 2))
    rc = lib.fit_dft_noalloc(ctypes.c_void_p(xh.ctypes.data), 2, 64, 128, 0, 8, ctypes.c_void_p(outd.data_ptr()),
                             None)
    assert rc == -1 and "device memory" in _native.last_error(None)
    rc = lib.fit_dft_noalloc(ctypes.c_void_p(xd.data_ptr()), 2, 64, 128, 0, 8, ctypes.c_void_p(outh.ctypes.data),
                             None)
    assert rc == -1 and "device memory" in _native.last_error(None)
    big = torch.zeros(65536, 1, dtype=torch.float64, device=dev)
    bout = torch.zeros(65536, 1, 2, dtype=torch.float64, device=dev)
    rc = lib.fit_dft_noalloc(ctypes.c_void_p(big.data_ptr()), 65536, 1, 4, 0, 1, ctypes.c_void_p(bout.data_ptr()),
                             None)
    assert rc == -1 and "signals per call" in _native.last_error(None)
    torch.cuda.synchronize(dev)
