"""dpl_process_coherence_noalloc: the solve without a caller workspace.

Its scratch (the LU-fallback counter and pixel list) is a static device array, so
the call allocates nothing.  The GPU tests call it twice in a row through the C ABI
on different inputs and compare each result with dpl_process_coherence on the same
input.  This file is collected last so that the test also runs after every other
GPU test in the same process.
"""

import numpy as np
import pytest

from oracle import phase_link as O


def _lib():
    from dolphin_gb300 import _build, _lib

    _build.build_library()
    return _lib, _lib.load()


def test_noalloc_rejects_sizes_beyond_the_static_scratch():
    L, lib = _lib()
    cap = lib.dpl_process_coherence_noalloc_max_pixels()
    assert cap == 1 << 20
    # the size check comes before any CUDA call, so this runs without a GPU
    st = lib.dpl_process_coherence_noalloc(None, cap + 1, 10, 0, 0.0, 0.0, 0, 1.0, 0, 1,
                                           None, None, None, None, None, None, None)
    assert st == L.DPL_ERR_UNSUPPORTED
    msg = lib.dpl_last_error_message().decode()
    assert "static scratch limit" in msg and str(cap) in msg


def _coherence(n, rows, cols, hw, seed):
    from dolphin_gb300.simulate import StackConfig, make_stack

    z = make_stack(StackConfig(nslc=n, rows=rows, cols=cols, seed=seed, ps_frac=0.0))
    return O.estimate_stack_covariance(z, hw, (1, 1)).reshape(-1, n, n)


def _outputs(torch, npix, n):
    f32, dev = torch.float32, "cuda"
    return dict(
        vec=torch.empty((npix, n), dtype=torch.complex64, device=dev),
        val=torch.empty((npix,), dtype=f32, device=dev),
        est=torch.empty((npix,), dtype=torch.uint8, device=dev),
        crlb=torch.empty((npix, n), dtype=f32, device=dev),
        tc=torch.empty((npix,), dtype=f32, device=dev),
        clos=torch.empty((npix, max(n - 2, 1)), dtype=f32, device=dev),
    )


def _args(D, C, npix, n, o, kw):
    return (D.ptr(C), npix, n, kw["use_evd"], kw["beta"], kw["zct"], kw["ref"], kw["looks"], kw["first_real"],
            kw["crlb"], D.ptr(o["vec"]), D.ptr(o["val"]), D.ptr(o["est"]), D.ptr(o["crlb"]), D.ptr(o["tc"]),
            D.ptr(o["clos"]) if n > 2 else None)


@pytest.mark.gpu
def test_noalloc_matches_workspace_entry_point_twice_in_a_row():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():  # pragma: no cover - CPU container
        pytest.skip("needs a CUDA GPU")
    from dolphin_gb300 import _device as D

    L, lib = _lib()
    # small windows and a beta-regularised |Gamma| put some pixels on the LU fallback
    # list (smallest eigenvalue of |Gamma|^-1 o C below 0.99) and others on EVD
    cases = [
        (_coherence(30, 40, 48, (2, 2), 501), dict(use_evd=0, beta=0.1, zct=0.0, ref=0, looks=2.0, first_real=0,
                                                  crlb=1)),
        (_coherence(12, 31, 29, (1, 2), 502), dict(use_evd=0, beta=0.05, zct=0.02, ref=3, looks=1.4,
                                                  first_real=2, crlb=1)),
    ]
    for C_host, kw in cases:
        npix, n = C_host.shape[0], C_host.shape[-1]
        C = D.to_device(C_host, np.complex64)
        ref = _outputs(torch, npix, n)
        ws = D.workspace(lib.dpl_process_coherence_workspace_size(npix))
        st = lib.dpl_process_coherence(*_args(D, C, npix, n, ref, kw), D.ptr(ws), ws.numel(), D.stream_handle())
        L.check(st, "dpl_process_coherence")
        got = _outputs(torch, npix, n)
        st = lib.dpl_process_coherence_noalloc(*_args(D, C, npix, n, got, kw), D.stream_handle())
        L.check(st, "dpl_process_coherence_noalloc")
        torch.cuda.synchronize()
        fallbacks = int(ws[:4].view(torch.int32).item())
        assert fallbacks > 0, "case should exercise the fallback list"
        r = {k: v.cpu().numpy() for k, v in ref.items()}
        g = {k: v.cpu().numpy() for k, v in got.items()}
        np.testing.assert_array_equal(g["est"], r["est"])
        np.testing.assert_allclose(g["vec"], r["vec"], rtol=0, atol=1e-6)
        np.testing.assert_allclose(g["val"], r["val"], rtol=1e-6, atol=0)
        np.testing.assert_allclose(g["crlb"], r["crlb"], rtol=1e-6, atol=0)
        np.testing.assert_allclose(g["tc"], r["tc"], rtol=0, atol=1e-6)
        if n > 2:
            np.testing.assert_allclose(g["clos"], r["clos"], rtol=0, atol=1e-6)


@pytest.mark.gpu
def test_noalloc_accepts_exactly_the_limit():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():  # pragma: no cover - CPU container
        pytest.skip("needs a CUDA GPU")
    from dolphin_gb300 import _device as D

    L, lib = _lib()
    npix, n = lib.dpl_process_coherence_noalloc_max_pixels(), 3
    rng = np.random.default_rng(503)
    gam = rng.uniform(0.2, 0.95, size=(npix, 1, 1)) ** np.abs(np.subtract.outer(np.arange(n), np.arange(n)))
    ph = rng.normal(scale=1.0, size=(npix, n))
    C_host = (gam * np.exp(1j * (ph[:, :, None] - ph[:, None, :]))).astype(np.complex64)
    kw = dict(use_evd=0, beta=0.0, zct=0.0, ref=0, looks=3.0, first_real=0, crlb=1)
    C = D.to_device(C_host, np.complex64)
    ref, got = _outputs(torch, npix, n), _outputs(torch, npix, n)
    ws = D.workspace(lib.dpl_process_coherence_workspace_size(npix))
    L.check(lib.dpl_process_coherence(*_args(D, C, npix, n, ref, kw), D.ptr(ws), ws.numel(), D.stream_handle()))
    L.check(lib.dpl_process_coherence_noalloc(*_args(D, C, npix, n, got, kw), D.stream_handle()))
    torch.cuda.synchronize()
    for k in ref:
        if k == "est":
            assert torch.equal(got[k], ref[k])
        else:
            a, b = torch.view_as_real(got[k]) if got[k].is_complex() else got[k], \
                torch.view_as_real(ref[k]) if ref[k].is_complex() else ref[k]
            assert torch.allclose(a, b, rtol=1e-6, atol=1e-6, equal_nan=True), k
