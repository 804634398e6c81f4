"""CPU-only checks: the C-ABI library loads and exports what include/dpl.h declares,
argument validation maps to the reference's exceptions, and host-side logic."""

import re
import types
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "dpl.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dpl_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from dolphin_gb300 import _build, _lib

    _build.build_library()
    return _lib.load()


def test_header_declares_the_api():
    names = declared_functions()
    for must in ("dpl_phase_link", "dpl_ps_block", "dpl_shp_glrt", "dpl_shp_ks", "dpl_covariance",
                 "dpl_process_coherence", "dpl_last_error_message"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_python_binding_covers_every_declared_symbol():
    from dolphin_gb300 import _lib

    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_version_and_limits(lib):
    assert lib.dpl_version() >= 1000
    assert lib.dpl_max_nslc() == 64


def test_invalid_arguments_fail_before_any_cuda_call(lib):
    from dolphin_gb300 import _lib

    st = lib.dpl_ps_block(None, 0, 10, 0.25, 0, 0.25, 1, None, None, None, None)
    assert st == _lib.DPL_ERR_INVALID_ARGUMENT
    assert b"bad shape" in lib.dpl_last_error_message()
    with pytest.raises(ValueError):
        _lib.check(st)
    prm = _lib.PlParams(nslc=65, rows=8, cols=8, hy=1, hx=1, sy=1, sx=1)
    st = lib.dpl_phase_link(prm, _lib.PlInputs(), _lib.PlOutputs(), None, 0, None)
    assert st == _lib.DPL_ERR_UNSUPPORTED
    prm = _lib.PlParams(nslc=5, rows=8, cols=8, hy=5, hx=1, sy=1, sx=1)
    st = lib.dpl_phase_link(prm, _lib.PlInputs(), _lib.PlOutputs(), None, 0, None)
    assert st == _lib.DPL_ERR_INVALID_ARGUMENT
    with pytest.raises(ValueError, match="half_window"):
        _lib.check(st)


def test_misaligned_complex_arrays_fail_before_any_cuda_call(lib):
    """Complex arrays are read as 64-bit elements: a pointer that breaks complex64's
    8-byte alignment (or a workspace off its 16-byte alignment) is refused up front."""
    from dolphin_gb300 import _lib

    odd, ok = 0x10004, 0x10000  # never dereferenced: the checks run before any launch
    st = lib.dpl_compress(odd, 3, 4, 4, ok, 4, 4, 0, ok, 0, 0, ok, None)
    assert st == _lib.DPL_ERR_INVALID_ARGUMENT
    assert b"8-byte aligned" in lib.dpl_last_error_message()
    st = lib.dpl_mlp_frame(ok, 4, 10, odd, 0, ok, None)
    assert st == _lib.DPL_ERR_INVALID_ARGUMENT
    prm = _lib.PlParams(nslc=5, rows=8, cols=8, hy=1, hx=1, sy=1, sx=1)
    full = dict(cpx_phase=ok, temp_coh=ok, eigenvalues=ok, estimator=ok, crlb_std_dev=ok)
    ws = lib.dpl_phase_link_workspace_size(prm)
    st = lib.dpl_phase_link(prm, _lib.PlInputs(slc=odd), _lib.PlOutputs(**full), ok, ws, None)
    assert st == _lib.DPL_ERR_INVALID_ARGUMENT
    st = lib.dpl_phase_link(prm, _lib.PlInputs(slc=ok), _lib.PlOutputs(**full), ok + 8, ws, None)
    assert st == _lib.DPL_ERR_INVALID_ARGUMENT
    assert b"16-byte aligned" in lib.dpl_last_error_message()
    st = lib.dpl_covariance(ok, 5, 8, 8, 1, 1, 1, 1, None, 0, odd, ok, 1 << 30, None)
    assert st == _lib.DPL_ERR_INVALID_ARGUMENT
    st = lib.dpl_process_coherence(odd, 4, 5, 0, 0.0, 0.0, 0, 1.0, 0, 1, ok, ok, ok, ok, ok, None, ok, 1 << 30,
                                   None)
    assert st == _lib.DPL_ERR_INVALID_ARGUMENT
    with pytest.raises(ValueError, match="8-byte aligned"):
        _lib.check(st)
    st = lib.dpl_similarity_prep(odd, 1, 4, 8, 8, None, 0, ok, 4, ok, None)
    assert st == _lib.DPL_ERR_INVALID_ARGUMENT
    st = lib.dpl_similarity(odd, 4, 8, 8, 3, 0, ok, None)
    assert st == _lib.DPL_ERR_INVALID_ARGUMENT
    assert b"8-byte aligned" in lib.dpl_last_error_message()
    st = lib.dpl_grow_nodata_region(ok + 2, ok, 0, 8, 8, 0.0, 0, 2, None)  # float32 at a 2-byte offset
    assert st == _lib.DPL_ERR_INVALID_ARGUMENT
    assert b"element size" in lib.dpl_last_error_message()


def test_workspace_sizes_are_positive(lib):
    from dolphin_gb300 import _lib

    prm = _lib.PlParams(nslc=30, rows=1034, cols=1046, hy=5, hx=11, sy=1, sx=1)
    n = lib.dpl_phase_link_workspace_size(prm)
    assert n > 30 * 1034 * 1046 * 8
    assert lib.dpl_shp_glrt_workspace_size(100, 101) >= 100 * 104 * 4
    assert lib.dpl_shp_ks_workspace_size(10, 20, 30) >= 10 * 20 * 30 * 4


def test_all_nan_message_matches_reference_format():
    """The exception text the workflow matches on ("are all NaNs", workflows/single.py:269)."""
    from dolphin_gb300.phase_link import PhaseLinkRuntimeError, _host_all_nan_check

    z = np.ones((4, 3, 3), np.complex64)
    z[1] = np.nan
    z[3] = np.nan
    with pytest.raises(PhaseLinkRuntimeError, match=r"slc_stack\[\[1 3\]\] out of 4 are all NaNs\."):
        _host_all_nan_check(z)


def test_ks_critical_distance_matches_reference(golden):
    from dolphin_gb300.shp import ks_critical_distance

    for n, alpha, d in golden("ks")["crit"]:
        assert ks_critical_distance(int(n), alpha) == d


def test_glrt_threshold():
    from dolphin_gb300.shp import glrt_threshold

    assert abs(glrt_threshold(0.001) - 10.827566170662733) < 1e-9


def test_install_into_dolphin_with_fake_modules():
    import dolphin_gb300 as dp
    from dolphin_gb300 import phase_link as pl

    class FakeError(Exception):
        pass

    mods = {name: types.ModuleType(name) for name, _ in dp._PATCH_TARGETS}
    mods["dolphin.phase_link._core"].PhaseLinkRuntimeError = FakeError
    saved = pl.PhaseLinkRuntimeError
    try:
        patched = dp.install_into_dolphin(modules=mods)
        assert len(patched) == len(dp._PATCH_TARGETS)
        assert mods["dolphin.workflows.single"].run_phase_linking is dp.run_phase_linking
        assert mods["dolphin.shp"].estimate_neighbors is dp.estimate_neighbors
        assert mods["dolphin.ps"].calc_ps_block is dp.calc_ps_block
        assert pl.PhaseLinkRuntimeError is FakeError
    finally:
        pl.PhaseLinkRuntimeError = saved


def test_block_plan_covers_frame_once():
    import bench

    plan = bench.block_plan(2100, 1500, 1024, (5, 11))
    cover = np.zeros((2100, 1500), np.int32)
    for ir, ic, tr, tc, orr, occ in plan:
        assert ir[0] <= orr[0] and ir[1] >= orr[1]
        assert tr[1] - tr[0] == orr[1] - orr[0] and tc[1] - tc[0] == occ[1] - occ[0]
        cover[orr[0]:orr[1], occ[0]:occ[1]] += 1
    assert (cover == 1).all()


def test_types_match_reference_field_order():
    from dolphin_gb300 import HalfWindow, ShpMethod, Strides

    assert HalfWindow(3, 5).y == 3 and Strides(2, 4).x == 4
    assert ShpMethod("glrt") is ShpMethod.GLRT and ShpMethod.NONE.value == "rect"


def test_deferred_checks_bookkeeping(monkeypatch):
    """deferred_checks() waits for and decodes every pending status in call order, raises
    the first failure as the synchronous call would, and keeps nested blocks apart."""
    from dolphin_gb300 import _lib
    from dolphin_gb300 import phase_link as pl

    log = []

    class Event:
        def __init__(self, tag):
            self.tag = tag

        def synchronize(self):
            log.append(("wait", self.tag))

    class Words:  # the "pointer" is the status the fake decoder returns
        def __init__(self, status):
            self.status = status

        def data_ptr(self):
            return self.status

    class FakeLib:
        def dpl_phase_link_status_words(self, nslc, words):
            log.append(("decode", nslc))
            return words

        def dpl_last_error_message(self):
            return b"slc_stack[[1]] out of 5 are all NaNs."

    monkeypatch.setattr(_lib, "load", lambda path=None: FakeLib())
    with pl.deferred_checks():
        pl._deferred.pending.append((5, Words(_lib.DPL_OK), Event("a")))
        with pl.deferred_checks():  # a nested block checks its own calls when it ends
            pl._deferred.pending.append((7, Words(_lib.DPL_OK), Event("inner")))
        assert log == [("wait", "inner"), ("decode", 7)]
        pl._deferred.pending.append((6, Words(_lib.DPL_OK), Event("b")))
    assert log[2:] == [("wait", "a"), ("decode", 5), ("wait", "b"), ("decode", 6)]
    assert getattr(pl._deferred, "pending", None) is None

    log.clear()
    with pytest.raises(pl.PhaseLinkRuntimeError, match="are all NaNs"):
        with pl.deferred_checks():
            pl._deferred.pending.append((5, Words(_lib.DPL_OK), Event("ok")))
            pl._deferred.pending.append((5, Words(_lib.DPL_ERR_ALL_NAN_SLC), Event("bad")))
            pl._deferred.pending.append((5, Words(_lib.DPL_OK), Event("after")))
    assert log == [("wait", "ok"), ("decode", 5), ("wait", "bad"), ("decode", 5)]
    assert getattr(pl._deferred, "pending", None) is None

    # an exception inside the block propagates without waiting on the pending calls
    log.clear()
    with pytest.raises(KeyError):
        with pl.deferred_checks():
            pl._deferred.pending.append((5, Words(_lib.DPL_OK), Event("x")))
            raise KeyError("inside")
    assert log == []
