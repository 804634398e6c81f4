"""Ministack batches: several phase-linking problems as one CUDA-graph replay.

A sequential dolphin run processes ministacks of different depth N (e.g. 15 new SLCs
plus the compressed SLCs of earlier ministacks).  ``PhaseLinkBatch`` takes a list of
device-resident stacks, runs PS selection, GLRT SHP selection and phase linking for
each, and after a first eager run captures the whole sequence once as a CUDA graph:
later ``run()`` calls replay it with one launch, reading the (updated in place)
input tensors and writing the same output tensors.  The per-call status (all-NaN
SLCs, device timeouts) is checked after the replay, as ``run_phase_linking`` does.

Per N, ``tune_forms`` chooses the covariance form (tensor cores or SIMT) and the
register solver's instance (row slots K and threads per pixel: several pixels per warp
for small N) by timing the candidates on a small synthetic stack of that depth once per
(N, half window, strides), and keeps the choice in a table that can be saved and loaded
as JSON.
"""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np

from . import _device as D
from . import _lib
from .phase_link import PhaseLinkOutput, _form_code
from .ps import calc_ps_block
from .shp import estimate_neighbors

__all__ = ["PhaseLinkBatch", "tune_forms"]

_TUNED: dict[tuple, dict] = {}


def _solver_candidates(n):
    """(slots, lanes) pairs the register solver offers for depth n: K = n rounded up to
    even and the next power of two (one or two warps as n needs), and every group size
    from the smallest that fits K up to a whole warp."""
    k0 = max(4, (n + 1) & ~1)
    ks = {k0}
    p2 = 4
    while p2 < k0:
        p2 *= 2
    if p2 <= 64 and (p2 > 32) == (k0 > 32):
        ks.add(p2)
    out = []
    for k in sorted(ks):
        if k > 32:
            out.append((k, 64))
            continue
        g = 8
        while g < k:
            g *= 2
        while g <= 32:
            out.append((k, g))
            g *= 2
    return out


def _time_call(fn, reps):
    import torch

    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def tune_forms(depths, half_window, strides=(1, 1), table_path=None, sample=192, reps=3):
    """Pick, for each stack depth N, the covariance form (tensor cores or SIMT) and the
    register solver's instance (row slots K and threads per pixel) by timing the
    candidates; returns {N: {"form": ..., "slots": K, "lanes": G}}.

    Timings use a seeded synthetic stack of ``sample x sample`` output pixels per depth,
    with its GLRT SHPs.  ``table_path`` (JSON) is read first and written back with any
    new entries.
    """
    from .phase_link import run_phase_linking
    from .ps import calc_ps_block as _ps
    from .shp import estimate_neighbors as _shp
    from .simulate import StackConfig, make_stack_torch

    hy, hx = (int(v) for v in half_window)
    sy, sx = (int(v) for v in strides)
    if table_path is not None and Path(table_path).exists():
        for k, v in json.loads(Path(table_path).read_text()).items():
            _TUNED[tuple(int(x) for x in k.split(","))] = v
    out = {}
    for n in sorted(set(int(d) for d in depths)):
        key = (n, hy, hx, sy, sx)
        if key not in _TUNED or not isinstance(_TUNED[key], dict):
            cfg = StackConfig(nslc=n, rows=sample * sy + 2 * hy, cols=sample * sx + 2 * hx, seed=1000 + n,
                              ps_frac=0.03)
            z = make_stack_torch(cfg)
            mean, disp, ps = _ps(z.abs(), 0.25, n)
            nb = _shp(halfwin_rowcol=(hy, hx), alpha=0.001, strides=(sy, sx), mean=mean, var=(disp * mean) ** 2,
                      nslc=n)
            kw = dict(ps_mask=ps, neighbor_arrays=nb, avg_mag=mean)
            forms = {f: _time_call(lambda f=f: run_phase_linking(z, (hy, hx), (sy, sx), covariance_form=f, **kw), reps)
                     for f in ("tensor", "simt")}
            form = min(forms, key=forms.get)
            solver = {}
            for k, g in _solver_candidates(n):
                solver[(k, g)] = _time_call(lambda k=k, g=g: run_phase_linking(
                    z, (hy, hx), (sy, sx), covariance_form=form, solver_slots=k, solver_lanes=g, **kw), reps)
            k, g = min(solver, key=solver.get)
            _TUNED[key] = {"form": form, "slots": k, "lanes": g,
                           "ms": {"forms": {f: round(v, 4) for f, v in forms.items()},
                                  "solver": {f"{kk},{gg}": round(v, 4) for (kk, gg), v in solver.items()}}}
        out[n] = {k: v for k, v in _TUNED[key].items() if k != "ms"}
    if table_path is not None:
        Path(table_path).write_text(json.dumps({",".join(map(str, k)): v for k, v in sorted(_TUNED.items())},
                                               indent=1))
    return out


def _choice(forms, n):
    """A tuned entry as (form, slots, lanes); a bare form string means default slots."""
    c = forms.get(n, "tensor")
    if isinstance(c, str):
        return c, 0, 0
    return c.get("form", "tensor"), int(c.get("slots", 0)), int(c.get("lanes", 0))


class PhaseLinkBatch:
    """PS + GLRT + phase linking over a list of (N_k, rows, cols) complex64 CUDA stacks.

    With ``persistent`` (the default) the whole batch is one ``dpl_phase_link_batch``
    call: the tensor-core covariance of every stack is one persistent launch over a
    work queue of (stack, tile) items, largest N first; ``persistent=False`` enqueues one
    ``dpl_phase_link`` per stack.  Parameters follow ``run_phase_linking`` (EMI/EVD,
    CRLB, references) and
    ``estimate_neighbors`` (GLRT ``alpha``); ``forms`` maps N to a ``tune_forms`` entry
    or to a bare covariance form, "tensor" or "simt" (default: ``tune_forms``).  ``graph=False`` runs every call eagerly.
    """

    def __init__(self, stacks, half_window, strides=(1, 1), alpha=0.001, ps_threshold=0.25, use_evd=False,
                 compute_crlb=True, reference_idx=0, forms=None, graph=True, persistent=True):
        self.stacks = list(stacks)
        for z in self.stacks:
            if not (D.is_device_tensor(z) and z.is_complex() and z.dim() == 3 and z.is_contiguous()):
                raise ValueError("PhaseLinkBatch needs contiguous 3-D complex CUDA tensors")
        self.hw = tuple(int(v) for v in half_window)
        self.st = tuple(int(v) for v in strides)
        self.alpha, self.thr = float(alpha), float(ps_threshold)
        self.use_evd, self.crlb, self.ref = bool(use_evd), bool(compute_crlb), int(reference_idx)
        depths = [int(z.shape[0]) for z in self.stacks]
        self.forms = dict(forms) if forms is not None else tune_forms(depths, self.hw, self.st)
        self.graph_enabled = bool(graph)
        self.persistent = bool(persistent)
        if self.persistent and len(self.stacks) > 16:
            raise ValueError("a persistent batch takes at most 16 stacks")
        self._graph = None
        self._outs = None
        self._calls = None  # per stack: (params, workspace tensor)

    def _enqueue(self):
        """Enqueue every stack's pipeline on the current stream; returns the outputs."""
        torch = D.require_cuda()
        lib = _lib.load()
        outs, calls = [], []
        hy, hx = self.hw
        sy, sx = self.st
        for z in self.stacks:
            n, rows, cols = (int(v) for v in z.shape)
            mean, disp, ps = calc_ps_block(z.abs(), self.thr, n)
            nb = estimate_neighbors(halfwin_rowcol=self.hw, alpha=self.alpha, strides=self.st, mean=mean,
                                    var=(disp * mean) ** 2, nslc=n)
            orow, ocol = rows // sy, cols // sx
            form, slots, lanes = _choice(self.forms, n)
            prm = _lib.PlParams(nslc=n, rows=rows, cols=cols, hy=hy, hx=hx, sy=sy, sx=sx,
                                use_evd=int(self.use_evd), beta=0.0, zero_correlation_threshold=0.0,
                                reference_idx=self.ref, mask_input_ps=0, use_max_ps=1, use_slc_amp=0,
                                baseline_lag=0, first_real_slc_idx=0, compute_crlb=int(self.crlb),
                                cov_form=_form_code(form), solver_slots=slots, solver_lanes=lanes)
            o = {
                "cpx": torch.empty((n, orow, ocol), dtype=torch.complex64, device=z.device),
                "tc": torch.empty((orow, ocol), dtype=torch.float32, device=z.device),
                "cnt": torch.empty((orow, ocol), dtype=torch.int32, device=z.device),
                "eig": torch.empty((orow, ocol), dtype=torch.float32, device=z.device),
                "est": torch.empty((orow, ocol), dtype=torch.uint8, device=z.device),
                "crlb": torch.empty((n, orow, ocol), dtype=torch.float32, device=z.device),
                "clos": torch.empty((orow, ocol, max(n - 2, 1)), dtype=torch.float32, device=z.device),
            }
            inp = _lib.PlInputs(slc=D.ptr(z), nodata_mask=None, ps_mask=D.ptr(ps), neighbors=D.ptr(nb),
                                avg_mag=D.ptr(mean))
            outp = _lib.PlOutputs(cpx_phase=D.ptr(o["cpx"]), temp_coh=D.ptr(o["tc"]), shp_counts=D.ptr(o["cnt"]),
                                  eigenvalues=D.ptr(o["eig"]), estimator=D.ptr(o["est"]),
                                  crlb_std_dev=D.ptr(o["crlb"]),
                                  closure_phases=D.ptr(o["clos"]) if n > 2 else None)
            o["_keep"] = (mean, disp, ps, nb)  # inputs of the captured kernels stay allocated
            outs.append(o)
            calls.append((prm, inp, outp))
        if self.persistent:
            # one dpl_phase_link_batch: the covariance of every stack in one work-queue launch
            k = len(calls)
            prms = (_lib.PlParams * k)(*[c[0] for c in calls])
            inps = (_lib.PlInputs * k)(*[c[1] for c in calls])
            outps = (_lib.PlOutputs * k)(*[c[2] for c in calls])
            nbytes = int(lib.dpl_phase_link_batch_workspace_size(prms, k))
            ws = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=self.stacks[0].device)
            _lib.check(lib.dpl_phase_link_batch(prms, inps, outps, k, D.ptr(ws), ws.numel(), D.stream_handle()),
                       "dpl_phase_link_batch")
            return outs, [("batch", prms, k, ws)]
        out_calls = []
        for prm, inp, outp in calls:
            ws = torch.empty(max(int(lib.dpl_phase_link_workspace_size(prm)), 256), dtype=torch.uint8,
                             device=self.stacks[0].device)
            _lib.check(lib.dpl_phase_link_async(prm, inp, outp, D.ptr(ws), ws.numel(), D.stream_handle()),
                       "dpl_phase_link_async")
            out_calls.append(("one", prm, 1, ws))
        return outs, out_calls

    def _check(self, calls):
        lib = _lib.load()
        for kind, prm, k, ws in calls:
            if kind == "batch":
                _lib.check(lib.dpl_phase_link_batch_status(prm, k, D.ptr(ws), ws.numel(), D.stream_handle()),
                           "dpl_phase_link_batch")
            else:
                _lib.check(lib.dpl_phase_link_status(prm, D.ptr(ws), ws.numel(), D.stream_handle()),
                           "dpl_phase_link")

    def run(self):
        """Process every stack; returns a list of ``PhaseLinkOutput`` (CUDA tensors)."""
        torch = D.require_cuda()
        if not self.graph_enabled:
            outs, calls = self._enqueue()
            self._check(calls)
            return [self._output(o) for o in outs]
        if self._graph is None:
            # eager warm-up (kernel attributes, libraries), then capture on a side stream
            outs, calls = self._enqueue()
            self._check(calls)
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(s), torch.cuda.graph(g, stream=s):
                self._outs, self._calls = self._enqueue()
            torch.cuda.current_stream().wait_stream(s)
            self._graph = g
        self._graph.replay()
        self._check(self._calls)
        return [self._output(o) for o in self._outs]

    @staticmethod
    def _output(o):
        return PhaseLinkOutput(o["cpx"], o["tc"], o["cnt"], o["eig"], o["est"], o["crlb"], o["clos"])
