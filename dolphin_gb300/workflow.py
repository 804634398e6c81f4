"""Wrapped-phase workflow on device arrays: the block loop of one ministack and the
sequential chain of ministacks with compressed SLCs.

* :class:`StridedBlockManager`, :func:`iter_blocks` -- io/_blocks.py:59-348: the
  output grid is walked without overlap, from a margin of round(half_window /
  strides) output pixels on every side; each output block is dilated by the strides
  and padded by the half window to give the input block, and the padding is trimmed
  from the results.
* :func:`grow_nodata_region` -- utils.py:613-660 on the GPU (``dpl_grow_nodata_region``).
* :func:`plan_ministacks` -- MiniStackPlanner.plan, stack.py:446-562, at the level of
  layer indices: which earlier compressed SLCs and which input layers each ministack
  holds, and its output and compression reference indices.
* :func:`run_wrapped_phase_single` -- workflows/single.py:43-405 without raster I/O:
  per block, SHP selection, ``run_phase_linking``, NaN -> 0, the compressed SLC of the
  real SLCs with their mean and amplitude dispersion (``calc_ps_block``), the trimmed
  results placed into full output rasters (the strided ones eroded by
  ``grow_nodata_region``, 2 pixels), then the median phase-similarity raster of the
  phase-linked SLCs (``create_similarities`` with search radius 7).
* :func:`run_wrapped_phase_sequential` -- workflows/sequential.py:31-227 without files:
  each ministack is the last ``max_num_compressed`` compressed SLCs followed by its real
  SLCs; its compressed SLC joins the list; the temporal-coherence and SHP-count rasters
  are averaged as ``gdal_calc`` does with NoDataValue 0 (0 where any ministack has 0,
  else the mean); with more than one ministack, a median similarity raster with search
  radius 11 is made from the last ministack's phase-linked SLCs, as the reference does.

Everything stays on the GPU: the stack, every block and every output raster are CUDA
tensors, and each step runs in the library's kernels.  What the reference does on
files only -- reading and writing rasters, repacking them to 12 mantissa bits,
skipping finished ministacks, moving files -- has no counterpart here; in particular
the similarity rasters are computed from the full-precision phases.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from enum import Enum
from typing import Iterator, NamedTuple, Optional, Sequence

import numpy as np

from . import _device as D
from . import _lib
from ._types import HalfWindow, ShpMethod, Strides
from .compress import compress
from .phase_link import _captured_checks, check_captured, deferred_checks, run_phase_linking
from .ps import calc_ps_block
from .shp import estimate_neighbors
from .similarity import stack_similarity

__all__ = [
    "BlockIndices",
    "CompressedSlcPlan",
    "MiniStackPlan",
    "SequentialOutput",
    "SingleOutput",
    "StridedBlockManager",
    "grow_nodata_region",
    "iter_blocks",
    "plan_ministacks",
    "run_wrapped_phase_sequential",
    "clear_loop_graphs",
    "run_wrapped_phase_single",
]


# ------------------------------------------------------------------------------------
# blocks
# ------------------------------------------------------------------------------------
@dataclass(frozen=True)
class BlockIndices:
    """Row and column slices of a 2-D block (io/_blocks.py:28-56)."""

    row_start: int
    row_stop: Optional[int]
    col_start: int
    col_stop: Optional[int]

    @property
    def row_slice(self) -> slice:
        return slice(self.row_start, self.row_stop)

    @property
    def col_slice(self) -> slice:
        return slice(self.col_start, self.col_stop)

    def __iter__(self):
        return iter((self.row_slice, self.col_slice))


def iter_blocks(arr_shape, block_shape, overlaps=(0, 0), start_offsets=(0, 0), end_margin=(0, 0)
                ) -> Iterator[BlockIndices]:
    """Blocks of ``block_shape`` over ``arr_shape``, row by row, from ``start_offsets`` up
    to ``end_margin`` before the end, each one ``overlaps`` back from the previous one
    (except at the last row or column); the last block of a row or column is cut short."""
    rows, cols = arr_shape
    height, width = block_shape
    height = rows if height is None else height
    width = cols if width is None else width
    r_over, c_over = overlaps
    if r_over >= height and height != rows:
        raise ValueError(f"row_overlap = {r_over} must be less than block height {height}")
    if c_over >= width and width != cols:
        raise ValueError(f"col_overlap = {c_over} must be less than block width {width}")
    last_r, last_c = rows - end_margin[0], cols - end_margin[1]
    r = start_offsets[0]
    while r < last_r:
        c = start_offsets[1]
        while c < last_c:
            yield BlockIndices(r, min(r + height, last_r), c, min(c + width, last_c))
            c += width
            if c < last_c:
                c -= c_over
        r += height
        if r < last_r:
            r -= r_over


def dilate_block(block: BlockIndices, strides) -> BlockIndices:
    sy, sx = strides
    return BlockIndices(block.row_start * sy, None if block.row_stop is None else block.row_stop * sy,
                        block.col_start * sx, None if block.col_stop is None else block.col_stop * sx)


def pad_block(block: BlockIndices, margins) -> BlockIndices:
    rm, cm = margins
    if block.row_start - rm < 0:
        raise ValueError(f"r_slice = {block.row_slice}, but r_margin = {rm}")
    if block.col_start - cm < 0:
        raise ValueError(f"c_slice = {block.col_slice}, but c_margin = {cm}")
    return BlockIndices(block.row_start - rm, block.row_stop + rm, block.col_start - cm, block.col_stop + cm)


def get_full_res_trim(no_pad: BlockIndices, padded: BlockIndices) -> BlockIndices:
    return BlockIndices(no_pad.row_start - padded.row_start, (no_pad.row_stop - padded.row_stop) or None,
                        no_pad.col_start - padded.col_start, (no_pad.col_stop - padded.col_stop) or None)


@dataclass
class StridedBlockManager:
    """Input/output block indices for a strided, half-window-padded block loop."""

    arr_shape: tuple
    block_shape: tuple
    strides: Strides = field(default_factory=lambda: Strides(1, 1))
    half_window: HalfWindow = field(default_factory=lambda: HalfWindow(0, 0))

    def _nodata(self, axis: int) -> int:
        return round(self.half_window[axis] / self.strides[axis])

    @property
    def output_shape(self):
        return (self.arr_shape[0] // self.strides[0], self.arr_shape[1] // self.strides[1])

    @property
    def out_block_shape(self):
        return (self.block_shape[0] // self.strides[0], self.block_shape[1] // self.strides[1])

    @property
    def output_margin(self):
        return (self._nodata(0), self._nodata(1))

    @property
    def input_padding_shape(self):
        return (self.strides[0] * self._nodata(0), self.strides[1] * self._nodata(1))

    def get_trimming_block(self) -> BlockIndices:
        ry, rx = self.output_margin
        return BlockIndices(ry, -ry if ry > 0 else None, rx, -rx if rx > 0 else None)

    def iter_outputs(self) -> Iterator[BlockIndices]:
        yield from iter_blocks(self.output_shape, self.out_block_shape, (0, 0), self.output_margin,
                               self.output_margin)

    def iter_blocks(self):
        """(output block, output trim, input block, input without padding, input trim)."""
        trim = self.get_trimming_block()
        for out in self.iter_outputs():
            no_pad = dilate_block(out, self.strides)
            padded = pad_block(no_pad, self.input_padding_shape)
            yield out, trim, padded, no_pad, get_full_res_trim(no_pad, padded)


# ------------------------------------------------------------------------------------
# rasters
# ------------------------------------------------------------------------------------
_DTYPE_CODES = {"float32": 0, "uint8": 1, "int8": 2, "int16": 3, "uint16": 4, "int32": 5}


def grow_nodata_region(arr, nodata: float, n_pixels: int = 1, copy: bool = True):
    """Set to ``nodata`` every pixel within ``n_pixels`` (square) of a nodata pixel.

    A 2-D CUDA tensor gives a CUDA tensor (with ``copy=False`` the result is written
    back into ``arr``); a host array gives a host array.
    """
    torch = D.require_cuda()
    on_device = D.is_device_tensor(arr)
    if on_device:
        src = arr.contiguous()
        name = str(src.dtype).replace("torch.", "")
    else:
        a = np.asarray(arr)
        name = a.dtype.name
        src = D.to_device(a)
    if src.dim() != 2:
        raise ValueError("Input array must be 2D.")
    if name not in _DTYPE_CODES:
        raise ValueError(f"grow_nodata_region: unsupported dtype {name}")
    out = torch.empty_like(src)
    nan = nodata is not None and isinstance(nodata, float) and math.isnan(nodata)
    lib = _lib.load()
    _lib.check(lib.dpl_grow_nodata_region(D.ptr(src), D.ptr(out), _DTYPE_CODES[name], src.shape[0], src.shape[1],
                                          0.0 if nan else float(nodata), int(nan), int(n_pixels), D.stream_handle()),
               "dpl_grow_nodata_region")
    if on_device:
        if not copy:
            arr.copy_(out)
            return arr
        return out
    res = D.to_host(out)
    if not copy:
        np.copyto(arr, res)
        return arr
    return res


# ------------------------------------------------------------------------------------
# ministack planning
# ------------------------------------------------------------------------------------
class CompressedSlcPlan(str, Enum):
    ALWAYS_FIRST = "always_first"
    FIRST_PER_MINISTACK = "first_per_ministack"
    LAST_PER_MINISTACK = "last_per_ministack"


@dataclass
class MiniStackPlan:
    """One ministack: ``compressed`` indexes the running list of compressed SLCs (the
    input's own compressed layers first, then one per earlier ministack); ``layers``
    indexes the input stack."""

    compressed: list
    layers: list
    is_compressed: list
    output_reference_idx: int
    compressed_reference_idx: int

    @property
    def first_real_slc_idx(self) -> int:
        for i, c in enumerate(self.is_compressed):
            if not c:
                return i
        raise ValueError("No real SLCs in ministack")

    @property
    def size(self) -> int:
        return len(self.is_compressed)


def plan_ministacks(is_compressed: Sequence[bool], ministack_size: int, max_num_compressed: int = 5,
                    compressed_slc_plan: CompressedSlcPlan | str = CompressedSlcPlan.ALWAYS_FIRST,
                    output_reference_idx: Optional[int] = None, compressed_idx: Optional[int] = None
                    ) -> list[MiniStackPlan]:
    """The ministacks MiniStackPlanner.plan makes for a stack whose layers are
    compressed (True) or real (False), compressed ones first."""
    plan = CompressedSlcPlan(compressed_slc_plan)
    flags = [bool(c) for c in is_compressed]
    n = len(flags)
    if ministack_size < 2:
        raise ValueError("Cannot create ministacks with size < 2")
    if ministack_size < n:
        if compressed_idx is not None:
            raise ValueError("Cannot set `compressed_idx` when creating multiple ministacks.")
        if plan == CompressedSlcPlan.LAST_PER_MINISTACK:
            raise ValueError("'last_per_ministack' cannot be used for multiple ministacks")
    first_real = next((i for i, c in enumerate(flags) if not c), None)
    if first_real is None:
        raise ValueError("No real SLCs in ministack")
    comp_ids = [i for i, c in enumerate(flags) if c]  # the input's compressed layers
    n_comp = len(comp_ids)
    out: list[MiniStackPlan] = []
    for start in range(first_real, n, ministack_size):
        layers = list(range(start, min(start + ministack_size, n)))
        keep = list(range(n_comp))[-max_num_compressed:]  # as sliced in the reference (0 keeps all)
        num_cc = len(keep)
        if compressed_idx is not None:
            comp_ref = compressed_idx
        elif plan == CompressedSlcPlan.ALWAYS_FIRST:
            comp_ref = max(0, num_cc - 1)
        elif plan == CompressedSlcPlan.LAST_PER_MINISTACK:
            comp_ref = -1
        else:
            # the reference assigns no compressed reference for this plan
            raise UnboundLocalError("cannot access local variable 'compressed_reference_idx' where it is not "
                                    "associated with a value")
        out_ref = output_reference_idx if output_reference_idx is not None else max(0, num_cc - 1)
        out.append(MiniStackPlan(compressed=keep, layers=layers,
                                 is_compressed=[True] * num_cc + [flags[i] for i in layers],
                                 output_reference_idx=out_ref, compressed_reference_idx=comp_ref))
        n_comp += 1
    return out


# ------------------------------------------------------------------------------------
# one ministack
# ------------------------------------------------------------------------------------
class SingleOutput(NamedTuple):
    pl_slcs: object          # (n - first_real, R', C') complex64: phase-linked real SLCs
    crlb: object             # (n - first_real, R', C') float32, or None
    closure_phases: object   # (R', C', n - 2) float32, or None
    comp_slc: object         # (R, C) complex64
    amp_dispersion: object   # (R, C) float32 (the compressed SLC's second band)
    temp_coh: object         # (R', C') float32
    shp_counts: object       # (R', C') uint16
    eigenvalues: object      # (R', C') float32
    estimator: object        # (R', C') uint8
    similarity: object       # (R', C') float32, or None


def run_wrapped_phase_single(slc_stack, *, half_window, strides=None, first_real_slc_idx: int = 0,
                             output_reference_idx: int = 0, compressed_reference_idx: int = 0, beta: float = 0.0,
                             zero_correlation_threshold: float = 0.0, use_evd: bool = False, nodata_mask=None,
                             ps_mask=None, amp_mean=None, amp_dispersion=None,
                             shp_method: ShpMethod | str = ShpMethod.NONE, shp_alpha: float = 0.05,
                             shp_nslc: Optional[int] = None, similarity_nearest_n: Optional[int] = None,
                             write_closure_phase: bool = True, write_crlb: bool = True,
                             block_shape=(512, 512), baseline_lag: Optional[int] = None,
                             similarity: bool = True, graph: bool = False) -> SingleOutput:
    """One ministack's block loop on a (n, R, C) complex stack (CUDA tensor or host
    array; the results are CUDA tensors).  ``half_window`` and ``strides`` are
    ``{"y": .., "x": ..}`` dicts or (y, x) pairs; ``amp_mean`` / ``amp_dispersion`` are
    the (R, C) rasters the reference reads from files (variance = (dispersion *
    mean) ** 2).

    ``graph`` (not in the reference): the whole block loop, similarity included, runs as
    one CUDA graph.  The first call with a given set of shapes, parameters and skipped
    blocks runs eagerly on the graph's own input buffers and captures the loop; later
    such calls copy their inputs into those buffers and replay it (one launch from the
    host), then check every block's phase-linking status in order.  The results are
    copies, the same as the eager loop's.  KS SHPs run eagerly."""
    torch = D.require_cuda()
    hw = _yx(half_window, HalfWindow)
    st = _yx(strides if strides is not None else (1, 1), Strides)
    stack = D.to_device(slc_stack, np.complex64)
    n, rows, cols = (int(v) for v in stack.shape)
    dev = stack.device
    if shp_nslc is None:
        shp_nslc = n
    nodata = torch.zeros((rows, cols), dtype=torch.bool, device=dev) if nodata_mask is None else \
        D.to_device(nodata_mask, np.uint8).bool()
    psm = torch.zeros((rows, cols), dtype=torch.bool, device=dev) if ps_mask is None else \
        D.to_device(ps_mask, np.uint8).bool()
    mean = None if amp_mean is None else D.to_device(amp_mean, np.float32)
    var = None
    if mean is not None and amp_dispersion is not None:
        var = (D.to_device(amp_dispersion, np.float32) * mean) ** 2
    method = ShpMethod(shp_method) if not isinstance(shp_method, ShpMethod) else shp_method

    mgr = StridedBlockManager((rows, cols), tuple(block_shape), st, hw)
    orow, ocol = mgr.output_shape
    nreal = n - first_real_slc_idx
    pl = torch.zeros((nreal, orow, ocol), dtype=torch.complex64, device=dev)
    crlb = torch.zeros((nreal, orow, ocol), dtype=torch.float32, device=dev) if write_crlb else None
    clos = torch.zeros((orow, ocol, max(n - 2, 0)), dtype=torch.float32, device=dev) if write_closure_phase else None
    comp = torch.zeros((rows, cols), dtype=torch.complex64, device=dev)
    disp = torch.zeros((rows, cols), dtype=torch.float32, device=dev)
    tcoh = torch.zeros((orow, ocol), dtype=torch.float32, device=dev)
    counts = torch.zeros((orow, ocol), dtype=torch.int32, device=dev)
    eig = torch.zeros((orow, ocol), dtype=torch.float32, device=dev)
    est = torch.zeros((orow, ocol), dtype=torch.uint8, device=dev)

    # The reference skips a block that is all nodata, all zero or all NaN, or that has an
    # all-NaN SLC (run_phase_linking raises PhaseLinkRuntimeError, which the loop catches).
    # Those decisions are taken for every block at once, with one read back to the host;
    # the block loop then runs without a host synchronisation per block, its phase-linking
    # status checks deferred to the end (any other error still raises).
    blocks = list(mgr.iter_blocks())
    checks = []
    for _o, _t, (ir, ic), _n, _f in blocks:
        cur = stack[:, ir, ic]
        nan = torch.isnan(cur)
        checks.append(torch.stack([nodata[ir, ic].all(), (cur == 0).all() | nan.all(),
                                   nan.flatten(1).all(dim=1).any()]))
    skip = torch.stack(checks).any(dim=1).tolist() if checks else []

    def loop(inp, rasters):
        # the blocks, the similarity and the uint16 shp_counts raster
        z, nd, ps_, mn, vr = inp
        for (out_b, trim, in_b, no_pad, in_trim), skipped in zip(blocks, skip):
            if not skipped:
                _single_block(z, out_b, trim, in_b, no_pad, in_trim, nd, ps_, mn, vr, hw, st, method, shp_alpha,
                              shp_nslc, use_evd, beta, zero_correlation_threshold, output_reference_idx,
                              baseline_lag, first_real_slc_idx, write_crlb, compressed_reference_idx, rasters)
        pl_, crlb_, clos_, comp_, disp_, tcoh_, counts_, eig_, est_ = rasters
        sim = None
        if similarity:
            sim = stack_similarity(pl_, search_radius=7, sim_type="median", nearest_n=similarity_nearest_n)
        return SingleOutput(pl_, crlb_, clos_, comp_, disp_, tcoh_, counts_.clamp(0, 65535).to(torch.uint16), eig_,
                            est_, sim)

    rasters = (pl, crlb, clos, comp, disp, tcoh, counts, eig, est)
    inputs = (stack, nodata, psm, mean, var)
    # the KS test copies a host table per call, which a graph cannot replay: eager
    if not graph or method == ShpMethod.KS:
        with deferred_checks():
            return loop(inputs, rasters)
    key = (str(dev), n, rows, cols, hw, st, first_real_slc_idx, output_reference_idx, compressed_reference_idx,
           float(beta), float(zero_correlation_threshold), bool(use_evd), method, float(shp_alpha), shp_nslc,
           similarity_nearest_n, bool(write_closure_phase), bool(write_crlb), tuple(block_shape), baseline_lag,
           bool(similarity), mean is None, var is None, tuple(skip))
    entry = _LOOP_GRAPHS.get(key)
    if entry is None:
        # eager run on the graph's own input buffers (it also sets up every kernel),
        # then the capture of the same loop on a side stream
        static_in = tuple(None if x is None else x.clone() for x in inputs)
        with deferred_checks():
            out = loop(static_in, rasters)
        calls = []
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(side), torch.cuda.graph(g, stream=side), _captured_checks(calls):
            captured = loop(static_in, rasters)
        torch.cuda.current_stream().wait_stream(side)
        while len(_LOOP_GRAPHS) >= _LOOP_GRAPHS_MAX:
            _LOOP_GRAPHS.pop(next(iter(_LOOP_GRAPHS)))
        _LOOP_GRAPHS[key] = (static_in, g, calls, captured)
    else:
        static_in, g, calls, out = entry
        for dst, src in zip(static_in, inputs):
            if dst is not None:
                dst.copy_(src)
        g.replay()
        check_captured(calls)
    return SingleOutput(*(None if x is None else x.clone() for x in out))


# Captured block loops (run_wrapped_phase_single(graph=True)), oldest first: the input
# buffers, the graph, its phase-linking calls (params, workspace) and its outputs.
_LOOP_GRAPHS: dict = {}
_LOOP_GRAPHS_MAX = 4


def clear_loop_graphs():
    """Drop the captured block loops and the device memory they hold."""
    _LOOP_GRAPHS.clear()


def _single_block(stack, out_b, trim, in_b, no_pad, in_trim, nodata, psm, mean, var, hw, st, method, shp_alpha,
                  shp_nslc, use_evd, beta, zero_correlation_threshold, output_reference_idx, baseline_lag,
                  first_real_slc_idx, write_crlb, compressed_reference_idx, rasters):
    """One block of the loop (workflows/single.py:215-294): SHPs, phase linking, the
    compressed SLC, and the trimmed results written into the output rasters."""
    torch = D.torch()
    pl, crlb, clos, comp, disp, tcoh, counts, eig, est = rasters
    ir, ic = in_b
    cur = stack[:, ir, ic].contiguous()
    amp_stack = cur.abs() if method == ShpMethod.KS else None
    nb = estimate_neighbors(halfwin_rowcol=(hw.y, hw.x), alpha=shp_alpha, strides=st,
                            mean=None if mean is None else mean[ir, ic].contiguous(),
                            var=None if var is None else var[ir, ic].contiguous(),
                            nslc=shp_nslc, amp_stack=amp_stack, method=method)
    out = run_phase_linking(cur, hw, st, use_evd=use_evd, beta=beta,
                            zero_correlation_threshold=zero_correlation_threshold,
                            reference_idx=output_reference_idx, nodata_mask=nodata[ir, ic].contiguous(),
                            ps_mask=psm[ir, ic].contiguous(), neighbor_arrays=nb, baseline_lag=baseline_lag,
                            avg_mag=None if mean is None else mean[ir, ic].contiguous(),
                            first_real_slc_idx=first_real_slc_idx, compute_crlb=write_crlb)
    cpx = torch.nan_to_num(out.cpx_phase)
    blk_crlb = torch.nan_to_num(out.crlb_std_dev)
    blk_tc = torch.nan_to_num(out.temp_coh)
    tr, tc_ = trim
    fr, fc = in_trim
    inner = cur[:, fr, fc].contiguous()
    bmean, bdisp, _ = calc_ps_block(inner[first_real_slc_idx:].abs().contiguous())
    bcomp = compress(inner, cpx[:, tr, tc_].contiguous(), first_real_slc_idx=first_real_slc_idx, slc_mean=bmean,
                     reference_idx=compressed_reference_idx)
    o_r, o_c = out_b.row_start, out_b.col_start
    part = cpx[first_real_slc_idx:, tr, tc_]
    h, w = part.shape[-2:]
    pl[:, o_r:o_r + h, o_c:o_c + w] = part
    if crlb is not None:
        crlb[:, o_r:o_r + h, o_c:o_c + w] = blk_crlb[first_real_slc_idx:, tr, tc_]
    if clos is not None:
        clos[o_r:o_r + h, o_c:o_c + w] = out.closure_phases[tr, tc_]
    p_r, p_c = no_pad.row_start, no_pad.col_start
    ch, cw = bcomp.shape
    comp[p_r:p_r + ch, p_c:p_c + cw] = bcomp
    disp[p_r:p_r + ch, p_c:p_c + cw] = bdisp
    for dst, src, nd in ((tcoh, blk_tc, 0.0), (counts, out.shp_counts.to(torch.int32), 0.0),
                         (eig, out.eigenvalues, 0.0), (est, out.estimator, 255.0)):
        dst[o_r:o_r + h, o_c:o_c + w] = grow_nodata_region(src[tr, tc_].contiguous(), nodata=nd, n_pixels=2)


def _yx(v, cls):
    if isinstance(v, dict):
        return cls(y=int(v["y"]), x=int(v["x"]))
    y, x = v
    return cls(int(y), int(x))


# ------------------------------------------------------------------------------------
# the sequential chain
# ------------------------------------------------------------------------------------
class SequentialOutput(NamedTuple):
    pl_slcs: object          # (real SLCs, R', C') complex64, every ministack's real SLCs in order
    crlb: object             # same shape, float32, or None
    closure_phases: list     # per ministack: (R', C', size - 2) float32 (or None)
    comp_slcs: list          # per ministack: (R, C) complex64
    temp_coh: list           # per ministack (R', C') float32, then the average if > 1 ministack
    shp_counts: list         # per ministack (R', C') uint16, then the average (int16) if > 1
    similarity: list         # per ministack (R', C') float32, then the radius-11 raster if > 1
    amp_dispersion: list     # per ministack: (R, C) float32 (the compressed SLCs' second band)
    ministacks: list         # the MiniStackPlans
    eigenvalues: list        # per ministack (R', C') float32 (written per ministack by the reference)
    estimator: list          # per ministack (R', C') uint8


def run_wrapped_phase_sequential(slc_stack, *, ministack_size: int, half_window, strides=None,
                                 is_compressed: Optional[Sequence[bool]] = None, nodata_mask=None, ps_mask=None,
                                 amp_mean=None, amp_dispersion=None, shp_method: ShpMethod | str = ShpMethod.NONE,
                                 shp_alpha: float = 0.05, shp_nslc: Optional[int] = None, use_evd: bool = False,
                                 beta: float = 0.0, zero_correlation_threshold: float = 0.0,
                                 similarity_nearest_n: Optional[int] = None,
                                 compressed_slc_plan: CompressedSlcPlan | str = CompressedSlcPlan.ALWAYS_FIRST,
                                 max_num_compressed: int = 100, output_reference_idx: Optional[int] = None,
                                 new_compressed_reference_idx: Optional[int] = None, write_closure_phase: bool = True,
                                 write_crlb: bool = True, block_shape=(512, 512), baseline_lag: Optional[int] = None,
                                 graph: bool = False) -> SequentialOutput:
    """The sequential estimator on a (n, R, C) complex stack: ministacks of
    ``ministack_size`` real SLCs, each led by the compressed SLCs of the ones before.
    ``graph``: each ministack's block loop as one CUDA graph (see
    ``run_wrapped_phase_single``)."""
    torch = D.require_cuda()
    stack = D.to_device(slc_stack, np.complex64)
    n = int(stack.shape[0])
    flags = [False] * n if is_compressed is None else [bool(c) for c in is_compressed]
    if len(flags) != n:
        raise ValueError(f"is_compressed has {len(flags)} entries for {n} layers")
    plans = plan_ministacks(flags, ministack_size, max_num_compressed, compressed_slc_plan, output_reference_idx,
                            new_compressed_reference_idx)
    if shp_nslc is None:
        shp_nslc = n
    comp_list = [stack[i] for i, c in enumerate(flags) if c]
    pls, crlbs, closes, comps, tcs, counts, sims, disps, eigs, ests = [], [], [], [], [], [], [], [], [], []
    for plan in plans:
        layers = [comp_list[i] for i in plan.compressed] + [stack[i] for i in plan.layers]
        cur = torch.stack(layers).contiguous()
        res = run_wrapped_phase_single(
            cur, half_window=half_window, strides=strides, first_real_slc_idx=plan.first_real_slc_idx,
            output_reference_idx=plan.output_reference_idx, compressed_reference_idx=plan.compressed_reference_idx,
            beta=beta, zero_correlation_threshold=zero_correlation_threshold, use_evd=use_evd,
            nodata_mask=nodata_mask, ps_mask=ps_mask, amp_mean=amp_mean, amp_dispersion=amp_dispersion,
            shp_method=shp_method, shp_alpha=shp_alpha, shp_nslc=shp_nslc, similarity_nearest_n=similarity_nearest_n,
            write_closure_phase=write_closure_phase, write_crlb=write_crlb, block_shape=block_shape,
            baseline_lag=baseline_lag, graph=graph)
        comp_list.append(res.comp_slc)
        pls.append(res.pl_slcs)
        crlbs.append(res.crlb)
        closes.append(res.closure_phases)
        comps.append(res.comp_slc)
        disps.append(res.amp_dispersion)
        tcs.append(res.temp_coh)
        counts.append(res.shp_counts)
        sims.append(res.similarity)
        eigs.append(res.eigenvalues)
        ests.append(res.estimator)
        last_pl = res.pl_slcs
    if len(tcs) > 1:
        tcs.append(_average_nodata0(tcs, torch.float32))
        counts.append(_average_nodata0(counts, torch.int16))
    if len(sims) > 1:
        sims.append(stack_similarity(last_pl, search_radius=11, sim_type="median", nearest_n=similarity_nearest_n))
    return SequentialOutput(torch.cat(pls), torch.cat(crlbs) if write_crlb else None, closes, comps, tcs, counts,
                            sims, disps, plans, eigs, ests)


def _average_nodata0(rasters, dtype):
    """gdal_calc's nanmean over rasters whose nodata value is 0: 0 wherever any input
    is 0, else the mean, converted (truncated) to ``dtype``."""
    torch = D.torch()
    a = torch.stack([r.to(torch.float32) for r in rasters])
    any_nd = (a == 0).any(0)
    m = torch.nanmean(a, 0)
    m = torch.where(any_nd, torch.zeros_like(m), m)
    return m.to(dtype)
