"""Numpy restatement of dolphin's phase-similarity raster (ORACLE, test infrastructure).

Only the tests and the bench's CPU baseline use this module; the product computes the
raster with ``dpl_similarity_prep`` / ``dpl_similarity`` on the GPU.

Follows ``similarity.py`` of the reference:

* ``phase_similarity`` 21-28: mean over the stack of Re(x1 conj x2); numba
  accumulates the float32 products in float64.
* ``_create_loop_and_run`` 96-117: a pixel is invalid where the sum over the stack of
  ``nan_to_num(z)`` is exactly 0; the comparison phasors are exp(i angle z) (complex
  input) or exp(i phase) (real input); the mask is cleared on invalid pixels, in place.
* ``_make_loop_function`` 120-173: for each unmasked pixel, every circle offset is
  clipped to the image; the pixel itself and masked neighbours are skipped; the
  summary (nanmedian or nanmax) of the remaining similarities is written, NaN when
  there are none.
* ``get_circle_idxs`` 176-254: concentric midpoint circles of radius 1 .. R-1, each
  extended inward along its rows until it meets the previous one.
* ``_calc_nearest_diffs`` 355-366 and ``_create_nearest_n_pairs`` 369-375: phase
  differences of the nearest-n pairs of a single-reference stack, via the incidence
  matrix of ``timeseries.get_incidence_matrix`` (594-644).

The offsets are enumerated ring by ring, as in the reference, because their order
(``sort_output=False``) and the exact set depend on those steps.
"""

from __future__ import annotations

import numpy as np

__all__ = [
    "circle_offsets",
    "max_similarity",
    "median_similarity",
    "nearest_diffs",
    "nearest_n_pairs",
    "phase_similarity",
    "similarity",
]


def circle_offsets(max_radius: int, min_radius: int = 0, sort_output: bool = True) -> np.ndarray:
    """(K, 2) (row, col) offsets of the search circle."""
    filled = np.zeros((max_radius, max_radius), dtype=bool)  # first-quadrant cells already covered
    filled[0, 0] = True
    found = []
    for ring in range(1, max_radius):
        emit = ring > min_radius
        if emit:
            found += [[ring, 0], [-ring, 0], [0, ring], [0, -ring]]
        filled[ring, 0] = filled[0, ring] = True
        # walk the first octant (b <= a) of the midpoint circle of radius `ring`
        a, b, decision, backlog = ring, 0, 1 - ring, 0
        while a > b:
            if backlog:
                backlog -= 1  # revisit the cells skipped while reaching inward
            else:
                b += 1
                if decision <= 0:
                    decision += 2 * b + 1
                else:
                    a -= 1
                    decision += 2 * b - 2 * a + 1
            if a < b:
                break
            while not filled[a - 1, b]:  # reach inward to the previous ring
                a -= 1
                backlog += 1
            filled[a, b] = filled[b, a] = True
            if emit:
                found += [[a, b], [-a, -b], [a, -b], [-a, b]]
                if a != b:
                    found += [[b, a], [-b, -a], [b, -a], [-b, a]]
            if backlog:
                a += 1
    return np.array(sorted(found)) if sort_output else np.array(found)


def phase_similarity(x1, x2) -> float:
    """Mean of Re(x1 conj x2); float32 products summed in float64."""
    x1, x2 = np.asarray(x1), np.asarray(x2)
    prod = (x1 * np.conj(x2)).real
    return float(np.sum(prod.astype(np.float64))) / len(x1)


def _phasors(ifg_stack):
    """Comparison phasors exp(i angle z) / exp(i phase) and the invalid mask."""
    z = np.asarray(ifg_stack)
    total = np.zeros(z.shape[1:], dtype=z.dtype)
    for layer in np.nan_to_num(z):  # numpy's reduction over the first axis: layer by layer
        total = total + layer
    invalid = total == 0
    if np.iscomplexobj(z):
        unit = np.exp(1j * np.angle(z))
    else:
        unit = np.exp(1j * z)
    return unit, invalid


def similarity(ifg_stack, search_radius: int, mask=None, kind: str = "median") -> np.ndarray:
    """median (``kind="median"``) or max similarity of each pixel with its neighbours."""
    unit, invalid = _phasors(ifg_stack)
    n, rows, cols = unit.shape
    out = np.full((rows, cols), np.nan, dtype=np.float32)
    if mask is None:
        mask = np.ones((rows, cols), dtype=bool)
    mask[invalid] = False
    if mask.shape != (rows, cols):
        raise ValueError(f"{unit.shape = }, but {mask.shape = }")
    offs = circle_offsets(search_radius)
    if len(offs) == 0:
        return out
    rr, cc = np.meshgrid(np.arange(rows), np.arange(cols), indexing="ij")
    sims = np.full((len(offs), rows, cols), np.nan)
    for k, (dr, dc) in enumerate(offs):
        r = np.clip(rr + dr, 0, rows - 1)
        c = np.clip(cc + dc, 0, cols - 1)
        prod = (unit * np.conj(unit[:, r, c])).real
        s = prod.astype(np.float64).sum(axis=0) / n
        use = mask & mask[r, c] & ~((r == rr) & (c == cc))
        sims[k][use] = s[use]
    with np.errstate(all="ignore"):
        import warnings

        with warnings.catch_warnings():
            warnings.simplefilter("ignore", RuntimeWarning)
            summary = np.nanmedian(sims, axis=0) if kind == "median" else np.nanmax(sims, axis=0)
    out[mask] = summary[mask]
    return out


def median_similarity(ifg_stack, search_radius: int, mask=None) -> np.ndarray:
    return similarity(ifg_stack, search_radius, mask, "median")


def max_similarity(ifg_stack, search_radius: int, mask=None) -> np.ndarray:
    return similarity(ifg_stack, search_radius, mask, "max")


def nearest_n_pairs(num_files: int, n: int = 3) -> list[tuple[int, int]]:
    """(i, j) with i < j <= i + n and j < num_files."""
    return [(i, j) for i in range(num_files) for j in range(i + 1, min(i + n, num_files - 1) + 1)]


def nearest_diffs(block, n: int) -> np.ndarray:
    """exp(i (phi_j - phi_i)) over the nearest-n pairs of a single-reference stack
    (layer t holds date t+1 against date 0); NaN where the pixel's layers sum to 0."""
    block = np.asarray(block)
    num, rows, cols = block.shape
    pairs = nearest_n_pairs(num + 1, n)
    A = np.zeros((len(pairs), num))
    for k, (i, j) in enumerate(pairs):
        if i >= 1:
            A[k, i - 1] = -1
        A[k, j - 1] = 1
    nodata = np.nan_to_num(block).sum(axis=0) == 0
    phase = np.angle(block) if np.iscomplexobj(block) else block
    diffs = (A @ phase.reshape(num, -1)).reshape(len(pairs), rows, cols)
    diffs[:, nodata] = np.nan
    return np.exp(1j * diffs)
