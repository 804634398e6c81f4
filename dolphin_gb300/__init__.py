"""GB300-native phase linking: a drop-in for dolphin's phase-linking hot path.

Public entry points keep the reference's names, arguments and outputs:

* :func:`run_phase_linking`  (dolphin.phase_link.run_phase_linking)
* :func:`estimate_neighbors` (dolphin.shp.estimate_neighbors)
* :func:`calc_ps_block`      (dolphin.ps.calc_ps_block)
* :func:`compress`           (dolphin.phase_link.compress)
* :func:`median_similarity`, :func:`max_similarity`, :func:`get_circle_idxs`
  (dolphin.similarity)
* :func:`run_wrapped_phase_single`, :func:`run_wrapped_phase_sequential` (the block
  loop of dolphin.workflows.single / .sequential on device arrays, without raster I/O)

:func:`deferred_checks` (not in the reference) lets a block loop of device-resident
``run_phase_linking`` calls run without a host synchronisation per call.

All compute runs in hand-written CUDA kernels for sm_103a behind the C ABI in
``include/dpl.h`` (``dolphin_gb300/_lib/libdpl.so``).  Importing this package
does not initialise CUDA, so it is safe in spawned worker processes.
"""

from __future__ import annotations

from ._types import HalfWindow, ShpMethod, Strides
from .batch import PhaseLinkBatch, tune_forms
from .compress import compress
from .phase_link import (
    EstimatorType,
    PhaseLinkOutput,
    PhaseLinkRuntimeError,
    deferred_checks,
    estimate_stack_covariance,
    process_coherence_matrices,
    run_phase_linking,
)
from .ps import calc_ps_block
from .shp import estimate_neighbors
from .similarity import get_circle_idxs, max_similarity, median_similarity, stack_similarity
from .workflow import (
    StridedBlockManager,
    clear_loop_graphs,
    grow_nodata_region,
    plan_ministacks,
    run_wrapped_phase_sequential,
    run_wrapped_phase_single,
)

__all__ = [
    "EstimatorType",
    "HalfWindow",
    "PhaseLinkBatch",
    "PhaseLinkOutput",
    "PhaseLinkRuntimeError",
    "ShpMethod",
    "Strides",
    "StridedBlockManager",
    "calc_ps_block",
    "clear_loop_graphs",
    "compress",
    "deferred_checks",
    "estimate_neighbors",
    "estimate_stack_covariance",
    "get_circle_idxs",
    "grow_nodata_region",
    "install_into_dolphin",
    "max_similarity",
    "median_similarity",
    "plan_ministacks",
    "process_coherence_matrices",
    "run_phase_linking",
    "run_wrapped_phase_sequential",
    "run_wrapped_phase_single",
    "stack_similarity",
    "tune_forms",
]

# (module, attribute) pairs of an installed dolphin that bind the hot path by name
# (workflows/single.py:18-23 imports run_phase_linking, shp and calc_ps_block).
_PATCH_TARGETS = (
    ("dolphin.phase_link", "run_phase_linking"),
    ("dolphin.phase_link._core", "run_phase_linking"),
    ("dolphin.workflows.single", "run_phase_linking"),
    ("dolphin.shp", "estimate_neighbors"),
    ("dolphin.ps", "calc_ps_block"),
    ("dolphin.workflows.single", "calc_ps_block"),
    ("dolphin.phase_link", "compress"),
    ("dolphin.phase_link._compress", "compress"),
    ("dolphin.workflows.single", "compress"),
    # similarity.py:300-303 looks median_similarity / max_similarity up at call time
    ("dolphin.similarity", "median_similarity"),
    ("dolphin.similarity", "max_similarity"),
)


def install_into_dolphin(modules=None):
    """Route an installed dolphin's phase-linking calls to this package.

    Rebinds each ``(module, attribute)`` in ``_PATCH_TARGETS`` that can be
    imported, and makes this package raise dolphin's own
    ``PhaseLinkRuntimeError`` so the workflow's ``except`` clauses keep working.
    ``modules`` (for tests) maps module names to already-imported module objects.
    Returns the list of patched ``module.attribute`` names.
    """
    import importlib

    from . import phase_link as _pl

    funcs = {
        "run_phase_linking": run_phase_linking,
        "estimate_neighbors": estimate_neighbors,
        "calc_ps_block": calc_ps_block,
        "compress": compress,
        "median_similarity": median_similarity,
        "max_similarity": max_similarity,
    }
    patched = []

    def get(name):
        if modules is not None:
            return modules.get(name)
        try:
            return importlib.import_module(name)
        except ImportError:
            return None

    core = get("dolphin.phase_link._core")
    if core is not None and hasattr(core, "PhaseLinkRuntimeError"):
        _pl.PhaseLinkRuntimeError = core.PhaseLinkRuntimeError
    for mod_name, attr in _PATCH_TARGETS:
        mod = get(mod_name)
        if mod is None:
            continue
        setattr(mod, attr, funcs[attr])
        patched.append(f"{mod_name}.{attr}")
    return patched
