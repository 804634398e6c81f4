"""Wrapped-phase workflow, CPU side: the block manager and the ministack planner against
the reference's own StridedBlockManager and MiniStackPlanner, and the workflow oracle
against a two-ministack sequential run made from the reference's per-block functions."""

import json

import numpy as np
import pytest

from oracle import workflow as OW
from parity import compare_workflow

NONE_IDX = -(2**31)


@pytest.fixture(scope="module")
def g(golden):
    return golden("workflow")


def _dec(v):
    return None if v == NONE_IDX else int(v)


def _blocks_ref(g, k):
    rows = g[f"blocks_{k}"]
    return [tuple(tuple(_dec(v) for v in r[4 * j:4 * j + 4]) for j in range(5)) for r in rows]


def test_block_manager_matches_reference(g):
    from dolphin_gb300._types import HalfWindow, Strides
    from dolphin_gb300.workflow import StridedBlockManager

    for k in range(int(g["nblock_cfgs"])):
        cfg = g[f"blocks_cfg_{k}"].tolist()
        mgr = StridedBlockManager(tuple(cfg[0:2]), tuple(cfg[2:4]), Strides(*cfg[4:6]), HalfWindow(*cfg[6:8]))
        got = [tuple((b.row_start, b.row_stop, b.col_start, b.col_stop) for b in blk) for blk in mgr.iter_blocks()]
        assert got == _blocks_ref(g, k), k
        assert OW.blocks(tuple(cfg[0:2]), tuple(cfg[2:4]), tuple(cfg[4:6]), tuple(cfg[6:8])) == _blocks_ref(g, k)


def test_planner_matches_reference(g):
    from dolphin_gb300.workflow import plan_ministacks

    for case in json.loads(str(g["plans"])):
        got = plan_ministacks([False] * case["n"], case["size"], case["max_comp"], case["plan"], case["out_ref"])
        assert len(got) == len(case["ministacks"])
        for p, ref in zip(got, case["ministacks"]):
            layers = [-(1 + c) for c in p.compressed] + p.layers
            assert layers == ref["layers"]
            assert p.is_compressed == ref["is_compressed"]
            assert (p.output_reference_idx, p.compressed_reference_idx) == (ref["out_ref"], ref["comp_ref"])
            assert p.first_real_slc_idx == ref["first_real"]
        if case["plan"] == "always_first":
            oracle = OW.plan(case["n"], case["size"], case["max_comp"], case["plan"], case["out_ref"])
            assert [o[0] for o in oracle] == [m["layers"] for m in case["ministacks"]]
            assert [(o[2], o[3]) for o in oracle] == [(m["out_ref"], m["comp_ref"]) for m in case["ministacks"]]


def test_planner_errors_and_existing_compressed():
    from dolphin_gb300.workflow import plan_ministacks

    with pytest.raises(ValueError):
        plan_ministacks([False] * 5, 1)
    with pytest.raises(ValueError):
        plan_ministacks([False] * 5, 2, compressed_idx=0)
    with pytest.raises(ValueError):
        plan_ministacks([False] * 5, 2, compressed_slc_plan="last_per_ministack")
    with pytest.raises(UnboundLocalError):
        plan_ministacks([False] * 5, 2, compressed_slc_plan="first_per_ministack")
    # two compressed inputs lead the stack: the first ministack starts after them and
    # carries both, the next one the last max_num_compressed
    p = plan_ministacks([True, True] + [False] * 6, 3, max_num_compressed=2)
    assert [x.layers for x in p] == [[2, 3, 4], [5, 6, 7]]
    assert [x.compressed for x in p] == [[0, 1], [1, 2]]
    assert [x.first_real_slc_idx for x in p] == [2, 2]
    assert p[0].compressed_reference_idx == 1


def test_oracle_grow_nodata_matches_reference(g):
    for k in range(int(g["ngrow"])):
        nd = float(g[f"grow_nd_{k}"])
        got = OW.grow_nodata_region(g[f"grow_in_{k}"], nd if not np.isnan(nd) else np.nan, int(g[f"grow_n_{k}"]))
        np.testing.assert_array_equal(got, g[f"grow_out_{k}"])


def _golden_run(g, k):
    keys = ("pl", "crlb", "clos", "comp", "disp", "tc", "counts", "eig", "est", "sim")
    return {key: g[f"seq{k}_{key}"] for key in keys}


def test_oracle_sequential_matches_reference(g):
    cfg = g["seq_cfg"].tolist()
    outs, _extra = OW.sequential(g["seq_slc"], cfg[6], tuple(cfg[0:2]), tuple(cfg[2:4]), tuple(cfg[4:6]),
                                 g["seq_nodata"], g["seq_ps"], g["seq_amp_mean"], g["seq_amp_disp"])
    assert len(outs) == 2
    for k, o in enumerate(outs):
        compare_workflow(o, _golden_run(g, k))
