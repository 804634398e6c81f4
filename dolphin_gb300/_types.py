"""Named tuples and enums of the reference's phase-linking interface (``_types.py:57-68``,
``workflows/config/_enums.py:9-16``), with the same field order (y, x)."""

from __future__ import annotations

from enum import Enum
from typing import NamedTuple


class Strides(NamedTuple):
    """Decimation/striding factor in the y (row) and x (column) directions."""

    y: int
    x: int


class HalfWindow(NamedTuple):
    """Half-window size in the y (row) and x (column) directions."""

    y: int
    x: int


class ShpMethod(str, Enum):
    """Method for finding SHPs during phase linking."""

    GLRT = "glrt"
    KS = "ks"
    RECT = "rect"
    NONE = "rect"
