"""CPU oracle for the phase-linking hot path.

ORACLE -- TEST INFRASTRUCTURE ONLY.  Nothing in ``dolphin_gb300`` imports this
package.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` use it, and only to check or time against the CUDA path.

``phase_link`` is a numpy restatement of the reference's algorithm
(dolphin, ``src/dolphin/phase_link``, ``src/dolphin/shp``, ``src/dolphin/ps.py``),
parametrised by precision: ``dtype=np.float32`` mirrors the reference's own
float32/complex64 arithmetic (jax with x64 disabled), ``dtype=np.float64`` is
the float64 oracle used to state every result's error.

Parity pin: ``tests/golden/*.npz`` were produced by running the reference's
own Python source (loaded from its checkout, with numpy stand-ins for the jax
and numba APIs it calls; see ``tests/golden/make_golden.py``).
``tests/test_oracle_golden.py`` checks this restatement against them.
"""

from . import phase_link  # noqa: F401
