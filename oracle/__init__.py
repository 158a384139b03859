"""CPU oracle for the LoopStructural discrete-interpolation hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in ``loopstructural_gb300`` imports this
package; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs
of ``bench.py`` use it, and there only as the checker or as the timed CPU
baseline -- never as the thing measured on the GPU or shipped.

The modules restate, in plain numpy/scipy, the algorithms of the reference
(Loop3D/LoopStructural 1.8.0, packages ``loop_common`` and
``loop_interpolation``).  Every function cites the reference file:line it
follows.  The restatement is pinned against golden vectors produced by the
reference itself (``tests/golden/make_golden.py`` imports the reference in a
container where it is available and writes ``tests/golden/*.npz``); the pins
are checked by ``tests/test_oracle_golden.py``.
"""

from . import fd_oracle, p1_oracle  # noqa: F401
