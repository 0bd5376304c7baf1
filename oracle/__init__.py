"""CPU oracle for the seistorch 2D wave-propagation hot path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline / reference arm of ``bench.py`` may import this package, and only
as the checker or the timed CPU baseline.  The product (``seistorch_gb300``)
never imports it and has no CPU fallback.

``fd2d`` restates, in numpy (float64 by default, any dtype on request), the
reference's discrete algorithms with file:line citations; ``adjoint`` holds
the exact discrete adjoints used as gradient oracles.  Parity of this
restatement is pinned against golden vectors produced by running the
reference's own code (``tests/golden/make_golden.py``).
"""
from . import fd2d  # noqa: F401
