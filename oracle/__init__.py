"""CPU oracle for the CabanaPIC hot path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
this package, and only as the test oracle or the reference arm.  The shipped
library (cabanapic_gb300) never imports it.
"""
from .oracle import Oracle, load  # noqa: F401
from . import energy_rule  # noqa: F401
from . import diagnostics  # noqa: F401
