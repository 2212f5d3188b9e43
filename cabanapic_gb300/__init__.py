"""GB300-native implementation of CabanaPIC's per-step particle hot path.

The CUDA kernels and the C ABI live in libcpic.so (csrc/, include/cpic/);
this package holds the host-side mirror of the reference's interface
(pic.py), its containers (arrays.py), layout helpers (layout.py), decks and
initializers (decks.py) and a time-loop driver (simulation.py).
"""
from . import layout, decks  # noqa: F401
