"""Copies the reference's golden energy histories into tests/golden/.

The reference's only regression data for this path are the 2stream-em energy
histories (tests/energy_comparison/energies_gold.2stream-em.{float,double} in
the reference tree: 6000 rows of `step time E B`).  The machines that run the
GPU tests do not have the reference tree, so the fixtures are committed; this script regenerates
them from a checkout of the reference.

usage: python tests/golden/make_golden.py REFERENCE_ROOT
   or: CABANAPIC_REFERENCE=REFERENCE_ROOT python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = ["energies_gold.2stream-em.float", "energies_gold.2stream-em.double"]


def main(ref_root: str) -> None:
    src_dir = os.path.join(ref_root, "tests", "energy_comparison")
    for name in NAMES:
        shutil.copyfile(os.path.join(src_dir, name), os.path.join(HERE, name))
        print("wrote", os.path.join(HERE, name))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CABANAPIC_REFERENCE")
    if not root:
        sys.exit(__doc__)
    main(root)
