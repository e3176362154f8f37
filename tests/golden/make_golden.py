"""Generates the committed fixtures under tests/golden/.

* rings.pts, swissroll.pts: the reference's own example inputs
  (examples/rings.pts: 400 x 2 f64; examples/swissroll.pts: 1000 x 3 f64),
  copied verbatim so the tests can run where the reference is absent.
* trp-cage.xtc, trp-cage.pdb: the reference's example trajectory (1000
  frames of the 60 backbone atoms of Trp-cage, GROMACS compressed
  coordinates) and its topology, copied verbatim.
* knn_data_*.npz: oracle outputs on those inputs (regression vectors of the
  oracle; the reference itself cannot be built without GROMACS, Boost,
  Berkeley DB and ARPACK).

Run from the repository root:
    python tests/golden/make_golden.py [REFERENCE_CHECKOUT]
The reference checkout defaults to $MDS_REFERENCE, else /root/reference.
"""
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MDS_REFERENCE", "/root/reference")
    REFERENCE_EXAMPLES = os.path.join(ref, "examples")
    for name in ("rings.pts", "swissroll.pts", "trp-cage.xtc", "trp-cage.pdb"):
        src = os.path.join(REFERENCE_EXAMPLES, name)
        if os.path.exists(src):
            shutil.copyfile(src, os.path.join(HERE, name))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    for name, dim, k in (("rings", 2, 12), ("swissroll", 3, 12)):
        x = np.fromfile(os.path.join(HERE, name + ".pts"), dtype=np.float64).reshape(-1, dim)
        d, i = O.knn_data(x, None, k)
        dc, ic = O.knn_data(x, None, k, correlation=True) if dim > 2 else (d[:0], i[:0])
        np.savez_compressed(os.path.join(HERE, f"knn_data_{name}.npz"), d=d, i=i, dc=dc, ic=ic)


if __name__ == "__main__":
    main()
