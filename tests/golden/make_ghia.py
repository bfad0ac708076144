"""Generate tests/golden/lid_driven_ghia.npz from the profiles FEN ships with its lid-driven
cavity test (test/small_test/navier_stokes/lid_driven/uref and vref).

Those two text files hold FEN's reference centreline profiles for the Re = 1000 cavity
(64^2, walls on every side, nu = 1e-3, lid velocity 1): uref is (y - 1/2, u) along the
vertical centreline, vref is (x - 1/2, v) along the horizontal one; FEN's postpro.py plots
them against the steady solution (postpro.py:50-66).  The arrays are stored unchanged, in
file order.  Run from the repository root with FEN's sources at ../reference or at the
path given as the first argument:

    python tests/golden/make_ghia.py /path/to/FEN
"""
import os
import sys

import numpy as np


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    src = sys.argv[1] if len(sys.argv) > 1 else os.path.join(here, "..", "..", "..", "reference")
    d = os.path.join(src, "test", "small_test", "navier_stokes", "lid_driven")
    uref = np.genfromtxt(os.path.join(d, "uref"))
    vref = np.genfromtxt(os.path.join(d, "vref"))
    out = os.path.join(here, "lid_driven_ghia.npz")
    np.savez(out, uref=uref, vref=vref)
    print(out, uref.shape, vref.shape)


if __name__ == "__main__":
    main()
