"""Write tests/golden/c0_pin.npz: the c0 system's integer G-sphere maps, a few
operator tables and the oracle's multishift solution for band 0.

The fixture pins the synthetic generator (bit-exact integer maps) and the
oracle across machines.  Regenerate with
    python tests/golden/make_c0.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import linter_ref  # noqa: E402
from oracle import oracle as O  # noqa: E402
from sternheimergw_gb300 import linter, synth  # noqa: E402


def main():
    s, f = synth.config("c0")
    bb = linter_ref.coulomb_rhs(s, 0)
    sh = linter.coulomb_shifts(s, f)
    op = O.PlaneWaveOperator(s)
    xx, ierr, iters, applies = O.bicgstab(op, bb[0], sh[0], lmax=4, threshold=1e-10)
    assert ierr == 0
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "c0_pin.npz")
    np.savez_compressed(out, mill=s["mill"], nl=s["nl"], mill_k=s["mill_k"], nl_k=s["nl_k"], nr=s["nr"],
                        g2kin=s["g2kin"], vrs=s["vrs"], dvan=s["dvan"], et=s["et"], alpha_pv=s["alpha_pv"],
                        bb0=bb[0], sigma0=sh[0], x0=xx, iters0=iters)
    print("wrote", out, "npw", s["npw"], "iters", iters)


if __name__ == "__main__":
    main()
