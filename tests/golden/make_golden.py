"""Generate tests/golden/weibel2d_small.npz: single-thread oracle outputs for a
fixed small 2D Weibel case (16 x 12 cells, 4 particles per cell per species,
seed 2024): the initial state, and the state, energies and CG iteration counts
after 1 and after 3 steps.  The reference has no golden vectors for this path;
these fixtures pin the oracle (C++ restatement) against itself across compilers
and machines, and give the GPU tests a stored target.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.oracle import Oracle2D  # noqa: E402
from wumingpic_gb300 import _build  # noqa: E402
from wumingpic_gb300.loader import Plasma2D, load_weibel2d  # noqa: E402

CASE = dict(nx=16, ny=12, ppc=4, seed=2024, drift=0.5, u_the=0.05)


def run():
    p = Plasma2D(**CASE)
    st = load_weibel2d(p)
    q, r = p.charges()
    o = Oracle2D(nx=p.nx, ny=p.ny, np_cap=p.np_cap, q=q, r=r, delt=p.delt, gfac=p.gfac, threads=1)
    out = {"up0": st.up.copy(), "uf0": st.uf.copy(), "np20": st.np2.copy(), "cumcnt0": st.cumcnt.copy()}
    for k in range(1, 4):
        rc = o.step(st)
        assert rc == 0, rc
        if k in (1, 3):
            out[f"up{k}"] = st.up.copy()
            out[f"uf{k}"] = st.uf.copy()
            out[f"np2{k}"] = st.np2.copy()
            out[f"cumcnt{k}"] = st.cumcnt.copy()
            out[f"energy{k}"] = o.energy(st.up, st.uf, st.np2)
            out[f"cg{k}"] = o.cg_iters()
    return p, out


if __name__ == "__main__":
    _build.build_oracle()
    p, out = run()
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weibel2d_small.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")
