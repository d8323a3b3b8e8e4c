"""Write the reference's Held-Suarez temperature sounding (data/held_suarez/t_vs_p.held_suarez)
as tests/golden/sounding/t_vs_p_held_suarez.npz: pressures [Pa] and temperatures [K] bottom level first,
the order in which read_t_vs_p stores them (src/shared/epic_funcs_io.c:4027-4088).  Run where the
reference tree is present; the fixture travels, the reference does not.

    python tests/golden/make_sounding.py [reference_dir]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_t_vs_p(path):
    with open(path) as fh:
        lines = fh.read().splitlines()
    body = lines[6:]                       # a six-line header, then the level count
    n = int(body[0].split()[0])
    rows = [ln.split() for ln in body[1:1 + n]]
    p = np.array([float(r[0]) for r in rows]) * 100.   # hPa -> Pa
    t = np.array([float(r[1]) for r in rows])
    return p[::-1].copy(), t[::-1].copy()  # bottom level first


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    p, t = read_t_vs_p(os.path.join(ref, "data", "held_suarez", "t_vs_p.held_suarez"))
    out = os.path.join(HERE, "sounding", "t_vs_p_held_suarez.npz")
    np.savez_compressed(out, p=p, t=t)
    print(out, p.size, "levels", p[0], "..", p[-1], "Pa")
