"""Field-by-field comparison of two EPIC states (test helper)."""
from __future__ import annotations

import numpy as np

from epic_gb300.abi import Fields

PROGNOSTIC = ("u", "v", "hdry", "theta")
DIAGNOSTIC = ("p3", "h3", "p2", "theta2", "t2", "t3", "rho2", "rho3", "exner3", "gz3", "mont3", "heat3",
              "pv3", "ri2", "div_uv3", "w3", "dzdt3")


def field_errors(a: Fields, b: Fields, names=None) -> dict:
    """Relative L2 and max relative error per field of a against b.

    Cells holding the time-scheme start flag (DBL_MAX) must agree exactly and are then left out.
    """
    out = {}
    for k in names or a.arrays.keys():
        x, y = a.arrays[k], b.arrays[k]
        big = np.abs(y) > 1e300
        if not np.array_equal(np.abs(x) > 1e300, big) or not np.array_equal(x[big], y[big]):
            out[k] = (float("inf"), float("inf"))
            continue
        x = np.where(big, 0., x)
        y = np.where(big, 0., y)
        den = np.linalg.norm(y.ravel())
        num = np.linalg.norm((x - y).ravel())
        scale = np.max(np.abs(y)) if y.size else 0.
        rel = num / den if den > 0 else num
        mx = np.max(np.abs(x - y)) / scale if scale > 0 else np.max(np.abs(x - y))
        out[k] = (float(rel), float(mx))
    return out


def worst(errs: dict) -> tuple[str, float]:
    k = max(errs, key=lambda n: errs[n][0])
    return k, errs[k][0]
