"""Comparison helpers shared by the parity tests."""
from __future__ import annotations

import numpy as np

FIELD_REL = 1e-4   # relative magnitude tolerance of a received field component
PHASE_RAD = 1e-3   # phase tolerance (rad)


def path_keys(paths):
    """Exact identity of a path set: receiver, launch, facet ids, coplanar ids,
    interaction kinds and ray count, in reference order."""
    return [(p["receiver"], p["launch"], p["n_rays"], tuple(p["tri"]), tuple(p["cop"]),
             tuple(p["kind"])) for p in paths]


def golden_paths(g):
    off = g["path_offset"]
    out = []
    for i in range(len(g["path_receiver"])):
        a, b = int(off[i]), int(off[i + 1])
        out.append({"receiver": int(g["path_receiver"][i]), "launch": int(g["path_launch"][i]),
                    "n_rays": b - a, "tri": g["tri"][a:b].tolist(), "cop": g["cop"][a:b].tolist(),
                    "kind": g["kind"][a:b].tolist(), "points": g["points"][a:b]})
    return out


def golden_field(g):
    return np.ascontiguousarray(g["field"], np.float64).view(np.complex128).reshape(-1, 3)


def _fp_class(v: float) -> str:
    if np.isnan(v):
        return "nan"
    if np.isinf(v):
        return "+inf" if v > 0 else "-inf"
    return "finite"


def field_close(a: np.ndarray, b: np.ndarray, rel=FIELD_REL, phase=PHASE_RAD, floor=None):
    """Per receiver and component: |a-b| <= rel*|b| in magnitude and phase
    within `phase` rad, ignoring components below `floor` (default 1e-9 of the
    receiver's largest finite component), which carry no phase information.
    A component with a NaN or infinite part (a receiver exactly at the
    transmitter: a zero-length path) must have the same NaN/+inf/-inf/finite
    pattern in both real and imaginary parts on both sides; it never passes
    by comparisons that are false for NaN."""
    a = np.asarray(a).reshape(-1, 3)
    b = np.asarray(b).reshape(-1, 3)
    assert a.shape == b.shape
    bad = []
    for k in range(len(b)):
        fin = [abs(v) for v in b[k] if np.isfinite(v)]
        scale = max(fin) if fin else 0.0
        fl = (floor if floor is not None else 1e-9) * max(scale, 1e-300)
        for j in range(3):
            x, y = a[k, j], b[k, j]
            if not (np.isfinite(x) and np.isfinite(y)):
                cx = (_fp_class(x.real), _fp_class(x.imag))
                cy = (_fp_class(y.real), _fp_class(y.imag))
                if cx != cy:
                    bad.append((k, j, x, y, "non-finite"))
                continue
            if abs(y) <= fl and abs(x) <= fl + rel * scale:
                continue
            if abs(abs(x) - abs(y)) > rel * abs(y) + fl:
                bad.append((k, j, x, y, "mag"))
                continue
            if abs(y) > 100 * fl and abs(np.angle(x / y)) > phase:
                bad.append((k, j, x, y, "phase"))
    return bad


def max_rel_err(a, b):
    """Largest |a - b| / |b| over the components that are finite on both
    sides (field_close checks that the non-finite ones agree)."""
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    m = np.isfinite(a) & np.isfinite(b) & (b != 0)
    if not m.any():
        return 0.0
    return float(np.max(np.abs(a[m] - b[m]) / np.abs(b[m])))
