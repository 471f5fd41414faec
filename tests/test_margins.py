"""The FP32 filters' error margins against the FP64 decisions they stand in for.

The capture stage decides most (node, receiver) pairs in FP32 and leaves the
rest to FP64: the correction cone culls receivers with planes formed in FP64
and rounded to FP32, loosened by 2 m, m = 2^-19 |n| (cmax + |img| + |T| + 1)
(sbr_capture.cuh, k_class_cones in sbr_trace.cuh); the reception test
(reception32 in sbr_kernels.cuh) calls a pair certain only outside
2^-16 (|s| + |c| + 1 + S + |P|) of the sphere's surface.  These tests replay
the FP32 arithmetic with numpy float32 on adversarial geometry (points on or
next to the boundaries, far image sources, small and large triangles) and
check that no FP32 decision contradicts the FP64 one."""
import numpy as np

F32 = np.float32
CONE_K = F32(1.9073486328125e-06)  # 2^-19
REC_K = F32(1.52587890625e-05)     # 2^-16


def _dot32(a, b):
    a = np.asarray(a, F32)
    b = np.asarray(b, F32)
    return F32(F32(F32(a[0] * b[0]) + F32(a[1] * b[1])) + F32(a[2] * b[2]))


def _norm32(a):
    return F32(np.sqrt(_dot32(a, a)))


def _scene(rng):
    scale = 10 ** rng.uniform(-1, 2)                   # triangle size 0.1 .. 100 m
    c0 = rng.uniform(-1000, 1000, 3)
    v = (c0 + rng.normal(0, scale, (3, 3))).astype(F32).astype(np.float64)
    d = rng.normal(size=3)
    img = c0 + d / np.linalg.norm(d) * 10 ** rng.uniform(0, 4)  # 1 m .. 10 km away
    return v, img


def test_cone_planes_never_reject_a_point_of_the_exact_cone():
    rng = np.random.default_rng(11)
    cmax = 1500.0
    checked = 0
    for _ in range(20000):
        v, img = _scene(rng)
        g = v.mean(0)
        tmag = (np.linalg.norm(img) + np.linalg.norm(v[0]) + np.linalg.norm(v[1] - v[0]) +
                np.linalg.norm(v[2] - v[0]))
        # a point on the plane through img and a random edge, beyond the triangle,
        # jittered by a few FP64 ulps either way
        k = rng.integers(3)
        e = v[k] + rng.uniform(0, 1) * (v[(k + 1) % 3] - v[k])
        x = img + rng.uniform(1.0, 5.0) * (e - img)
        x = x + rng.normal(0, 1e-12, 3) * np.linalg.norm(x)
        if np.linalg.norm(x) > cmax:
            continue
        inside, passes, usable = True, True, True
        for kk in range(3):
            a, b = v[kk] - img, v[(kk + 1) % 3] - img
            n = np.cross(a, b)
            gc = n @ (g - img)
            n = n if gc > 0 else -n
            nn = np.linalg.norm(n)
            m = CONE_K * (F32(nn) * F32(cmax) + F32(nn) * F32(tmag + 1.0))
            if not abs(gc) > 4 * m:
                usable = False  # k_capture uses no cone for such a class
                break
            inside &= bool(n @ (x - img) >= 0)
            lhs = _dot32(n.astype(F32), x.astype(F32))
            passes &= bool(lhs >= F32(F32(n @ img) - F32(2) * m))
        if not usable:
            continue
        checked += 1
        assert passes or not inside
    assert checked > 10000


def _reception64(s, t, c, path_len, tanb):
    rd, w = t - s, c - s
    t0 = (rd @ w) / (rd @ rd)
    if t0 < 0:
        return False
    t0 = min(t0, 1.0)
    p = s + t0 * rd
    return np.linalg.norm(c - p) <= (path_len + np.linalg.norm(p)) * tanb


def _reception32(s, u, seg_len, S, c, tanb):
    s, u, c = s.astype(F32), u.astype(F32), c.astype(F32)
    w = (c - s).astype(F32)
    lam = _dot32(u, w)
    mag = F32(_norm32(s) + _norm32(c) + F32(1))
    ml = REC_K * mag
    if lam < -ml:
        return 0
    if lam <= ml:
        return -1
    lc = min(lam, F32(seg_len))
    p = (s + (lc * u).astype(F32)).astype(F32)
    npn = _norm32(p)
    dist = _norm32((c - p).astype(F32))
    rad = F32(F32(F32(S) + npn) * F32(tanb))
    mr = REC_K * F32(mag + F32(S) + npn)
    if dist > rad + mr:
        return 0
    if dist < rad - mr:
        return 1
    return -1


def test_reception_margin_agrees_with_the_fp64_test():
    rng = np.random.default_rng(12)
    tanb = np.tan(np.arccos(-1 / np.sqrt(5)) / (3 * 10))  # level 9
    decided = 0
    for _ in range(20000):
        s = rng.uniform(-800, 800, 3)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        seg = 10 ** rng.uniform(-1, 3)
        t = s + seg * d
        S = rng.uniform(0, 3000)
        # a receiver near the sphere's surface around a point of the segment
        p = s + rng.uniform(-0.1, 1.1) * seg * d
        r = (S + np.linalg.norm(p)) * tanb
        margin = float(REC_K) * (np.linalg.norm(s) + np.linalg.norm(p) + r + 1 + S +
                                 np.linalg.norm(p))
        off = rng.normal(size=3)
        # within a few margins of the surface: decided pairs sit just outside it
        c = p + off / np.linalg.norm(off) * (r + rng.uniform(-3, 3) * margin)
        v32 = _reception32(s, d, seg, S, c, tanb)
        if v32 < 0:
            continue
        decided += 1
        assert bool(v32) == _reception64(s, t, c, S, tanb)
    assert decided > 5000
