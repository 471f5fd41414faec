"""Seeded synthetic scenes for the SBR hot path.

The reference ships no benchmark scenes, so workloads are generated here:
an axis-aligned-box city over a ground plane (small and urban-canyon sizes),
and a fractal terrain with extruded polygons (large scene).  Every random
draw comes from a project-written PCG32 stream and every coordinate is
formed with IEEE +,-,*,/ only before rounding to float32, so the same seed
gives bit-identical triangles on any host.  Scenes are written as binary
STL (the reference's input format, SBRSolver_rev2/StlReader.h) plus a
per-triangle material-id list, because the reference assigns materials per
triangle after loading (Triangle::materialId, SBRSolver_rev2/Triangle.h:30).

Material constants: relative permittivity as given for each workload;
conductivities follow ITU-R P.2040-1 Table 3 (sigma = c * f_GHz**d) for
concrete (c=0.0326, d=0.8095) and glass (c=0.0043, d=1.1925).
"""
from __future__ import annotations

import math
import os
import struct
from dataclasses import dataclass, field
from typing import List, Sequence, Tuple

import numpy as np


class PCG32:
    """PCG-XSH-RR 64/32 (O'Neill 2014), the published minimal generator."""

    MULT = 6364136223846793005
    MASK = (1 << 64) - 1

    def __init__(self, seed: int, stream: int = 54):
        self.state = 0
        self.inc = ((stream << 1) | 1) & self.MASK
        self.next_u32()
        self.state = (self.state + seed) & self.MASK
        self.next_u32()

    def next_u32(self) -> int:
        old = self.state
        self.state = (old * self.MULT + self.inc) & self.MASK
        xorshifted = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xorshifted >> rot) | (xorshifted << ((-rot) & 31))) & 0xFFFFFFFF

    def uniform(self, lo: float, hi: float) -> float:
        """lo + (hi-lo)*k/2**32 with k a 32-bit draw: exact dyadic arithmetic."""
        return lo + (hi - lo) * (self.next_u32() / 4294967296.0)

    def randint(self, n: int) -> int:
        return self.next_u32() % n

    def normal(self) -> float:
        """Box-Muller; used only for scenes that are not golden fixtures."""
        u1 = (self.next_u32() + 1.0) / 4294967297.0
        u2 = self.next_u32() / 4294967296.0
        return math.sqrt(-2.0 * math.log(u1)) * math.cos(2.0 * math.pi * u2)


def p2040_sigma(c: float, d: float, f_hz: float) -> float:
    return c * (f_hz / 1e9) ** d


# (frequency, transmissionLoss, reflectionLoss, relPermittivityRe,
#  relPermittivityIm, relConductivity): MaterialProperties field order,
#  SBRSolver_rev2/common/DataStructures.h:20-28, optionally followed by a wall
#  thickness in metres (slab coefficients; the reference's is always 0).
Material = Tuple[float, ...]


@dataclass
class Scene:
    name: str
    tri: np.ndarray          # (n, 3, 3) float32 vertices v1, v2, v3
    normal: np.ndarray       # (n, 3) float32 facet normals (as written to the STL)
    material_id: np.ndarray  # (n,) int32
    materials: List[Material]

    @property
    def n_tri(self) -> int:
        return int(self.tri.shape[0])


@dataclass
class Request:
    """One propagation solve; argument meaning of RTSolver::ExecuteRayTracing
    (SBRSolver_rev2/RTSolver.h:25-37) plus the antenna type the reference
    hard-codes (FieldCompute.cpp:117, 1 = Hertzian)."""

    tx: Tuple[float, float, float]
    rx: np.ndarray                      # (m, 3) float64
    max_reflection: int
    max_transmission: int
    frequency: float
    tessellation: int
    tx_coord_sys: Tuple[float, ...] = (1, 0, 0, 0, 1, 0, 0, 0, 1)  # row-major 3x3
    pt: float = 1.0
    use_fresnel: bool = True
    antenna: int = 1


@dataclass
class Workload:
    name: str
    scene: Scene
    request: Request
    notes: dict = field(default_factory=dict)


# ---------------------------------------------------------------- geometry

class _MeshBuilder:
    def __init__(self):
        self.tris: List[Tuple[Tuple[float, float, float], ...]] = []
        self.normals: List[Tuple[float, float, float]] = []
        self.mats: List[int] = []

    def tri(self, a, b, c, n, mat):
        self.tris.append((tuple(a), tuple(b), tuple(c)))
        self.normals.append(tuple(n))
        self.mats.append(int(mat))

    def quad(self, a, b, c, d, n, mat):
        """Quad a-b-c-d (counter-clockwise seen from the normal side)."""
        self.tri(a, b, c, n, mat)
        self.tri(a, c, d, n, mat)

    def box(self, x0, y0, x1, y1, z0, z1, mat):
        """Axis-aligned box: 6 faces x 2 triangles, outward facet normals."""
        self.quad((x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1), (0, 0, 1), mat)
        self.quad((x0, y0, z0), (x0, y1, z0), (x1, y1, z0), (x1, y0, z0), (0, 0, -1), mat)
        self.quad((x0, y0, z0), (x1, y0, z0), (x1, y0, z1), (x0, y0, z1), (0, -1, 0), mat)
        self.quad((x1, y1, z0), (x0, y1, z0), (x0, y1, z1), (x1, y1, z1), (0, 1, 0), mat)
        self.quad((x0, y1, z0), (x0, y0, z0), (x0, y0, z1), (x0, y1, z1), (-1, 0, 0), mat)
        self.quad((x1, y0, z0), (x1, y1, z0), (x1, y1, z1), (x1, y0, z1), (1, 0, 0), mat)

    def build(self, name, materials) -> Scene:
        tri = np.asarray(self.tris, dtype=np.float64).astype(np.float32)
        nrm = np.asarray(self.normals, dtype=np.float64).astype(np.float32)
        mat = np.asarray(self.mats, dtype=np.int32)
        return Scene(name, tri, nrm, mat, list(materials))


def _f32(x: float) -> float:
    return float(np.float32(x))


def _ground(mb: _MeshBuilder, half: float, mat: int):
    mb.quad((-half, -half, 0.0), (half, -half, 0.0), (half, half, 0.0), (-half, half, 0.0),
            (0, 0, 1), mat)


def _box_city(seed: int, half: float, n_boxes: int, foot: Tuple[float, float],
              height: Tuple[float, float], keep_clear: Sequence[Tuple[float, float]],
              box_mats: Sequence[int], pitch: float = 0.0, gap: float = 5.0):
    """Box footprints/heights.  pitch > 0 places one box per cell of a
    pitch x pitch lattice (streets between cells); pitch == 0 scatters boxes
    with rejection of overlaps.  Boxes never cover a point in keep_clear."""
    rng = PCG32(seed)
    boxes = []

    def covers(x0, y0, x1, y1, pts, margin=2.0):
        return any(x0 - margin <= px <= x1 + margin and y0 - margin <= py <= y1 + margin
                   for px, py in pts)

    if pitch > 0:
        n_side = int(round(2 * half / pitch))
        cells = [(i, j) for i in range(n_side) for j in range(n_side)]
        for (i, j) in cells[:n_boxes]:
            cx0 = -half + i * pitch
            cy0 = -half + j * pitch
            for _attempt in range(64):
                w = _f32(rng.uniform(*foot))
                d = _f32(rng.uniform(*foot))
                x0 = _f32(cx0 + gap + rng.uniform(0.0, max(pitch - 2 * gap - w, 0.0)))
                y0 = _f32(cy0 + gap + rng.uniform(0.0, max(pitch - 2 * gap - d, 0.0)))
                h = _f32(rng.uniform(*height))
                mat = box_mats[rng.randint(len(box_mats))]
                x1, y1 = _f32(x0 + w), _f32(y0 + d)
                if not covers(x0, y0, x1, y1, keep_clear):
                    boxes.append((x0, y0, x1, y1, h, mat))
                    break
    else:
        while len(boxes) < n_boxes:
            w = _f32(rng.uniform(*foot))
            d = _f32(rng.uniform(*foot))
            cx = rng.uniform(-half + 20.0, half - 20.0)
            cy = rng.uniform(-half + 20.0, half - 20.0)
            h = _f32(rng.uniform(*height))
            mat = box_mats[rng.randint(len(box_mats))]
            x0, y0 = _f32(cx - w / 2), _f32(cy - d / 2)
            x1, y1 = _f32(x0 + w), _f32(y0 + d)
            if covers(x0, y0, x1, y1, keep_clear):
                continue
            if any(not (x1 + 1 < b[0] or b[2] + 1 < x0 or y1 + 1 < b[1] or b[3] + 1 < y0)
                   for b in boxes):
                continue
            boxes.append((x0, y0, x1, y1, h, mat))
    return boxes


def small_scene(seed: int = 0x5B5) -> Workload:
    """Plain small workload: 200 m ground (eps_r=15, sigma=0.005) plus 10
    axis-aligned boxes (footprints U(10,30) m, heights U(10,40) m), one
    half-wave dipole Tx at (0,0,10), 2.4 GHz, level-6 icosahedron, 16 Rx on a
    4x4 grid at 1.5 m, 3 reflections, no transmission.  122 triangles."""
    f = 2.4e9
    tx = (0.0, 0.0, 10.0)
    g = [-75.0, -25.0, 25.0, 75.0]
    rx = np.array([(x, y, 1.5) for x in g for y in g], dtype=np.float64)
    clear = [(tx[0], tx[1])] + [(p[0], p[1]) for p in rx]
    mats = [(f, 0.0, 0.0, 15.0, 0.0, 0.005),
            (f, 0.0, 0.0, 5.31, 0.0, round(p2040_sigma(0.0326, 0.8095, f), 6))]
    mb = _MeshBuilder()
    _ground(mb, 100.0, 0)
    for (x0, y0, x1, y1, h, m) in _box_city(seed, 100.0, 10, (10.0, 30.0), (10.0, 40.0),
                                            clear, [1]):
        mb.box(x0, y0, x1, y1, 0.0, h, m)
    scene = mb.build("small", mats)
    req = Request(tx=tx, rx=rx, max_reflection=3, max_transmission=0, frequency=f,
                  tessellation=6, antenna=2)
    return Workload("small_L6_R3", scene, req, {"seed": seed})


def slab_walls(wl: Workload, widths: Sequence[float]) -> Workload:
    """The same workload with finite-thickness walls: material i gets
    thickness widths[i] (m) and the request switches to the slab
    coefficients (use_fresnel False, FieldCompute.cpp:255-262,284-291)."""
    mats = [tuple(m[:6]) + (float(w),) for m, w in zip(wl.scene.materials, widths)]
    wl.scene.materials = mats
    wl.request.use_fresnel = False
    wl.name = wl.name + "_slab"
    return wl


# A transmitter frame rotated 53.13 degrees about z and 67.38 degrees about x:
# the product of two rotations with Pythagorean-triple entries (3-4-5 and
# 5-12-13), each entry one correctly rounded division, so the matrix is the
# same bits on every machine.
ROTATED_TX_FRAME = (3 / 5, -4 / 13, 48 / 65,
                    4 / 5, 3 / 13, -36 / 65,
                    0.0, 12 / 13, 5 / 13)


def request_variant(name: str) -> Workload:
    """Request options the reference's main() never sets, on seeded scenes:
    the isotropic and half-wave patterns (FieldCompute.cpp:153-183), a
    rotated transmitter frame (txCoordSys), a transmit power other than 1 W
    and the Fresnel switch off (RTSolver.h:25-37).

    small_L5_R4T1_halfwave_rotated: small scene, level 5, 4 reflections and 1
      transmission, half-wave dipole in the rotated frame, 2.5 W at 3.5 GHz.
    urban_L5_R3T1_rx1600_halfwave_rotated: urban canyon at level 5 with
      receivers every 25 m, 3 reflections and 1 transmission, the same
      antenna, frame, power and frequency.
    urban_L5_R3T1_rx1600_isotropic_nofresnel: the same urban solve with the
      isotropic pattern at 0.1 W and 60 GHz and the slab coefficients of
      zero-width walls (the reference's useFresnelCoeff = false: reflection 0,
      transmission 1)."""
    if name == "small_L5_R4T1_halfwave_rotated":
        wl = small_scene()
        q = wl.request
        q.tessellation, q.max_reflection, q.max_transmission = 5, 4, 1
        q.antenna, q.tx_coord_sys, q.pt, q.frequency = 2, ROTATED_TX_FRAME, 2.5, 3.5e9
    elif name == "urban_L5_R3T1_rx1600_halfwave_rotated":
        wl = urban_scene(level=5, rx_pitch=25.0, max_reflection=3, max_transmission=1)
        q = wl.request
        q.antenna, q.tx_coord_sys, q.pt, q.frequency = 2, ROTATED_TX_FRAME, 2.5, 3.5e9
    elif name == "urban_L5_R3T1_rx1600_isotropic_nofresnel":
        wl = urban_scene(level=5, rx_pitch=25.0, max_reflection=3, max_transmission=1)
        q = wl.request
        q.antenna, q.pt, q.frequency, q.use_fresnel = 0, 0.1, 60e9, False
    else:
        raise KeyError(name)
    wl.name = name
    return wl


def urban_scene(seed: int = 0x5B5 + 1, level: int = 9, rx_pitch: float = 10.0,
                max_reflection: int = 6, max_transmission: int = 1) -> Workload:
    """Synthetic urban canyon: 1 km x 1 km ground plus 400 boxes on a 50 m
    lattice (streets >= 10 m), heights U(10,60) m, concrete (eps_r=5.31) or
    glass (eps_r=6.27) 50/50, isotropic Tx at 28 GHz at a street crossing,
    level-9 icosahedron (2,621,442 rays), 6 reflections + 1 transmission,
    10,000 Rx on a 10 m grid at 1.5 m.  4,802 triangles."""
    f = 28e9
    tx = (0.0, 0.0, 20.0)
    n = int(round(1000.0 / rx_pitch))
    coords = [-500.0 + rx_pitch / 2 + rx_pitch * i for i in range(n)]
    rx = np.array([(x, y, 1.5) for x in coords for y in coords], dtype=np.float64)
    concrete = (f, 0.0, 0.0, 5.31, 0.0, round(p2040_sigma(0.0326, 0.8095, f), 6))
    glass = (f, 0.0, 0.0, 6.27, 0.0, round(p2040_sigma(0.0043, 1.1925, f), 6))
    mats = [concrete, concrete, glass]  # 0 ground, 1 concrete walls, 2 glass
    mb = _MeshBuilder()
    _ground(mb, 500.0, 0)
    for (x0, y0, x1, y1, h, m) in _box_city(seed, 500.0, 400, (15.0, 35.0), (10.0, 60.0),
                                            [(tx[0], tx[1])], [1, 2], pitch=50.0):
        mb.box(x0, y0, x1, y1, 0.0, h, m)
    scene = mb.build("urban", mats)
    req = Request(tx=tx, rx=rx, max_reflection=max_reflection,
                  max_transmission=max_transmission, frequency=f, tessellation=level,
                  antenna=0)
    return Workload(f"urban_L{level}_R{max_reflection}T{max_transmission}", scene, req,
                    {"seed": seed, "rx_pitch": rx_pitch})


def reference_main_scene(stl_bytes: bytes | None = None) -> Workload:
    """The scene the reference's main() runs (SBRSolver_rev2.cpp:24-136):
    ground.stl (10 m x 1001 m strip), Tx (0,0,5), Rx line (0,0..2999,3),
    metal material, 1.8 GHz, 1 reflection, level 2, txCoordSys rows
    {0,1,0},{0,0,1},{1,0,0}, Hertzian pattern."""
    # ground.stl: two facets, normal +z (SBRSolver_rev2/data/stl_files/ground.stl)
    tri = np.array([[[-5, -1, 0], [5, -1, 0], [5, 1000, 0]],
                    [[-5, -1, 0], [5, 1000, 0], [-5, 1000, 0]]], dtype=np.float32)
    nrm = np.array([[0, 0, 1], [0, 0, 1]], dtype=np.float32)
    scene = Scene("reference_main", tri, nrm, np.zeros(2, np.int32),
                  [(1.8e9, 221.13, 0.05, 1.0, 0.0, 1e6)])
    rx = np.array([(0.0, float(i), 3.0) for i in range(3000)], dtype=np.float64)
    req = Request(tx=(0.0, 0.0, 5.0), rx=rx, max_reflection=1, max_transmission=0,
                  frequency=1.8e9, tessellation=2, tx_coord_sys=(0, 1, 0, 0, 0, 1, 1, 0, 0),
                  pt=1.0, use_fresnel=True, antenna=1)
    return Workload("reference_main", scene, req)


# ------------------------------------------------------------------ output

def write_stl(scene: Scene, path: str) -> None:
    """Binary STL: 80-byte header, uint32 count, 50-byte facets."""
    n = scene.n_tri
    rec = np.zeros(n, dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")]))
    rec["n"] = scene.normal
    rec["v"] = scene.tri
    with open(path, "wb") as fh:
        fh.write(b"sbr synthetic scene".ljust(80, b" "))
        fh.write(struct.pack("<I", n))
        fh.write(rec.tobytes())


def write_oracle_case(wl: Workload, directory: str, antenna: int | None = None) -> str:
    """Writes the STL, material ids, receivers and a case file in the format
    the reference harness reads; returns the case-file path."""
    os.makedirs(directory, exist_ok=True)
    sc, rq = wl.scene, wl.request
    stl = os.path.join(directory, "scene.stl")
    write_stl(sc, stl)
    tm = os.path.join(directory, "trimat.txt")
    np.savetxt(tm, sc.material_id, fmt="%d")
    rxp = os.path.join(directory, "rx.txt")
    with open(rxp, "w") as fh:
        fh.write(f"{len(rq.rx)}\n")
        for p in rq.rx:
            fh.write("%.17g %.17g %.17g\n" % tuple(p))
    case = os.path.join(directory, "case.txt")
    with open(case, "w") as fh:
        fh.write(f"stl {stl}\ntrimat {tm}\nrx {rxp}\nout {os.path.join(directory, 'out.txt')}\n")
        fh.write(f"materials {len(sc.materials)}\n")
        for m in sc.materials:
            fh.write(" ".join("%.17g" % v for v in m[:6]) + "\n")
        widths = [m[6] if len(m) > 6 else 0.0 for m in sc.materials]
        if any(w != 0.0 for w in widths):
            fh.write(f"widths {len(widths)} " + " ".join("%.17g" % w for w in widths) + "\n")
        fh.write("tx %.17g %.17g %.17g\n" % tuple(rq.tx))
        fh.write("txcs " + " ".join("%.17g" % v for v in rq.tx_coord_sys) + "\n")
        fh.write(f"refl {rq.max_reflection}\ntrans {rq.max_transmission}\n")
        fh.write(f"tess {rq.tessellation}\nantenna {rq.antenna if antenna is None else antenna}\n")
        fh.write("freq %.17g\npt %.17g\nfresnel %d\n" % (rq.frequency, rq.pt, int(rq.use_fresnel)))
    return case


def _diamond_square(n: int, rng: np.random.Generator, roughness: float = 0.55) -> np.ndarray:
    """(n+1) x (n+1) fractal height field (diamond-square, Fournier et al. 1982),
    n a power of two, values scaled to [-1, 1]."""
    h = np.zeros((n + 1, n + 1), np.float64)
    h[0, 0], h[0, n], h[n, 0], h[n, n] = rng.uniform(-1, 1, 4)
    step, amp = n, 1.0
    while step > 1:
        half = step // 2
        # diamond: centres of squares
        c = (h[0:-1:step, 0:-1:step] + h[step::step, 0:-1:step] + h[0:-1:step, step::step] +
             h[step::step, step::step]) / 4.0
        h[half::step, half::step] = c + rng.uniform(-amp, amp, c.shape)
        # square: edge midpoints (average of available neighbours)
        for (i0, j0) in ((0, half), (half, 0)):
            ii, jj = np.meshgrid(np.arange(i0, n + 1, step), np.arange(j0, n + 1, step), indexing="ij")
            acc = np.zeros(ii.shape)
            cnt = np.zeros(ii.shape)
            for di, dj in ((-half, 0), (half, 0), (0, -half), (0, half)):
                a, b = ii + di, jj + dj
                m = (a >= 0) & (a <= n) & (b >= 0) & (b <= n)
                acc[m] += h[a[m], b[m]]
                cnt[m] += 1
            h[ii, jj] = acc / cnt + rng.uniform(-amp, amp, ii.shape)
        step, amp = half, amp * roughness
    h -= h.min()
    h /= max(h.max(), 1e-12)
    return 2.0 * h - 1.0


def large_scene(seed: int = 0x5B5 + 3, level: int = 10, n_rx: int = 50000,
                max_reflection: int = 8, cells: int = 512, spacing: float = 2.0,
                n_poly: int = 2000) -> Workload:
    """Large scene for the precision study: a cells x cells fractal terrain
    (diamond-square, +/-20 m relief, `spacing` m grid: 2*cells^2 triangles)
    plus n_poly extruded convex polygons (4-12 sides, circumradius U(5,15) m,
    heights lognormal(mu=3, sigma=0.5) m) standing on it; half-wave Tx at
    3.5 GHz 30 m above the centre, level-10 icosahedron (10,485,762 rays),
    8 reflections, n_rx receivers 1.5 m above the terrain at seeded
    positions.  With the defaults: 524,288 + the polygons' triangles."""
    rng = np.random.default_rng(seed)
    f = 3.5e9
    H = 20.0 * _diamond_square(cells, rng)
    half = cells * spacing / 2.0
    xs = -half + spacing * np.arange(cells + 1)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    V = np.stack([X, Y, H], -1).astype(np.float32)

    def height(x, y):
        gx = np.clip((x + half) / spacing, 0, cells - 1e-6)
        gy = np.clip((y + half) / spacing, 0, cells - 1e-6)
        i, j = np.floor(gx).astype(int), np.floor(gy).astype(int)
        fx, fy = gx - i, gy - j
        return ((1 - fx) * (1 - fy) * H[i, j] + fx * (1 - fy) * H[i + 1, j] +
                (1 - fx) * fy * H[i, j + 1] + fx * fy * H[i + 1, j + 1])

    # terrain: two triangles per cell, normals from the float vertices
    a = V[:-1, :-1].reshape(-1, 3)
    b = V[1:, :-1].reshape(-1, 3)
    c = V[1:, 1:].reshape(-1, 3)
    d = V[:-1, 1:].reshape(-1, 3)
    t1 = np.stack([a, b, c], 1)
    t2 = np.stack([a, c, d], 1)
    tri = np.concatenate([t1, t2], 0).astype(np.float32)

    def normals(t):
        t = t.astype(np.float64)
        nrm = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
        nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)
        return nrm.astype(np.float32)

    tris, nrms, mats = [tri], [normals(tri)], [np.zeros(len(tri), np.int32)]
    tx = (0.0, 0.0, float(height(np.array(0.0), np.array(0.0))) + 30.0)
    mb = _MeshBuilder()
    for _ in range(n_poly):
        while True:
            cx, cy = rng.uniform(-half + 20, half - 20, 2)
            if (cx - tx[0]) ** 2 + (cy - tx[1]) ** 2 > 30.0 ** 2:
                break
        k = int(rng.integers(4, 13))
        r = rng.uniform(5.0, 15.0)
        ang = np.sort(rng.uniform(0, 2 * np.pi, k))
        px, py = cx + r * np.cos(ang), cy + r * np.sin(ang)
        hgt = float(np.exp(rng.normal(3.0, 0.5)))
        z0 = float(min(height(px, py).min(), height(np.array(cx), np.array(cy)))) - 0.5
        z1 = z0 + hgt
        P = [(float(np.float32(x)), float(np.float32(y))) for x, y in zip(px, py)]
        z0, z1 = float(np.float32(z0)), float(np.float32(z1))
        mat = 1 + int(rng.integers(0, 2))
        for i in range(k):
            (x0, y0), (x1, y1) = P[i], P[(i + 1) % k]
            nx, ny = (y1 - y0), -(x1 - x0)
            ln = max((nx * nx + ny * ny) ** 0.5, 1e-12)
            mb.quad((x0, y0, z0), (x1, y1, z0), (x1, y1, z1), (x0, y0, z1), (nx / ln, ny / ln, 0.0), mat)
        for i in range(1, k - 1):  # fans: top (+z) and bottom (-z)
            mb.tri((P[0][0], P[0][1], z1), (P[i][0], P[i][1], z1), (P[i + 1][0], P[i + 1][1], z1), (0, 0, 1), mat)
            mb.tri((P[0][0], P[0][1], z0), (P[i + 1][0], P[i + 1][1], z0), (P[i][0], P[i][1], z0), (0, 0, -1), mat)
    if mb.tris:
        tris.append(np.asarray(mb.tris, np.float64).astype(np.float32))
        nrms.append(np.asarray(mb.normals, np.float64).astype(np.float32))
        mats.append(np.asarray(mb.mats, np.int32))
    tri = np.concatenate(tris, 0)
    nrm = np.concatenate(nrms, 0)
    mat = np.concatenate(mats, 0)
    # drop facets whose float corners coincide (degenerate); keep the rest in order
    e1 = tri[:, 1].astype(np.float64) - tri[:, 0]
    e2 = tri[:, 2].astype(np.float64) - tri[:, 0]
    good = (np.linalg.norm(np.cross(e1, e2), axis=1) > 0) & \
        ~np.all(tri[:, 0] == tri[:, 1], 1) & ~np.all(tri[:, 0] == tri[:, 2], 1) & \
        ~np.all(tri[:, 1] == tri[:, 2], 1)
    tri, nrm, mat = tri[good], nrm[good], mat[good]
    ground = (f, 0.0, 0.0, 15.0, 0.0, 0.035)  # medium-dry ground
    concrete = (f, 0.0, 0.0, 5.31, 0.0, round(p2040_sigma(0.0326, 0.8095, f), 6))
    glass = (f, 0.0, 0.0, 6.27, 0.0, round(p2040_sigma(0.0043, 1.1925, f), 6))
    scene = Scene("large", tri, nrm, mat, [ground, concrete, glass])
    rx_xy = rng.uniform(-half + 1.0, half - 1.0, (n_rx, 2))
    rx = np.column_stack([rx_xy, height(rx_xy[:, 0], rx_xy[:, 1]) + 1.5]).astype(np.float64)
    req = Request(tx=tx, rx=rx, max_reflection=max_reflection, max_transmission=0,
                  frequency=f, tessellation=level, antenna=2)
    return Workload(f"large_L{level}_R{max_reflection}", scene, req, {"seed": seed})


def batched_workload(seed: int = 0x5B5 + 2, n_tx: int = 256):
    """Many transmitters on the urban canyon: n_tx seeded street-crossing
    positions 10-40 m high, icosahedron levels U{6..9}, patterns U{isotropic,
    Hertzian, half-wave}, 5 reflections, no transmission, 28 GHz, and 4,096
    receivers shared by every request on a 64 x 64 grid at 1.5 m.  Returns
    the workload (its request is the urban canyon's own) and the requests."""
    wl = urban_scene()
    rng = np.random.default_rng(seed)
    g = -500.0 + (1000.0 / 64) * (np.arange(64) + 0.5)
    rx = np.array([(x, y, 1.5) for x in g for y in g], np.float64)
    reqs = []
    for _ in range(n_tx):
        tx = (float(rng.integers(-10, 10) * 50.0), float(rng.integers(-10, 10) * 50.0),
              float(rng.uniform(10, 40)))
        reqs.append(Request(tx=tx, rx=rx, max_reflection=5, max_transmission=0,
                            frequency=28e9, tessellation=int(rng.integers(6, 10)),
                            antenna=int(rng.integers(0, 3))))
    return wl, reqs
