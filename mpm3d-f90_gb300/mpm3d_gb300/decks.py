"""Writers of .mpm decks for the benchmark workloads and the parity cases.

Every deck is plain reference syntax (DataIn.f90 keyword table), so the
reference itself could read it. Numbers are written as float32-representable
decimals ('%.9g' of a float32), because the reference reads every real as a
32-bit REAL (FFI.f90:110); the deck therefore states exactly the values both
sides compute with. Random inputs use numpy's PCG64 generator with a fixed
seed.

Workloads (sizes as in the benchmark configurations):
  taylor_bar   -- copper cylinder R 3.2 mm, L 32.4 mm, 0.4 mm spacing, 8 ppc,
                  190 m/s onto a rigid wall; Johnson-Cook with failure ('jcf',
                  type 7) + linear EOS; USF, linear shape functions.
  soil_slope   -- 20 m high 45 degree slope, 0.1 m spacing jittered +-1%,
                  Drucker-Prager (c 10 kPa, phi 20 deg), gravity; GIMP, USF.
  dam_break    -- 4 x 2 x 2 m water column in a 10 x 2 x 4 m tank, 1 cm
                  spacing; null material + weakly compressible EOS; B-spline,
                  MUSL.
  soft_beam    -- neo-Hookean cantilever; SGMP, MUSL (serving scenes).
  cook_membrane-- the tapered Cook panel under a distributed tip shear.
"""
from __future__ import annotations

import math
from typing import Iterable, Optional

import numpy as np


def f32s(x: float) -> str:
    """Decimal that reads back to the same float32 (tokens stay <= 20 chars)."""
    return "%.9g" % float(np.float32(x))


def _points_block(ids_start: int, mat: int, mass: np.ndarray, xyz: np.ndarray) -> str:
    n = xyz.shape[0]
    m = np.asarray(mass, dtype=np.float32)
    p = xyz.astype(np.float32)
    if m.ndim == 0:
        m = np.full(n, m, dtype=np.float32)
    lines = ["%d %d %.9g %.9g %.9g %.9g" % (ids_start + i, mat, m[i], p[i, 0], p[i, 1], p[i, 2])
             for i in range(n)]
    return "\n".join(lines)


class DeckWriter:
    """Accumulates the sections of a deck in the reference's keyword order."""

    def __init__(self, title: str):
        self.title = title
        self.head: list[str] = []
        self.bodies: list[str] = []
        self.tail: list[str] = []
        self.nbmp = 0
        self.nbbo = 0
        self.nbco = 1

    def kw(self, line: str) -> None:
        self.head.append(line)

    def points(self, mat: int, mass, xyz: np.ndarray, com: int = 1) -> tuple[int, int]:
        n = xyz.shape[0]
        first = self.nbmp + 1
        self.bodies.append(f"part poin {com} {n}\n" + _points_block(first, mat, np.asarray(mass), xyz))
        self.nbmp += n
        self.nbbo += 1
        return first, first + n - 1

    def block(self, mat: int, density: float, dp: float, origin, counts, com: int = 1) -> tuple[int, int]:
        nx, ny, nz = counts
        first = self.nbmp + 1
        self.bodies.append(
            f"part bloc {com} {mat} {f32s(density)} {f32s(dp)} {f32s(origin[0])} {f32s(origin[1])} "
            f"{f32s(origin[2])} {nx} {ny} {nz}")
        self.nbmp += nx * ny * nz
        self.nbbo += 1
        return first, first + nx * ny * nz - 1

    def text(self) -> str:
        out = [f"mpm3d *** {self.title}", f"nbco {self.nbco}", f"nbbo {self.nbbo}", f"nbmp {self.nbmp}"]
        out += self.head
        out += self.bodies
        out += self.tail
        out.append("endi")
        return "\n".join(out) + "\n"


def _grid_lines(span, dcell) -> list[str]:
    return [f"spx {f32s(span[0][0])} {f32s(span[0][1])}",
            f"spy {f32s(span[1][0])} {f32s(span[1][1])}",
            f"spz {f32s(span[2][0])} {f32s(span[2][1])}",
            f"dcel {f32s(dcell)}"]


def taylor_bar(dp: float = 4e-4, radius: float = 3.2e-3, length: float = 32.4e-3,
               velocity: float = -190.0, dtscale: float = 0.1, epf: float = 100.0) -> str:
    """Copper Taylor bar (8 particles per cell: cell = 2 dp)."""
    h = 2 * dp
    n = int(math.ceil(radius / dp))
    ij = np.arange(-n, n)
    cx = (ij + 0.5) * dp
    X, Y = np.meshgrid(cx, cx, indexing="xy")
    inside = X ** 2 + Y ** 2 < radius ** 2
    xs, ys = X[inside], Y[inside]
    nl = int(round(length / dp))
    pts = []
    for k in range(nl):
        z = (k + 0.5) * dp
        pts.append(np.stack([xs, ys, np.full(xs.shape, z)], axis=1))
    xyz = np.concatenate(pts, axis=0)
    rho, E, nu = 8930.0, 1.17e11, 0.35
    K = E / (3 * (1 - 2 * nu))
    half = 16 * h
    w = DeckWriter("taylor bar, Johnson-Cook + linear EOS, USF")
    w.kw("nmat 1")
    w.head += _grid_lines(((-half, half), (-half, half), (0.0, 42 * h)), h)
    w.kw(f"dtsc {f32s(dtscale)}")
    w.kw("endt 1.0")
    w.kw("usf on")
    w.kw("fixe 0 0 0 0 1 0")
    w.kw("mate")
    # num jcf density E nu A B n C m roomt melt specheat epso epf
    w.kw(f"1 jcf {f32s(rho)} {f32s(E)} {f32s(nu)} 9e7 2.92e8 0.31 0.025 1.09 293 1356 383 1 {f32s(epf)}")
    w.kw(f"seos 1 1 0 {f32s(K)} 0 0 0 0 0 0")
    w.points(1, rho * dp ** 3, xyz)
    w.tail += ["velo", f"body 1 0 0 {f32s(velocity)}", "endv"]
    return w.text()


def dp_parameters(cohesion: float, phi_deg: float) -> tuple[float, float, float, float]:
    """Drucker-Prager (q_phi, k_phi, q_psi, tension) matched to Mohr-Coulomb in
    plane strain: q = 3 tan(phi)/sqrt(9 + 12 tan^2 phi), k = 3c/sqrt(...),
    associated dilatancy off (q_psi = 0), tension cut-off at the cone apex k/q."""
    t = math.tan(math.radians(phi_deg))
    r = math.sqrt(9 + 12 * t * t)
    q = 3 * t / r
    k = 3 * cohesion / r
    tens = k / q if q > 0 else 0.0
    return q, k, 0.0, tens


def soil_slope(dp: float = 0.1, width: float = 3.0, height: float = 20.0, crest: float = 10.0,
               jitter: float = 0.01, seed: int = 0x5EED, dtscale: float = 0.3,
               cohesion: float = 1e4, phi: float = 20.0) -> str:
    """45 degree slope on a rigid base, GIMP (cell = 2 dp), gravity along -z."""
    h = 2 * dp
    nx = int(round((crest + height) / dp))
    nz = int(round(height / dp))
    ny = int(round(width / dp))
    xi = (np.arange(nx) + 0.5) * dp
    zk = (np.arange(nz) + 0.5) * dp
    X, Z = np.meshgrid(xi, zk, indexing="xy")
    top = np.where(X <= crest, height, height - (X - crest))
    keep = Z < top
    xs, zs = X[keep], Z[keep]
    pts = []
    for j in range(ny):
        y = (j + 0.5) * dp
        pts.append(np.stack([xs, np.full(xs.shape, y), zs], axis=1))
    xyz = np.concatenate(pts, axis=0)
    rng = np.random.default_rng(seed)
    xyz = xyz + rng.uniform(-jitter * dp, jitter * dp, size=xyz.shape)
    rho, E, nu = 2000.0, 5e7, 0.3
    q, k, qpsi, tens = dp_parameters(cohesion, phi)
    w = DeckWriter("soil slope, Drucker-Prager, GIMP, USF")
    w.kw("nmat 1")
    lx = crest + height + 0.3 * height
    w.head += _grid_lines(((0.0, lx), (0.0, width), (0.0, height + 0.2 * height)), h)
    w.kw(f"dtsc {f32s(dtscale)}")
    w.kw("endt 100.0")
    w.kw("usf on")
    w.kw("gimp")
    w.kw("fixe 2 0 2 2 1 0")
    w.kw("mate")
    w.kw(f"1 dpm {f32s(rho)} {f32s(E)} {f32s(nu)} {f32s(q)} {f32s(k)} {f32s(qpsi)} {f32s(tens)}")
    w.points(1, rho * dp ** 3, xyz)
    w.tail += ["load", "grav 1 0 0 -9.81", "endl"]
    return w.text()


def dam_break(dp: float = 0.01, h: float = 0.02, water=(4.0, 2.0, 2.0), tank=(10.0, 2.0, 4.0),
              dtscale: float = 0.5, bulk: float = 2.2e6, viscosity: float = 1e-3) -> str:
    """Water column in a tank with slip walls; quadratic B-spline, MUSL. The
    grid has one extra cell outside each wall so that the wall is the second,
    fixed node layer."""
    rho = 1000.0
    nx, ny, nz = (int(round(water[i] / dp)) for i in range(3))
    w = DeckWriter("dam break, null material + weakly compressible EOS, B-spline, MUSL")
    w.kw("nmat 1")
    w.head += _grid_lines(((-h, tank[0] + h), (-h, tank[1] + h), (-h, tank[2] + h)), h)
    w.kw(f"dtsc {f32s(dtscale)}")
    w.kw("endt 100.0")
    w.kw("musl on")
    w.kw("bimp")
    w.kw("bulk 1.5 0.06")
    w.kw("fixe 2 2 2 2 2 0")
    w.kw("mate")
    w.kw(f"1 null {f32s(rho)} {f32s(bulk)} {f32s(viscosity)}")
    w.kw(f"seos 1 4 {f32s(math.sqrt(bulk / rho))}")
    w.block(1, rho, dp, (0.0, 0.0, 0.0), (nx, ny, nz))
    w.tail += ["load", "grav 1 0 0 -9.81", "endl"]
    return w.text()


def soft_beam(dp: float = 0.25, length: float = 6.0, depth: float = 1.0, thick: float = 1.0,
              young: float = 1e7, nu: float = 0.3, rho: float = 1000.0, dtscale: float = 0.5,
              shape: str = "sgmp", scheme: str = "musl", gravity: float = -9.81, tlmpm: bool = False) -> str:
    """Cantilever soft beam clamped at x = 0 (neo-Hookean). With SGMP the grid
    has one extra layer beyond the clamped face (the reference's rule for
    fixed boundaries under SGMP). tlmpm: the total Lagrangian form ('TLmp',
    with the deformation gradient tracked, 'UVFp')."""
    h = 2 * dp
    nx, ny, nz = int(round(length / dp)), int(round(thick / dp)), int(round(depth / dp))
    w = DeckWriter(f"soft beam, neo-Hookean, {shape}, {scheme}")
    w.kw("nmat 1")
    pad = h if shape == "sgmp" else 0.0
    z0 = 2.0
    w.head += _grid_lines(((-pad, length + 2.0), (0.0, thick), (0.0, z0 + depth + 1.0)), h)
    w.kw(f"dtsc {f32s(dtscale)}")
    w.kw("endt 100.0")
    w.kw(f"{scheme} on")
    if shape in ("sgmp", "gimp", "bimp"):
        w.kw(shape)
    if tlmpm:
        w.kw("TLmp")
        w.kw("UVFp")
    w.kw("fixe 1 0 2 2 0 0")
    w.kw("mate")
    w.kw(f"1 neoh {f32s(rho)} {f32s(young)} {f32s(nu)}")
    w.block(1, rho, dp, (0.0, 0.0, z0), (nx, ny, nz))
    w.tail += ["load", f"grav 1 0 0 {f32s(gravity)}", "endl"]
    return w.text()


def generic_block(material_line: str, eos_line: Optional[str] = None, *, dp: float = 0.5,
                  counts=(8, 4, 6), shape: Optional[str] = None, scheme: str = "usf",
                  velocity=(0.0, 0.0, -5.0), gravity: Optional[float] = -9.81, dtscale: float = 0.5,
                  fixed: str = "0 0 0 0 1 0", rho: float = 1000.0, extra: Iterable[str] = ()) -> str:
    """Small block test case for any material line ('1 elas 1000 1e7 0.3')."""
    h = 2 * dp
    w = DeckWriter("block parity case")
    w.kw("nmat 1")
    pad = 2 * h
    lx, ly, lz = (counts[i] * dp for i in range(3))
    w.head += _grid_lines(((-pad, lx + pad), (-pad, ly + pad), (0.0, lz + 3 * pad)), h)
    w.kw(f"dtsc {f32s(dtscale)}")
    w.kw("endt 100.0")
    w.kw(f"{scheme} on")
    if shape:
        w.kw(shape)
    w.kw(f"fixe {fixed}")
    for e in extra:
        w.kw(e)
    w.kw("mate")
    w.kw(material_line)
    if eos_line:
        w.kw(eos_line)
    w.block(1, rho, dp, (0.0, 0.0, h), counts)
    w.tail += ["velo", "body 1 %s %s %s" % tuple(f32s(v) for v in velocity), "endv"]
    if gravity is not None:
        w.tail += ["load", f"grav 1 0 0 {f32s(gravity)}", "endl"]
    return w.text()


def contact_blocks(shape: Optional[str] = None, scheme: str = "usf", fricfa: float = 0.0, normbody: int = 0,
                   dp: float = 0.25, speed: float = 4.0, counts=(6, 4, 4), gap_cells: float = 1.0) -> str:
    """Two elastic blocks on separate grid components driven into each other
    along x (block 1 at +speed, block 2 at -speed, a gap of `gap_cells` cells),
    with Bardenhagen's contact ('cont lagr fricfa normbody'); block 2 also
    slides in y so that friction acts. Cell = 2 dp (8 particles per cell)."""
    h = 2 * dp
    w = DeckWriter(f"contact of two blocks, {shape or 'linear'}, {scheme}")
    w.nbco = 2
    w.kw("nmat 1")
    lx, ly, lz = (counts[i] * dp for i in range(3))
    x2 = lx + gap_cells * h
    w.head += _grid_lines(((-2 * h, x2 + lx + 2 * h), (-2 * h, ly + 2 * h), (-2 * h, lz + 2 * h)), h)
    w.kw("dtsc 0.4")
    w.kw("endt 100.0")
    w.kw(f"{scheme} on")
    if shape:
        w.kw(shape)
    w.kw(f"cont lagr {f32s(fricfa)} {normbody}")
    w.kw("fixe 0 0 0 0 0 0")
    w.kw("mate")
    w.kw("1 elas 1000 1e6 0.3")
    w.block(1, 1000.0, dp, (0.0, 0.0, 0.0), counts, com=1)
    w.block(1, 1000.0, dp, (x2, 0.0, 0.0), counts, com=2)
    w.tail += ["velo", f"body 1 {f32s(speed)} 0 0", f"body 2 {f32s(-speed)} {f32s(speed * 0.5)} 0", "endv"]
    return w.text()


# Grid and run settings of the two published Cook-membrane resolutions
# (VolumetricLockingEx/Cook_membrane/*5776p and *23072p): cell size, spans per
# variant, time-step scale, damping factor and the number formats of the
# particle mass and the edge loads. Other spacings use the 5776 settings.
_COOK_LAYOUT = {
    0.5: dict(dcell=1.0, dtscale="0.9", damp="0.3", mass_fmt="%.6f", load_fmt="%.6f",
              spans={"mpm": ((0, 50), (0, 62), (-0.5, 0.5)), "gimp": ((-1, 50), (-1, 62), (-1, 1)),
                     "bimp": ((-1, 50), (-1, 62), (-1, 1)), "sgmp": ((-1, 50), (-1, 62), (-0.5, 0.5))}),
    0.25: dict(dcell=0.5, dtscale="0.8", damp="0.2", mass_fmt="%.6g", load_fmt="%.5g",
               spans={"mpm": ((0, 48.5), (0, 61), (-0.25, 0.25)), "gimp": ((-0.5, 48.5), (-0.5, 61), (-0.5, 0.5)),
                      "bimp": ((-0.5, 48.5), (-0.5, 61), (-0.5, 0.5)),
                      "sgmp": ((-0.5, 48.5), (-0.5, 61), (-0.25, 0.25))}),
}


def cook_membrane(variant: str = "mpm", spacing: float = 0.5, young: float = 70.0, nu: float = 0.499,
                  rho: float = 1.0, total_load: float = 1.0, extra: Iterable[str] = ()) -> str:
    """Cook's tapered panel (corners (0,0), (48,44), (48,60), (0,44), unit
    thickness, plane strain through roller z faces), clamped at x = 0 and
    loaded by a vertical shear on the x = 48 edge, run quasi-statically (load
    ramp 'QuLo 15', mass damping 'Damp'); neo-Hookean, MUSL.

    variant: 'mpm' (linear), 'gimp', 'bimp' (B-spline) or 'sgmp'. Particles
    sit on a regular lattice clipped to the panel, rows by increasing y
    (mass = area/n; the edge particles carry 1/(m-1) of the load, the two
    corner particles half of that). Spacing 0.5 and 0.25 give the two
    published resolutions (5776 and 23072 particles: cell 1 and 0.5, their
    spans, time-step scale, damping factor and number formats); extra:
    further keyword lines (output settings)."""
    ds = spacing
    xs = (np.arange(int(round(48 / ds))) + 0.5) * ds
    ys = (np.arange(int(round(60 / ds))) + 0.5) * ds
    pts = []
    for y in ys:
        for x in xs:
            if y >= 44.0 / 48.0 * x and y <= 44.0 + 16.0 / 48.0 * x:
                pts.append((x, y, 0.0))
    xyz = np.array(pts)
    n = xyz.shape[0]
    area = 48.0 * (44.0 + 16.0) / 2.0
    lay = _COOK_LAYOUT.get(spacing, _COOK_LAYOUT[0.5])
    mass = lay["mass_fmt"] % (rho * area / n)
    w = DeckWriter(f"Cook membrane, neo-Hookean, {variant}")
    w.kw("nmat 1")
    w.head += _grid_lines(lay["spans"][variant], lay["dcell"])
    w.kw("fixe 1 0 0 0 2 2")
    w.kw(f"dtsc {lay['dtscale']}")
    w.kw("endt 30")
    w.kw("musl on")
    if variant != "mpm":
        w.kw(variant)
    w.kw("smoo")
    w.kw("QuLo 15")
    w.kw(f"Damp {lay['damp']}")
    for e in extra:
        w.kw(e)
    w.kw(f"curv disy {n}")
    w.kw("mate")
    w.kw(f"1 neoh {f32s(rho)} {f32s(young)} {f32s(nu)}")
    first = w.nbmp + 1
    lines = ["%d 1 %s %.9g %.9g %.9g" % (first + i, mass, xyz[i, 0], xyz[i, 1], xyz[i, 2]) for i in range(n)]
    w.bodies.append(f"part poin 1 {n}\n" + "\n".join(lines))
    w.nbmp += n
    w.nbbo += 1
    right = np.where(np.isclose(xyz[:, 0], xs[-1]))[0]
    per = total_load / max(1, len(right) - 1)
    loads = ["load"]
    for k, i in enumerate(right):
        f = per * (0.5 if k in (0, len(right) - 1) else 1.0)
        loads.append(("part %d 0 " + lay["load_fmt"] + " 0") % (i + 1, f))
    loads.append("endl")
    w.tail += loads
    return w.text()


# Published tip vertical displacement (m) of the Cook membrane with 5776
# particles (VolumetricLockingEx/ExamplesResults.pdf, Table 1), by variant.
COOK_TIP_PUBLISHED = {"mpm": 0.2489, "gimp": 0.2512, "bimp": 0.2620, "sgmp": 0.2678}
# The same with 23072 particles (spacing 0.25, cell 0.5; same table).
COOK_TIP_PUBLISHED_23072 = {"mpm": 0.2692, "gimp": 0.2688, "bimp": 0.2711, "sgmp": 0.2739}


def _fast_points(ids_start: int, mat: int, mass: float, xyz: np.ndarray) -> str:
    """'part poin' body lines for large point sets (vectorised formatting)."""
    n = xyz.shape[0]
    p = xyz.astype(np.float32).astype(np.float64)
    ids = np.arange(ids_start, ids_start + n)
    m = float(np.float32(mass))
    cols = [ids.astype(str), np.full(n, str(mat)), np.full(n, "%.9g" % m)]
    cols += [np.char.mod("%.9g", p[:, k]) for k in range(3)]
    out = cols[0]
    for c in cols[1:]:
        out = np.char.add(np.char.add(out, " "), c)
    return "\n".join(out.tolist())


def serving_scene(rng: np.random.Generator, np_min: int = 2000, np_max: int = 400000,
                  kind: Optional[str] = None) -> tuple[str, int, str]:
    """One scene of the serving workload: a Cook membrane panel (extruded two
    particles thick, plane strain through roller z faces) or a cantilever soft
    beam, each with probability 1/2; particle count log-uniform in
    [np_min, np_max]; cell size h = 2 x spacing (8 particles per cell);
    neo-Hookean with E log-uniform in [1, 100] MPa, nu uniform in [0.3, 0.49],
    rho 1000; SGMP with one extra grid layer beyond the clamped and roller
    faces; MUSL. Returns (deck text, particle count, kind)."""
    if kind is None:
        kind = "cook" if rng.random() < 0.5 else "beam"
    target = math.exp(rng.uniform(math.log(np_min), math.log(np_max)))
    young = math.exp(rng.uniform(math.log(1e6), math.log(1e8)))
    nu = rng.uniform(0.3, 0.49)
    rho = 1000.0
    if kind == "beam":
        # 6 x 1 x 1 m beam clamped at x = 0
        dp = (6.0 / target) ** (1.0 / 3.0)
        nx, ny, nz = max(2, int(round(6.0 / dp))), max(2, int(round(1.0 / dp))), max(2, int(round(1.0 / dp)))
        h = 2 * dp
        w = DeckWriter("serving scene: soft beam, neo-Hookean, sgmp, musl")
        w.kw("nmat 1")
        lx, ly, lz = nx * dp, ny * dp, nz * dp
        # the beam hangs 2 m above the grid floor: the free end of the
        # softest beams falls about a metre in the 500 steps of a scene, and
        # must stay inside the grid; SGMP wants one cell of grid beyond the
        # clamped face and beyond the roller faces
        z0 = 2.0
        w.head += _grid_lines(((-h, lx + 2 * h), (-h, ly + h), (0.0, z0 + lz + 2 * h)), h)
        w.kw("dtsc 0.5")
        w.kw("endt 100.0")
        w.kw("musl on")
        w.kw("sgmp")
        w.kw("fixe 1 0 2 2 0 0")
        w.kw("mate")
        w.kw(f"1 neoh {f32s(rho)} {f32s(young)} {f32s(nu)}")
        w.block(1, rho, dp, (0.0, 0.0, z0), (nx, ny, nz))
        w.tail += ["load", f"grav 1 0 0 {f32s(-9.81)}", "endl"]
        return w.text(), nx * ny * nz, kind
    # Cook panel (48 x 44..60 m), two particles through the thickness
    area = 48.0 * (44.0 + 16.0) / 2.0
    dp = math.sqrt(2.0 * area / target)
    xs = (np.arange(int(round(48 / dp))) + 0.5) * dp
    ys = (np.arange(int(round(60 / dp))) + 0.5) * dp
    X, Y = np.meshgrid(xs, ys)
    X, Y = X.ravel(), Y.ravel()
    keep = (Y >= 44.0 / 48.0 * X) & (Y <= 44.0 + 16.0 / 48.0 * X)
    X, Y = X[keep], Y[keep]
    h = 2 * dp
    zs = np.array([0.5, 1.5]) * dp
    xyz = np.concatenate([np.stack([X, Y, np.full_like(X, z)], axis=1) for z in zs])
    n = xyz.shape[0]
    mass = rho * area * (2 * dp) / n
    w = DeckWriter("serving scene: Cook membrane, neo-Hookean, sgmp, musl")
    w.kw("nmat 1")
    w.head += _grid_lines(((-h, 48.0 + 2 * h), (-2 * h, 62.0 + 2 * h), (-h, 2 * dp + h)), h)
    w.kw("fixe 1 0 0 0 2 2")
    w.kw("dtsc 0.9")
    w.kw("endt 30")
    w.kw("musl on")
    w.kw("sgmp")
    w.kw("QuLo 15")
    w.kw("Damp 0.3")
    w.kw("mate")
    w.kw(f"1 neoh {f32s(rho)} {f32s(young)} {f32s(nu)}")
    first = w.nbmp + 1
    w.bodies.append(f"part poin 1 {n}\n" + _fast_points(first, 1, mass, xyz))
    w.nbmp += n
    w.nbbo += 1
    right = np.where(np.isclose(xyz[:, 0], xs[-1]))[0]
    total = young * 1e-3 * 16.0 * (2 * dp)  # shear traction 1e-3 E on the loaded edge
    per = total / max(1, len(right))
    loads = ["load"] + ["part %d 0 %s 0" % (i + 1, f32s(per)) for i in right] + ["endl"]
    w.tail += loads
    return w.text(), n, kind


def granular_column(scale: float = 1.0, radius: float = 0.5, height: float = 1.0, dtscale: float = 0.5,
                    rho: float = 2650.0, young: float = 1e7, nu: float = 0.3, phi: float = 30.0,
                    cohesion: float = 0.0) -> tuple[str, int]:
    """Granular column collapse: a cylinder (radius 0.5 m, height 1 m) of
    Drucker-Prager sand (phi 30 deg, c 0) on a rough floor, GIMP, MUSL,
    gravity. At scale 1 the particle spacing is 2.307 mm (about 64 M
    particles; 5.2 particles per cell) on a 512 x 512 x 256 grid of 4 mm cells;
    `scale` multiplies spacing and cell size. The cylinder is a stack of
    one-layer discs (the 'cicl' generator, DataIn.f90:792-838), one body per
    layer, so the deck stays a few kB at any particle count. Returns (deck
    text, particle count)."""
    dp = float(np.float32(2.307e-3 * scale))
    h = 4e-3 * scale
    nr = int(round(radius / dp))
    nl = int(round(height / dp))
    # particles per layer, with the reader's arithmetic (DataIn.f90:810-817)
    ix = np.arange(1 - nr, nr + 1, dtype=np.float64)
    t = (ix - 1) * dp + 0.0 + 0.5 * dp
    A, B = np.meshgrid(t, t)
    r2 = float(nr) * dp
    per_layer = int(np.count_nonzero(A * A + B * B < r2 * r2))
    n = per_layer * nl
    half = 1.024  # 2.048 x 2.048 x 1.024 m domain (512 x 512 x 256 cells of 4 mm at scale 1)
    q, k, qpsi, tens = dp_parameters(cohesion, phi)
    w = DeckWriter("granular column collapse, Drucker-Prager, GIMP, MUSL")
    w.nbmp = n
    w.nbbo = nl
    w.kw("nmat 1")
    w.head += _grid_lines(((-half, half), (-half, half), (0.0, half)), h)
    w.kw(f"dtsc {f32s(dtscale)}")
    w.kw("endt 100.0")
    w.kw("musl on")
    w.kw("gimp")
    w.kw("fixe 0 0 0 0 1 0")
    w.kw("mate")
    w.kw(f"1 dpm {f32s(rho)} {f32s(young)} {f32s(nu)} {f32s(q)} {f32s(k)} {f32s(qpsi)} {f32s(tens)}")
    for layer in range(nl):
        w.bodies.append(f"part cicl 1 1 {f32s(rho)} {f32s(dp)} 0 0 {f32s(layer * dp)} {nr}")
    w.tail += ["load"] + [f"grav {b + 1} 0 0 -9.81" for b in range(nl)] + ["endl"]
    return w.text(), n
