"""The reference's example decks, regenerated for the parity tests.

The GPU machine carries no copy of the reference tree, so each example deck of
MPM3D-F90 that the parity tests run (Data/*.mpm and
VolumetricLockingEx/**/*.mpm) is written here again by this project's deck
writer from its parameters: the same keywords, materials, equations of state,
boundary codes, loads, velocities, output requests and particle sets. Where
the reference tree is present, tests/test_reference_decks.py checks that each
regenerated deck parses into exactly the reference deck's data (every field of
the parsed record, bit for bit). Two particle sets are not generated by a
rule: the Cook membranes are (decks.cook_membrane), the Taylor bar of
Data/Taylor.mpm is a clipped lattice (below), and the soil slope of
Data/Slopefail.mpm is a meshed cross-section, kept as a fixture under
tests/golden/ (made by tests/golden/make_reference_fixtures.py).

REFERENCE_DECKS maps the deck's path in the reference tree to its generator.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "mpm3d-f90_gb300"))

from mpm3d_gb300 import decks  # noqa: E402
from mpm3d_gb300.decks import DeckWriter, _fast_points, _grid_lines, f32s  # noqa: E402

GOLDEN = os.path.join(HERE, "golden")


def _writer(title: str, nmat: int, span, dcell: float, kws) -> DeckWriter:
    w = DeckWriter(title)
    w.kw(f"nmat {nmat}")
    w.head += _grid_lines(span, dcell)
    for k in kws:
        w.kw(k)
    return w


def _block(w: DeckWriter, mat: int, rho: float, dp: float, origin, counts, com: int = 1) -> None:
    w.block(mat, rho, dp, origin, counts, com)


# ------------------------------------------------------------- Data/ decks
def _deto(shape: str) -> str:
    """1-D detonation of a TNT bar (Data/Deto1k.mpm, BSMPMDeto1k.mpm,
    SGDeto1k.mpm): JWL high explosive, 4000 particles, MUSL, Jaumann rate,
    bulk viscosity; linear, B-spline or SGMP shapes."""
    span = {"mpm": ((0.0, 101.0), (0.0, 0.05), (0.0, 0.05)),
            "bimp": ((-100.0, 101.0), (-0.05, 0.1), (-0.05, 0.1)),
            "sgmp": ((-0.05, 101.0), (-0.025, 0.025), (-0.025, 0.025))}[shape]
    kws = ["dtsc 0.1", "endt " + ("0.015" if shape == "mpm" else "0.005"), "outt 1e-3", "rptt 1e-4",
           "musl on", "jaum on", "bulk 1.5 0.06"]
    if shape != "mpm":
        kws.append(shape)
    kws += {"mpm": ["tecp", "para"], "bimp": ["tecp"], "sgmp": ["para"]}[shape]
    kws += ["outr pres", "outr velx"]
    if shape == "mpm":
        kws += ["curv pres 500", "curv pres 1600", "curv pres 2800", "curv pres 3900"]
    kws.append({"mpm": "fixe 2 0 2 2 2 2", "bimp": "fixe 0 0 2 2 2 2", "sgmp": "fixe 2 0 2 2 2 2"}[shape])
    kws += ["mate", f"1 hiex {f32s(1.63e-3)} 6930",
            f"seos 1 3 {f32s(3.712e5)} {f32s(3.21e3)} 4.15 0.95 0.3 6993", "deto 0 0 0"]
    w = _writer("1D TNT", 1, span, 0.05, kws)
    _block(w, 1, 1.63e-3, 0.025, (0.0, 0.0, 0.0), (4000, 1, 1))
    return w.text()


def tnt3d() -> str:
    """Data/TNT3D.mpm: a TNT cube detonated at a corner inside a
    Johnson-Cook (+ Gruneisen) copper shell of three blocks; MUSL."""
    # the deck gives its materials before the cell size, so the grid-mass
    # cut-off (CutOff * DCell**3 * 1e-5 / nmat, DataIn.f90:524) is taken with
    # DCell = 0: the regenerated deck keeps that order
    w = DeckWriter("test detonation simulation")
    w.kw("nmat 2")
    for k in ["deto 0 0 0", "mate", f"1 hiex {f32s(1.63e-3)} 6930",
              f"2 sjc {f32s(8.9e-3)} {f32s(117.0e3)} 0.31 90 392 0.5 0 {f32s(1e-3)}",
              f"seos 1 3 {f32s(3.712e5)} {f32s(3.21e3)} 4.15 0.95 0.35 6000",
              f"seos 2 2 {f32s(3.3e3)} 1.49 1.96 0", "tecp"]:
        w.kw(k)
    w.head += _grid_lines(((0.0, 25.0), (0.0, 25.0), (0.0, 25.0)), 1.0)
    for k in ["fixe 2 0 2 0 2 0", "dtsc 0.2", "endt 0.006", "musl on", "jaum on", "outt 3e-4", "rptt 5e-5",
              "pt2d 0 5 0 10 0 10", "outr pres"]:
        w.kw(k)
    _block(w, 1, 1.63e-3, 0.5, (0.0, 0.0, 0.0), (20, 20, 20))
    _block(w, 2, 8.9e-3, 0.5, (10.0, 0.0, 0.0), (10, 30, 20))
    _block(w, 2, 8.9e-3, 0.5, (0.0, 10.0, 0.0), (20, 10, 20))
    _block(w, 2, 8.9e-3, 0.5, (0.0, 0.0, 10.0), (30, 30, 10))
    return w.text()


def lead_impact() -> str:
    """Data/LeadHypervelocityImpact.mpm: a lead sphere (sphere generator)
    at 6580 m/s onto a lead plate on a second grid component; Johnson-Cook
    with failure + Gruneisen, MUSL."""
    kws = ["fixe 0 0 0 0 0 0", f"dtsc {f32s(0.001)}", "endt 0.03", "outt 0.002", "rptt 0.001", "musl on",
           "jaum on", "tecp", "pt2d -50 250 0 80 -80 80", "outr epef", "outr seqv", "outr fail", "outr velx",
           "outr cels", "mate",
           f"1 sjcf {f32s(11.350e-3)} {f32s(22.4e3)} 0.42 12 125 1 0 {f32s(1e-3)} 3",
           f"seos 1 2 {f32s(2.092e3)} 1.45 2 0"]
    w = _writer("test hypervelocity impact of lead sphere on lead plate", 1,
                ((-50.0, 250.0), (-80.0, 80.0), (-80.0, 80.0)), 2.12, kws)
    w.nbco = 2
    w.bodies.append(f"part sphe 1\n1 {f32s(13.5180e-3)} 1.06 -7.5 0 0 7")
    w.nbbo += 1
    _block(w, 1, 13.5180e-3, 1.06, (0.0, -80.0, -80.0), (6, 151, 151), com=2)
    w.nbmp = 138278  # the sphere generator's count (nbmp is read, the generators fill it)
    w.tail += ["velo", "body 1 6580 0 0", "endv"]
    return w.text()


def taylor_ref() -> str:
    """Data/Taylor.mpm: the copper Taylor bar of Johnson (1988), R 3.8 mm,
    L 25.4 mm, 0.38 mm lattice clipped to the cylinder (316 points per layer,
    67 layers, layers outermost, then x, then y), 'sjc' + Gruneisen, MUSL,
    190 m/s."""
    k = np.arange(20)
    c = np.round(-3.61 + 0.38 * k, 2)
    X, Y = np.meshgrid(c, c, indexing="ij")  # x outer, y inner
    inside = (X ** 2 + Y ** 2) <= 3.8 ** 2
    xs, ys = X[inside], Y[inside]
    layers = [np.stack([xs, ys, np.full(xs.shape, np.round(0.19 + 0.38 * j, 2))], axis=1) for j in range(67)]
    xyz = np.concatenate(layers)
    kws = ["musl on", "tecp", "para", "dtsc 0.8", "endt 0.08", "outt 0.008", "rptt 0.001", "jaum on",
           "outr epef", "outr seqv", "fixe 0 0 0 0 2 0", "mate",
           f"1 sjc {f32s(8.93e-3)} {f32s(117.0e3)} 0.35 157 425 1 0 {f32s(1e-3)}",
           "seos 1 2 3940 1.49 1.96 0"]
    w = _writer("taylor3, Johnson1988", 1, ((-11.4, 11.4), (-11.4, 11.4), (0.0, 26.6)), 0.76, kws)
    n = xyz.shape[0]
    w.bodies.append(f"part poin 1 {n}\n" + _fast_points(1, 1, 4.900070e-4, xyz))
    w.nbmp += n
    w.nbbo += 1
    w.tail += ["velo", "body 1 0 0 -190", "endv"]
    return w.text()


def slopefail() -> str:
    """Data/Slopefail.mpm: a 20 m slope on a 15 m foundation (plane strain,
    two particles through the thickness), Drucker-Prager, USF, gravity. The
    particle set is the fixture tests/golden/slopefail_points.npz."""
    z = np.load(os.path.join(GOLDEN, "slopefail_points.npz"))
    mass, xyz = z["mass"], np.stack([z["x"], z["y"], z["z"]], axis=1)
    kws = ["dtsc 0.2", "endt 15", "outt 0.2", "rptt 0.05", "usf on", "jaum on", "bulk 1.5 0.06", "tecp",
           "outr epef", "outr seqv", "outr pres", "pt2d 0 180 -2 4 -20 25", "fixe 2 2 2 2 1 0", "mate",
           f"1 dpm {f32s(2.1e3)} {f32s(0.7e8)} 0.3 0.3545 {f32s(9.74e3)} 0 {f32s(27.48e3)}"]
    w = _writer("slopefail", 1, ((0.0, 110.0), (0.0, 1.0), (-15.0, 20.0)), 1.0, kws)
    w.points(1, mass, xyz)
    w.tail += ["load", "grav 1 0 0 -9.8", "endl"]
    return w.text()


# ------------------------------------------------- VolumetricLockingEx/ decks
def dam(variant: str) -> str:
    """VolumetricLockingEx/DamBreak/{MPM/Dam_R2, SGMPM/Dam_SGR2,
    SGMPMvsPressure/Dam_SGR2}.mpm: a water column collapsing under gravity
    (null material + weakly compressible EOS), plane strain, MUSL, stress
    smoothing; linear or SGMP shapes."""
    if variant == "mpm":
        span, dcell, dts, et, ot, rt = ((0, 4.125), (0, 2.125), (0, 0.125)), 0.125, "0.8", "0.68", "0.01", "0.002"
        blk, mat, eos, bulk, curves = (997.5, 0.025, (0, 0, 0.05), (40, 80, 1)), "1 null 997.5 2e9 0.001", \
            "seos 1 4 1415", "bulk 1.5 0.06", ["curv disy 3161", "curv disx 40"]
    elif variant == "sgmp":
        span, dcell, dts, et, ot, rt = ((-0.125, 4.25), (-0.125, 2.125), (0, 0.125)), 0.125, "0.8", "0.68", \
            "0.01", "0.002"
        blk, mat, eos, bulk, curves = (997.5, 0.025, (0, 0, 0.05), (40, 80, 1)), "1 null 997.5 2e9 0.001", \
            "seos 1 4 1415", "bulk 1.5 1.0", ["curv disy 3161", "curv disx 40"]
    else:  # SGMP, fine resolution (pressure study)
        span, dcell, dts, et, ot, rt = ((-0.0019, 0.2869), (-0.0019, 0.1159), (0, 0.0019)), 0.0019, "0.9", \
            "0.14", "0.001", "0.0005"
        blk, mat, eos, bulk, curves = (1000.0, 4.75e-4, (0, 0, 7.125e-4), (120, 240, 1)), \
            "1 null 1000 2e7 0.001", "seos 1 4 141.5", "bulk 1.5 0.5", ["curv disy 28681", "curv disx 120"]
    kws = [f"dtsc {dts}", f"endt {et}", f"outt {ot}", f"rptt {rt}", "musl on"]
    if variant != "mpm":
        kws.append("sgmp")
    kws += ["smoo", bulk, "para"] + curves + ["fixe 2 0 2 0 2 2", "mate", mat, eos]
    w = _writer("3D DamBreak_withoutBarrier", 1, span, dcell, kws)
    rho, dp, org, cnt = blk
    _block(w, 1, rho, dp, org, cnt)
    w.tail += ["load", "grav 1 0 -9.81 0", "endl"]
    return w.text()


def free_soft_beam(shape: str, nu: str) -> str:
    """VolumetricLockingEx/FreeSoftBeam/{MPM,SGMPM}_v0p{3,499}: a free
    neo-Hookean beam set swinging by a sine velocity profile ('vsin'),
    plane strain, MUSL; linear or SGMP shapes."""
    wide = nu == "0.3" or shape == "sgmp"
    span = ((-1.5, 2.1 if nu == "0.3" else 2.0), (-0.1, 6.2 if wide else 6.1), (0.0, 0.1))
    kws = ["dtsc 0.9", "endt 3", "outt 0.1", "rptt 0.01", "musl on", "para"]
    if shape == "sgmp":
        kws.append("sgmp")
    kws.append("curv disx 2400")
    if shape == "mpm" and nu == "0.3":
        kws.append("outr pres")
    kws += ["fixe 0 0 0 0 2 2", "mate", f"1 neoh 1100 {f32s(17e6)} {nu}"]
    w = _writer("FreeSoftBeam_NeoHook", 1, span, 0.1, kws)
    _block(w, 1, 1100.0, 0.05, (-1.0, 0.0, 0.025), (20, 120, 1))
    w.tail += ["velo", "vsin 1", "endv"]
    return w.text()


def soft_beam_tl(shape: str, mesh: str) -> str:
    """VolumetricLockingEx/SoftBeam/{SBTL,SBSGTL}_{0p1,0p05}mesh: a
    neo-Hookean cantilever in the total Lagrangian form ('TLmp', 'UVFp'),
    struck sideways at 10 m/s, plane strain, MUSL, stress smoothing; linear
    or SGMP shapes."""
    fine = mesh == "0p05"
    h = 0.05 if fine else 0.1
    if shape == "sgmp":
        span = ((-1.05, 0.05), (-0.05, 6.05), (0.0, 0.05)) if fine else ((-1.1, 0.1), (-0.1, 6.1), (0.0, 0.1))
    else:
        span = ((-1.0, 0.0), (0.0, 6.0), (0.0, h))
    kws = ["dtsc 0.9", "endt 1.2", "outt 0.1", "rptt 0.02", "musl on"]
    if shape == "sgmp":
        kws.append("sgmp")
    kws += ["smoo", "UVFp", "TLmp"]
    if fine:
        kws += ["bulk 1.5 0.06", f"curv disx 9600", "para"]
    else:
        kws += ["para", "curv disx 2400", "outr pres"]
    kws += ["fixe 0 0 1 0 2 2", "mate", f"1 neoh 1100 {f32s(17e6)} 0.499"]
    w = _writer("SoftBeam_TLMPM", 1, span, h, kws)
    if fine:
        _block(w, 1, 1100.0, 0.025, (-1.0, 0.0, 0.0125), (40, 240, 1))
    else:
        _block(w, 1, 1100.0, 0.05, (-1.0, 0.0, 0.025), (20, 120, 1))
    w.tail += ["velo", "body 1 10 0 0", "endv"]
    return w.text()


_COOK_OUT = ("outt 5", "rptt 0.5", "para")

REFERENCE_DECKS = {
    "Data/Deto1k.mpm": lambda: _deto("mpm"),
    "Data/BSMPMDeto1k.mpm": lambda: _deto("bimp"),
    "Data/SGDeto1k.mpm": lambda: _deto("sgmp"),
    "Data/TNT3D.mpm": tnt3d,
    "Data/LeadHypervelocityImpact.mpm": lead_impact,
    "Data/Taylor.mpm": taylor_ref,
    "Data/Slopefail.mpm": slopefail,
    "VolumetricLockingEx/DamBreak/MPM/Dam_R2.mpm": lambda: dam("mpm"),
    "VolumetricLockingEx/DamBreak/SGMPM/Dam_SGR2.mpm": lambda: dam("sgmp"),
    "VolumetricLockingEx/DamBreak/SGMPMvsPressure/Dam_SGR2.mpm": lambda: dam("sgmp_fine"),
    "VolumetricLockingEx/FreeSoftBeam/MPM_v0p3/FreeSB_MPM.mpm": lambda: free_soft_beam("mpm", "0.3"),
    "VolumetricLockingEx/FreeSoftBeam/MPM_v0p499/FreeSB_MPM.mpm": lambda: free_soft_beam("mpm", "0.499"),
    "VolumetricLockingEx/FreeSoftBeam/SGMPM_v0p3/FreeSB_SGMPM.mpm": lambda: free_soft_beam("sgmp", "0.3"),
    "VolumetricLockingEx/FreeSoftBeam/SGMPM_v0p499/FreeSB_SGMPM.mpm": lambda: free_soft_beam("sgmp", "0.499"),
    "VolumetricLockingEx/SoftBeam/SBTL_0p1mesh/SBTL.mpm": lambda: soft_beam_tl("mpm", "0p1"),
    "VolumetricLockingEx/SoftBeam/SBTL_0p05mesh/SBTL.mpm": lambda: soft_beam_tl("mpm", "0p05"),
    "VolumetricLockingEx/SoftBeam/SBSGTL_0p1mesh/SBSGTL.mpm": lambda: soft_beam_tl("sgmp", "0p1"),
    "VolumetricLockingEx/SoftBeam/SBSGTL_0p05mesh/SBSGTL.mpm": lambda: soft_beam_tl("sgmp", "0p05"),
}
for _v, _p in {"mpm": "MPM", "gimp": "GIMP", "bimp": "BSMPM", "sgmp": "SG"}.items():
    _f5 = {"mpm": "Cookmo_MPM", "gimp": "Cookmo_Gimp", "bimp": "Cookmo_Bimp", "sgmp": "Cookmo_SG"}[_v]
    _f23 = {"mpm": "Cookmo_0p5m", "gimp": "Cookmo_GIMP0p5m", "bimp": "Cookmo_BS0p5m", "sgmp": "Cookmo_SG0p5m"}[_v]
    REFERENCE_DECKS[f"VolumetricLockingEx/Cook_membrane/{_p}5776p/{_f5}.mpm"] = \
        (lambda v=_v: decks.cook_membrane(v, 0.5, extra=_COOK_OUT))
    REFERENCE_DECKS[f"VolumetricLockingEx/Cook_membrane/{_p}23072p/{_f23}.mpm"] = \
        (lambda v=_v: decks.cook_membrane(v, 0.25, extra=_COOK_OUT))
