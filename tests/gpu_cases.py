"""Parity cases shared by the GPU tests: small decks that the oracle runs in
seconds, each exercising one shape family / scheme / material path; and the
strict-form comparison the parity tests share."""
import sys
import os

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "mpm3d-f90_gb300"))

from mpm3d_gb300 import decks  # noqa: E402

# name -> (deck text factory, steps)
CASES = {
    "taylor_small_usf_jcf_linear": (lambda: decks.taylor_bar(dp=8e-4), 100),
    "slope_small_usf_dp_gimp": (lambda: decks.soil_slope(dp=0.5, width=2.0), 60),
    "dam_small_musl_null_bspline": (lambda: decks.dam_break(dp=0.1, h=0.2), 40),
    "beam_musl_neoh_sgmp": (lambda: decks.soft_beam(), 60),
    "beam_usl_neoh_linear": (lambda: decks.soft_beam(shape="mpm", scheme="usl"), 60),
    "cook_musl_neoh_quasistatic": (lambda: decks.cook_membrane(), 60),
    # Cook panels carry 'smoo': stress smoothing every step, one per shape family
    "cook_smooth_gimp": (lambda: decks.cook_membrane("gimp", spacing=1.0), 40),
    "cook_smooth_bspline": (lambda: decks.cook_membrane("bimp", spacing=1.0), 40),
    "cook_smooth_sgmp": (lambda: decks.cook_membrane("sgmp", spacing=1.0), 40),
    # two blocks on separate grid components meeting head-on (Lagr_NodContact)
    "contact_linear_usf": (lambda: decks.contact_blocks(None, "usf", fricfa=0.0, normbody=0), 50),
    "contact_gimp_musl_friction": (lambda: decks.contact_blocks("gimp", "musl", fricfa=0.3, normbody=1), 50),
    "contact_bspline_usl_friction": (lambda: decks.contact_blocks("bimp", "usl", fricfa=0.3, normbody=2), 50),
    # total Lagrangian form (neo-Hookean soft beam under gravity), one per shape family
    "tl_beam_linear_usf": (lambda: decks.soft_beam(shape="mpm", scheme="usf", tlmpm=True), 40),
    "tl_beam_gimp_musl": (lambda: decks.soft_beam(shape="gimp", scheme="musl", tlmpm=True), 40),
    "tl_beam_bspline_usl": (lambda: decks.soft_beam(shape="bimp", scheme="usl", tlmpm=True), 40),
    "tl_beam_sgmp_musl": (lambda: decks.soft_beam(shape="sgmp", scheme="musl", tlmpm=True), 40),
    "block_usf_elastic": (lambda: decks.generic_block("1 elas 1000 1e7 0.3"), 60),
    "block_musl_pla1_gimp": (lambda: decks.generic_block("1 pla1 1000 1e7 0.3 2e4", shape="gimp",
                                                         scheme="musl", velocity=(1.0, 0.0, -20.0)), 60),
    "block_usl_pla2_bspline": (lambda: decks.generic_block("1 pla2 1000 1e7 0.3 2e4 1e5", shape="bimp",
                                                           scheme="usl", velocity=(0.0, 2.0, -20.0)), 60),
    "block_usf_john": (lambda: decks.generic_block(
        "1 john 8930 1.17e11 0.35 9e7 2.92e8 0.31 0.025 1.09 293 1356 383 1", dp=4e-4,
        velocity=(0.0, 0.0, -150.0), rho=8930.0, dtscale=0.2, gravity=None), 80),
    "block_musl_sjc_gruneisen": (lambda: decks.generic_block(
        "1 sjc 8930 1.17e11 0.35 1.57e8 4.25e8 1.0 0.0 1e-3", "seos 1 2 3940 1.49 1.96 0", dp=4e-4,
        velocity=(0.0, 0.0, -200.0), rho=8930.0, dtscale=0.2, gravity=None, scheme="musl"), 80),
    "block_usf_sjcf_gruneisen": (lambda: decks.generic_block(
        "1 sjcf 8930 1.17e11 0.35 9e7 2.92e8 0.31 0.025 1 0.02", "seos 1 2 3940 1.49 1.96 0", dp=4e-4,
        velocity=(0.0, 0.0, -300.0), rho=8930.0, dtscale=0.2, gravity=None), 80),
    "block_musl_hiex_jwl": (lambda: decks.generic_block(
        "1 hiex 1630 6930", "seos 1 3 3.712e11 3.21e9 4.15 0.95 0.3 6.993e9", dp=5e-4,
        velocity=(0.0, 0.0, 0.0), rho=1630.0, dtscale=0.1, gravity=None, scheme="musl",
        extra=["deto 0 0 0"]), 60),
}


PARTICLE_FIELDS = ["Xp", "XX", "VXp", "VOL", "SM", "Seqv", "SD", "epeff", "sig_y", "ie", "q",
                   "celsius_t", "failure", "icell", "XN", "cp", "Spre", "PK"]
GRID_FIELDS = ["Mg", "PXg", "FXg"]


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(np.max(np.abs(b)), 1e-300) if b.size else 1.0
    return float(np.max(np.abs(a - b)) / scale) if a.size else 0.0


def run_pair(gpu_mod, oracle_mod, text, steps, precision, libm):
    """The GPU form `precision` and the oracle on libm `libm`, both advanced
    `steps` steps from the same deck text."""
    deck = gpu_mod.Deck.parse(text)
    g = gpu_mod.MpmStep(deck, precision=precision, device=0)
    o = oracle_mod.Oracle(deck_text=text, libm=libm)
    g.run(steps, graph=False)
    g.sync()
    o.run(steps)
    return g, o


def check_strict(g, o, name, steps):
    """The FP64 strict form against the oracle on the project libm: the same
    step count, time and DT; every grid and particle field bit-identical; the
    sums over particles (energies, momentum, contact force), which the GPU
    reduces in a fixed tree and the oracle sequentially, equal to rounding."""
    gs, os_ = g.scalars(), o.scalars()
    assert gs["istep"] == os_["istep"] == steps
    fg, fo = g.contact_force(), o.contact_force()
    assert np.all(np.abs(fg - fo) <= 1e-12 * max(np.abs(fo).max(), 1e-300)), (fg, fo)
    assert gs["DT"] == os_["DT"], (gs["DT"], os_["DT"])
    assert gs["CurrentTime"] == os_["CurrentTime"]
    bad = []
    for f in GRID_FIELDS + PARTICLE_FIELDS:
        a, b = g.download(f), o.download(f)
        if not np.array_equal(a, b):
            diff = np.argwhere(a != b)
            bad.append((f, int(diff.shape[0]), rel(a, b)))
    assert not bad, f"{name}: fields differ from the oracle: {bad}"
    v = o.download("VXp")
    mass = o.download("mass")
    mom_scale = float(np.sum(mass * np.abs(v).max(axis=0)))
    for k in ("EngKinetic", "EngInternal"):
        assert abs(gs[k] - os_[k]) <= 1e-12 * max(abs(os_[k]), 1e-300), (k, gs[k], os_[k])
    for k in ("Momentum_x", "Momentum_y", "Momentum_z"):
        assert abs(gs[k] - os_[k]) <= 1e-12 * max(mom_scale, 1e-300), (k, gs[k], os_[k])
