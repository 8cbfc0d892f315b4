"""GPU step vs the CPU oracle, through the C ABI (marked gpu).

MPM_FP64_STRICT (reference summation order, no FMA, project libm) must be
bit-identical to the oracle built with the same libm after N steps: nodal
mass / momentum / force and every particle field. MPM_FP64_NATIVE (CUDA libm)
is compared with the oracle on the system libm at 1e-10 relative, the
tolerance the FP64 path is specified to meet -- except where the choice of
libm by itself moves the CPU result further: Johnson-Cook plasticity rounds
the equivalent stress to REAL(4) and branches on it, so a 1-ulp difference in
pow / log can flip a particle between the elastic and plastic branch. For
those fields the bar is twice the spread between the oracle on the project
libm and the oracle on glibc for the same deck and steps.
"""
import numpy as np
import pytest

from gpu_cases import CASES

PARTICLE_FIELDS = ["Xp", "XX", "VXp", "VOL", "SM", "Seqv", "SD", "epeff", "sig_y", "ie", "q",
                   "celsius_t", "failure", "icell", "XN", "cp", "Spre", "PK"]
GRID_FIELDS = ["Mg", "PXg", "FXg"]


def _run_pair(gpu_mod, oracle_mod, text, steps, precision, libm):
    deck = gpu_mod.Deck.parse(text)
    g = gpu_mod.MpmStep(deck, precision=precision, device=0)
    o = oracle_mod.Oracle(deck_text=text, libm=libm)
    g.run(steps, graph=False)
    g.sync()
    o.run(steps)
    return g, o


def _rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale) if a.size else 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_strict_bit_identical(gpu_mod, oracle_mod, name):
    make, steps = CASES[name]
    text = make()
    g, o = _run_pair(gpu_mod, oracle_mod, text, steps, "fp64", "project")
    gs, os_ = g.scalars(), o.scalars()
    assert gs["istep"] == os_["istep"] == steps
    # the total contact force is summed over nodes in a fixed tree order on the
    # GPU, node by node on the CPU
    fg, fo = g.contact_force(), o.contact_force()
    assert np.all(np.abs(fg - fo) <= 1e-12 * max(np.abs(fo).max(), 1e-300)), (fg, fo)
    assert gs["DT"] == os_["DT"], (gs["DT"], os_["DT"])
    assert gs["CurrentTime"] == os_["CurrentTime"]
    bad = []
    for f in GRID_FIELDS + PARTICLE_FIELDS:
        if f == "XN" and "sgmp" in name:
            pass
        a, b = g.download(f), o.download(f)
        if not np.array_equal(a, b):
            diff = np.argwhere(a != b)
            bad.append((f, int(diff.shape[0]), _rel(a, b)))
    assert not bad, f"{name}: fields differ from the oracle: {bad}"
    # energies are reduced in a fixed tree order on the GPU, sequentially on the
    # CPU: equal to rounding, measured against the sum of the magnitudes
    v = o.download("VXp")
    mass = o.download("mass")
    mom_scale = float(np.sum(mass * np.abs(v).max(axis=0)))
    for k in ("EngKinetic", "EngInternal"):
        assert abs(gs[k] - os_[k]) <= 1e-12 * max(abs(os_[k]), 1e-300), (k, gs[k], os_[k])
    for k in ("Momentum_x", "Momentum_y", "Momentum_z"):
        assert abs(gs[k] - os_[k]) <= 1e-12 * max(mom_scale, 1e-300), (k, gs[k], os_[k])


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_native_within_1e10(gpu_mod, oracle_mod, name):
    make, steps = CASES[name]
    text = make()
    g, o = _run_pair(gpu_mod, oracle_mod, text, steps, "native", "system")
    op = oracle_mod.Oracle(deck_text=text, libm="project")
    op.run(steps)
    for f in ["PXg", "Mg", "SM", "SD", "Xp", "VXp"]:
        spread = _rel(op.download(f), o.download(f))  # libm choice alone, on the CPU
        tol = max(1e-10, 2.0 * spread)
        r = _rel(g.download(f), o.download(f))
        assert r <= tol, (name, f, r, spread)
