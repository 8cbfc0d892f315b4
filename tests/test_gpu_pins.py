"""End-to-end pins on the GPU (marked gpu).

1. The eight Cook-membrane decks (linear, GIMP, B-spline, SGMP; 5776 and
   23072 particles), regenerated exactly, run in FP64 to the reference's
   quasi-static exit test (MPM3D.f90:152-156) and compared with the tip
   vertical displacements of VolumetricLockingEx/ExamplesResults.pdf, Table 1.
   The 5776-particle decks must round to the published values (4 digits).
   The 23072-particle decks as shipped in the reference tree end 0.3-0.5%
   below the table (0.2678 / 0.2680 / 0.2702 / 0.2731 against 0.2692 /
   0.2688 / 0.2711 / 0.2739), although by then they have settled (the tips
   move by less than 1e-4 from t = 100 to t = 220), while the 5776 runs are
   still creeping at the exit test and match the table at that instant: the
   table's 23072 figures come from settings other than the shipped decks'.
   Those four are held to 0.6% of the table.
2. The 1000-step Taylor bar: the full bar (16 k particles, Johnson-Cook with
   failure + linear EOS, USF) for 1000 steps. The strict FP64 form must be bit
   identical to the oracle with the same libm; against the oracle on glibc the
   nodal momentum and particle stress must agree to 1e-10 relative, or to the
   spread the libm choice causes on the CPU alone if that is larger.
"""
import numpy as np
import pytest


def _tip(step_obj, x0):
    return step_obj.download("Xp")[1, -1] - x0


@pytest.mark.gpu
@pytest.mark.parametrize("particles", [5776, 23072])
@pytest.mark.parametrize("variant", ["mpm", "gimp", "bimp", "sgmp"])
def test_cook_membrane_published_tip_displacement(gpu_mod, variant, particles):
    from mpm3d_gb300 import decks

    spacing = 0.5 if particles == 5776 else 0.25
    published = decks.COOK_TIP_PUBLISHED if particles == 5776 else decks.COOK_TIP_PUBLISHED_23072
    deck = gpu_mod.Deck.parse(decks.cook_membrane(variant, spacing))
    assert deck.nb_particle == particles
    s = gpu_mod.MpmStep(deck, precision="fp64", device=0)
    x0 = s.download("Xp")[1, -1]
    n = 0
    while True:
        s.step()
        n += 1
        sc = s.scalars()
        if sc["CurrentTime"] > 30 and sc["EngKinetic"] / (sc["EngKinetic"] + sc["EngInternal"]) < 0.005 \
                and sc["CurrentTime"] > 100:
            break
        assert n < 80000
    tip = _tip(s, x0)
    print(f"cook {variant} {particles}: tip {tip:.6f} after {n} steps (published {published[variant]})")
    if particles == 5776:
        assert round(tip, 4) == published[variant], (variant, particles, tip, n)
    else:
        assert abs(tip - published[variant]) <= 0.006 * published[variant], (variant, particles, tip, n)


def _rel(a, b):
    s = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b)) / s) if s > 0 else float(np.max(np.abs(a - b)))


@pytest.mark.gpu
def test_taylor_bar_1000_steps_vs_oracle(gpu_mod, oracle_mod):
    from mpm3d_gb300 import decks

    text = decks.taylor_bar()
    deck = gpu_mod.Deck.parse(text)
    g = gpu_mod.MpmStep(deck, precision="fp64", device=0)
    g.run(1000, graph=True)
    g.sync()
    op = oracle_mod.Oracle(deck_text=text, libm="project")
    op.run(1000)
    for f in ("PXg", "Mg", "FXg", "SM", "SD", "Xp", "VXp", "epeff", "celsius_t", "ie"):
        assert np.array_equal(g.download(f), op.download(f)), f
    assert float(np.max(op.download("epeff"))) > 0.05  # the bar has yielded
    og = oracle_mod.Oracle(deck_text=text, libm="system")
    og.run(1000)
    for f in ("PXg", "SM", "SD"):
        spread = _rel(op.download(f), og.download(f))
        r = _rel(g.download(f), og.download(f))
        print(f"taylor 1000 steps {f}: GPU vs glibc oracle {r:.2e}, libm spread {spread:.2e}")
        assert r <= max(1e-10, 2 * spread), (f, r, spread)
