"""Larger workloads through size-independent properties: the granular
column (GIMP, MUSL, Drucker-Prager) at 1/4 of the benchmark spacing (about 1 M
particles on a 128 x 128 x 64 grid) -- mixed against FP64, grid mass equal to
particle mass, and the batch / alone identity."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(a)))


@pytest.fixture(scope="module")
def column(built):
    from mpm3d_gb300 import Deck, decks
    text, n = decks.granular_column(4.0)
    d = Deck.parse(text)
    assert d.nb_particle == n
    return d


def test_column_mixed_vs_fp64(column):
    from mpm3d_gb300 import MpmStep
    a = MpmStep(column, "fp64")
    b = MpmStep(column, "mixed")
    a.run(20)
    b.run(20)
    for f in ["PXg", "Mg", "SM", "SD", "Xp", "VXp"]:
        err = _rel(a.download(f), b.download(f))
        assert err <= 1e-5, f"{f}: {err:.3g}"


def test_column_grid_mass_equals_particle_mass(column):
    """Every particle is inside the grid and GIMP weights sum to one, so the
    grid holds the particles' mass (FP64 form to rounding; the mixed form to
    the FP32 rounding of the weights)."""
    from mpm3d_gb300 import MpmStep
    pm = float(np.sum(column.particles()["mass"]))
    for form, tol in (("fp64", 1e-12), ("mixed", 1e-6)):
        s = MpmStep(column, form)
        s.run(3)
        gm = float(np.sum(s.download("Mg")))
        assert abs(gm - pm) <= tol * pm, f"{form}: grid {gm} particles {pm}"


def test_column_batch_identity(column, built):
    """The column alone and beside a second scene in one batch: bit-identical."""
    from mpm3d_gb300 import Batch, Deck, decks
    other = Deck.parse(decks.dam_break(dp=0.05, h=0.1))
    with Batch() as b1:
        i = b1.add(column, 10)
        b1.run(10)
        ref = b1.download(i, "Xp")
    with Batch() as b2:
        b2.add(other, 10)
        i = b2.add(column, 10)
        b2.run(10)
        np.testing.assert_array_equal(b2.download(i, "Xp"), ref)
