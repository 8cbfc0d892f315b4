"""Restart snapshots of the FP64 and mixed forms: a run saved half-way and
continued in a new context from the file ends bit-identical to the
uninterrupted run."""
import numpy as np
import pytest

from gpu_cases import CASES

pytestmark = pytest.mark.gpu

FIELDS = ["Xp", "VXp", "SM", "SD", "VOL", "ie", "epeff", "celsius_t", "Seqv", "PXg", "Mg"]


@pytest.mark.parametrize("name", ["taylor_small_usf_jcf_linear", "beam_musl_neoh_sgmp", "block_musl_sjc_gruneisen"])
def test_restart_bit_identical(built, tmp_path, name):
    from mpm3d_gb300 import Deck, MpmStep
    mk, steps = CASES[name]
    d = Deck.parse(mk())
    half = steps // 2
    a = MpmStep(d, "fp64")
    a.run(half)
    snap = str(tmp_path / "state.snap")
    a.save(snap)
    a.run(steps - half)
    b = MpmStep(d, "fp64")
    b.load(snap)
    b.run(steps - half)
    for f in FIELDS:
        np.testing.assert_array_equal(a.download(f), b.download(f), err_msg=f"{name} {f}")
    sa, sb = a.scalars(), b.scalars()
    for k in ("istep", "CurrentTime", "DT", "EngKinetic", "EngInternal"):
        assert sa[k] == sb[k], k


@pytest.mark.parametrize("name", ["slope_small_usf_dp_gimp", "beam_musl_neoh_sgmp", "block_musl_sjc_gruneisen",
                                  "dam_small_musl_null_bspline", "taylor_small_usf_jcf_linear"])
def test_restart_bit_identical_mixed(built, tmp_path, name):
    from mpm3d_gb300 import Deck, MpmStep
    mk, steps = CASES[name]
    d = Deck.parse(mk())
    half = steps // 2
    a = MpmStep(d, "mixed")
    a.run(half)
    snap = str(tmp_path / "state.snap")
    a.save(snap)
    a.run(steps - half)
    b = MpmStep(d, "mixed")
    b.run(1)  # a context that has run steps of its own is overwritten by the load
    b.load(snap)
    b.run(steps - half)
    for f in ["Xp", "VXp", "SM", "SD", "VOL", "ie", "epeff", "Seqv", "PXg", "Mg"]:
        np.testing.assert_array_equal(a.download(f), b.download(f), err_msg=f"{name} {f}")
    sa, sb = a.scalars(), b.scalars()
    for k in ("istep", "CurrentTime", "DT", "EngKinetic", "EngInternal"):
        assert sa[k] == sb[k], k


def test_snapshot_refuses_other_deck_and_precision(built, tmp_path):
    from mpm3d_gb300 import Deck, MpmError, MpmStep
    d1 = Deck.parse(CASES["block_usf_elastic"][0]())
    d2 = Deck.parse(CASES["block_usf_john"][0]())
    a = MpmStep(d1, "fp64")
    a.run(2)
    snap = str(tmp_path / "s.snap")
    a.save(snap)
    with pytest.raises(MpmError):
        MpmStep(d2, "fp64").load(snap)
    with pytest.raises(MpmError):
        MpmStep(d1, "mixed").load(snap)
    m = MpmStep(d1, "mixed")
    m.run(2)
    msnap = str(tmp_path / "m.snap")
    m.save(msnap)
    with pytest.raises(MpmError):
        MpmStep(d2, "mixed").load(msnap)
    with pytest.raises(MpmError):
        MpmStep(d1, "fp64").load(msnap)
