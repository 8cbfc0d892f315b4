"""The reference's own example decks through the GPU step (marked gpu).

Every example deck of the reference tree (Data/*.mpm and
VolumetricLockingEx/**/*.mpm, regenerated exactly by tests/reference_decks.py)
runs in the FP64 strict form for a step count the CPU oracle finishes in a
few seconds, and must be bit-identical to the oracle: every grid and particle
field, DT and time. These decks hold the reference's own edge cases: a
material section read before the cell size (TNT3D: a grid-mass cut-off of 0),
two grid components without contact and the sphere generator
(LeadHypervelocityImpact), JWL detonation with lighting times (Deto1k and its
B-spline / SGMP forms), Johnson-Cook with failure, Gruneisen, Drucker-Prager
on a meshed slope, the sine velocity profile 'vsin', the total Lagrangian
form and stress smoothing. The Cook membranes run to their published end
points in tests/test_gpu_pins.py.
"""
import pytest

from gpu_cases import check_strict, run_pair
from reference_decks import REFERENCE_DECKS

STEPS = {
    "Data/Deto1k.mpm": 200, "Data/BSMPMDeto1k.mpm": 200, "Data/SGDeto1k.mpm": 200,
    "Data/TNT3D.mpm": 100, "Data/LeadHypervelocityImpact.mpm": 10, "Data/Taylor.mpm": 60,
    "Data/Slopefail.mpm": 100,
    "VolumetricLockingEx/DamBreak/MPM/Dam_R2.mpm": 200,
    "VolumetricLockingEx/DamBreak/SGMPM/Dam_SGR2.mpm": 200,
    "VolumetricLockingEx/DamBreak/SGMPMvsPressure/Dam_SGR2.mpm": 60,
    "VolumetricLockingEx/FreeSoftBeam/MPM_v0p3/FreeSB_MPM.mpm": 200,
    "VolumetricLockingEx/FreeSoftBeam/MPM_v0p499/FreeSB_MPM.mpm": 200,
    "VolumetricLockingEx/FreeSoftBeam/SGMPM_v0p3/FreeSB_SGMPM.mpm": 200,
    "VolumetricLockingEx/FreeSoftBeam/SGMPM_v0p499/FreeSB_SGMPM.mpm": 200,
    "VolumetricLockingEx/SoftBeam/SBTL_0p1mesh/SBTL.mpm": 200,
    "VolumetricLockingEx/SoftBeam/SBTL_0p05mesh/SBTL.mpm": 100,
    "VolumetricLockingEx/SoftBeam/SBSGTL_0p1mesh/SBSGTL.mpm": 200,
    "VolumetricLockingEx/SoftBeam/SBSGTL_0p05mesh/SBSGTL.mpm": 100,
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(STEPS))
def test_reference_deck_strict_bit_identical(gpu_mod, oracle_mod, name):
    steps = STEPS[name]
    g, o = run_pair(gpu_mod, oracle_mod, REFERENCE_DECKS[name](), steps, "fp64", "project")
    check_strict(g, o, name, steps)
    g.close()
    o.close()
