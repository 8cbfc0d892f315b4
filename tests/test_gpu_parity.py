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
import pytest

from gpu_cases import CASES, check_strict, rel as _rel, run_pair as _run_pair


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_strict_bit_identical(gpu_mod, oracle_mod, name):
    make, steps = CASES[name]
    g, o = _run_pair(gpu_mod, oracle_mod, make(), steps, "fp64", "project")
    check_strict(g, o, name, steps)


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
