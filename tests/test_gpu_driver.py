"""The C command-line driver (host/mpm3d_gpu_main.c), the stand-in for the
reference's time loop (MPM3D.f90:62-160) while no Fortran compiler exists to
build the ISO_C_BINDING shim: run on a deck for a fixed number of steps in the
FP64 strict form, it must write the same curve and energy files as the CPU
oracle driven through the same output writer, and end in the oracle's state
bit for bit. The run uses the shim's memory sequence (--pinned: the deck
page-locked around mpm_create, the final read-back into mpm_host_alloc
memory), so that sequence runs on a GPU although the shim itself cannot be
compiled here."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "mpm3d-f90_gb300", "_build", "mpm3d_gpu")
STEPS = 40
CURVES = ["curv seqv 3", "curv disz 40", "curv stsx 7", "curv velz 12", "curv pres 100", "curv fail 5",
          "curv damg 9", "curv cels 2"]


def _deck_text():
    from mpm3d_gb300 import decks
    return decks.generic_block(
        "1 john 8930 1.17e11 0.35 9e7 2.92e8 0.31 0.025 1.09 293 1356 383 1", dp=4e-4,
        velocity=(0.0, 0.0, -150.0), rho=8930.0, dtscale=0.2, gravity=None, extra=CURVES)


def _oracle_files(oracle_mod, gpu_mod, text, job):
    """The same files written from the oracle's state after each step."""
    from mpm3d_gb300 import Deck, Output
    d = Deck.parse(text)
    o = oracle_mod.Oracle(deck_text=text, libm="project")
    out = Output(d, job)
    items = out.curve_items()
    for _ in range(STEPS):
        o.step()
        vals = []
        for p, f, c in items:
            name = [k for k, v in gpu_mod.FIELDS.items() if v == f][0]
            a = o.download(name)
            vals.append(a[c][p] if a.ndim == 2 else a[p])
        out.curve(np.array(list(o.scalars().values())), vals)
    out.close()
    return o


@pytest.mark.parametrize("pinned", [False, True])
def test_driver_files_and_state_match_oracle(gpu_mod, oracle_mod, tmp_path, pinned):
    text = _deck_text()
    (tmp_path / "gpu").mkdir()
    (tmp_path / "cpu").mkdir()
    deck = tmp_path / "gpu" / "run.mpm"
    deck.write_text(text)
    cmd = [DRIVER, str(deck), "--steps", str(STEPS), "--report", "0", "--dump", str(tmp_path / "final.bin")]
    if pinned:
        cmd.append("--pinned")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Time per particle cycle" in r.stdout
    o = _oracle_files(oracle_mod, gpu_mod, text, str(tmp_path / "cpu" / "run"))
    for f in ["run_curv.dat", "EnergyPlot.dat", "MomentumPlot.dat"]:
        a = (tmp_path / "gpu" / f).read_text()
        b = (tmp_path / "cpu" / f).read_text()
        assert len(a.splitlines()) == (STEPS + 1 if f == "run_curv.dat" else STEPS), f
        if f != "MomentumPlot.dat":
            assert a == b, f
            continue
        # momentum sums: the GPU's fixed reduction tree and the oracle's
        # sequential loop round differently in components that are zero up
        # to rounding
        ra = np.array([[float(x) for x in ln.split()] for ln in a.splitlines()])
        rb = np.array([[float(x) for x in ln.split()] for ln in b.splitlines()])
        assert np.all(ra[:, 0] == rb[:, 0])
        assert np.abs(ra[:, 1:] - rb[:, 1:]).max() <= 1e-12 * np.abs(rb[:, 1:]).max()
    n = o.nb_particle
    raw = np.fromfile(tmp_path / "final.bin", dtype=np.float64)
    assert raw.size == 13 * n
    off = 0
    for name, comp in (("Xp", 3), ("VXp", 3), ("SM", 1), ("SD", 6)):
        got = raw[off:off + comp * n]
        off += comp * n
        np.testing.assert_array_equal(got, o.download(name).ravel(), err_msg=name)
    o.close()
