"""Result files (DataOut.f90 layouts) from host arrays: Fortran edit
descriptors, the curve / energy / momentum rows, Tecplot and ParaView
frames. Host code only."""
import os

import numpy as np
import pytest


def test_fortran_e_descriptor(gpu_mod):
    from mpm3d_gb300 import format_e
    assert format_e(12, 4, 1.2345) == "  0.1234E+01"   # 1.2345 is 1.23449999... in binary
    assert format_e(12, 4, -0.5) == " -0.5000E+00"
    assert format_e(12, 4, 0.0) == "  0.0000E+00"
    assert format_e(12, 4, 123456.0) == "  0.1235E+06"
    assert format_e(12, 4, 9.99995) == "  0.1000E+02"
    assert format_e(12, 4, -2.5e-7) == " -0.2500E-06"
    assert format_e(12, 4, 1e100) == "  0.1000+101"     # three-digit exponents drop the E
    assert format_e(10, 3, 3.0e-4) == " 0.300E-03"


def _deck(extra):
    from mpm3d_gb300 import Deck, decks
    return Deck.parse(decks.generic_block("1 elas 1000 1e7 0.3", counts=(2, 2, 2), extra=extra))


def test_curve_energy_momentum_rows(gpu_mod, tmp_path):
    from mpm3d_gb300 import FIELDS, Output
    d = _deck(["curv seqv 3", "curv disz 5", "curv stsx 2", "curv fail 1"])
    job = str(tmp_path / "job")
    with Output(d, job) as out:
        items = out.curve_items()
        assert items == [(2, FIELDS["Seqv"], 0), (4, FIELDS["Xp"], 2), (1, FIELDS["SD"], 0), (1, FIELDS["SM"], 0),
                         (0, FIELDS["failure"], 0)]
        sc = np.zeros(16)
        sc[1], sc[3], sc[4], sc[5:8] = 1e-3, 2.0, 3.0, (0.1, -0.2, 0.3)
        xp5 = d.particles()["Xp"][2, 4]
        out.curve(sc, [7.0, xp5 - 0.25, 1.5, -0.5, 1.0])
    lines = open(job + "_curv.dat").read().splitlines()
    assert lines[0] == "Time engk1       engi1       seqv3       disz5       stsx2       fail1       "
    assert lines[1] == ("  0.1000E-02  0.2000E+01  0.3000E+01  0.7000E+01 -0.2500E+00  0.1000E+01"
                        "           1")
    e = open(str(tmp_path / "EnergyPlot.dat")).read().splitlines()
    assert e == ["  0.1000E-02  0.5000E+01  0.2000E+01  0.3000E+01"]
    mo = open(str(tmp_path / "MomentumPlot.dat")).read().splitlines()
    assert mo == ["  0.1000E-02  0.1000E+00 -0.2000E+00  0.3000E+00"]


def test_tecplot_and_paraview_frames(gpu_mod, tmp_path):
    from mpm3d_gb300 import Output
    d = _deck(["outr seqv", "outr pres", "tecp", "para"])
    n = d.nb_particle
    p = d.particles()
    f = {"xp": p["Xp"], "vxp": p["VXp"], "fxp": p["FXp"], "mass": p["mass"], "seqv": np.arange(n, dtype=float),
         "sm": -np.ones(n), "vol": np.ones(n), "celsius": np.zeros(n), "dmg": np.zeros(n), "sd": np.zeros(6 * n),
         "epeff": np.zeros(n), "spre": np.full(n, 2.5)}
    job = str(tmp_path / "run")
    sc = np.zeros(16)
    with Output(d, job) as out:
        out.anim(sc, f)
        sc[1] = 2e-4
        out.anim(sc, f)
    tec = open(job + "_anim.dat").read().splitlines()
    assert tec[0].startswith('TITLE = "') and len(tec[0]) == len('TITLE = ""') + 60
    # names go through the A2, A4, A1 descriptors of format 20 in turn
    assert tec[1] == 'VARIABLES= "X"   "Y"   "Z"  "m"seq"'
    assert tec[2] == 'ZONE T="time 0.000E+00"'
    assert len(tec) == 2 + 2 * (1 + n)
    assert tec[3 + n] == 'ZONE T="time 0.200E-03"'
    row = tec[3]
    assert len(row) == 3 * 12 + 3 + 12 + 12  # X Y Z, material (I3), seqv, pressure
    assert row[36:39] == "  1" and row[-12:] == "  0.1000E+01"
    assert os.path.exists(job + "_anim_1.vtu") and os.path.exists(job + "_anim_2.vtu")
    vtu = open(job + "_anim_1.vtu").read().splitlines()
    k = vtu.index('            <DataArray type="Float32" Name="Smoothpressure" Format="ascii">')
    assert vtu[k + 1] == "                  0.2500E+01"
    k = vtu.index('            <DataArray type="Float32" Name="SmoothMeanNormalStress" Format="ascii">')
    assert vtu[k + 1] == "                 -0.2500E+01"
    pvd = open(job + "_anim.pvd").read().splitlines()
    assert pvd[-2:] == ["    </Collection>", "</VTKFile>"]
    assert pvd[3] == f'    <DataSet timestep="  0.0000E+00" group="" part="0" file="{job}_anim_1.vtu"/>'
    vtu = open(job + "_anim_2.vtu").read()
    assert f'<Piece NumberOfPoints="{n}" NumberOfCells="{n}">' in vtu and vtu.count("<DataArray") == 1 + 20 + 3
    grid = open(job + "_Grid.vtu").read()
    assert 'Name="connectivity"' in grid and grid.rstrip().endswith("</VTKFile>")


def test_contact_force_plot(gpu_mod, tmp_path):
    """With contact on, OutCurve also writes ContforcPlot.dat (time and the
    total contact force, 4E12.4) next to EnergyPlot.dat."""
    from mpm3d_gb300 import Deck, Output, decks
    d = Deck.parse(decks.contact_blocks())
    job = str(tmp_path / "blocks")
    with Output(d, job) as out:
        out.contact(2e-3, [1.5, -0.25, 0.0])
    rows = open(str(tmp_path / "ContforcPlot.dat")).read().splitlines()
    assert rows == ["  0.2000E-02  0.1500E+01 -0.2500E+00  0.0000E+00"]
