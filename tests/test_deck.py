"""The .mpm reader (include/mpm_deck.h) against the reference's FFI /
DataIn rules: field splitting, REAL(4) conversion, keyword matching, order
constraints, generators and error reporting. CPU only."""
import math
import re
import os

import numpy as np
import pytest

HEAD = "nbco 1\nnbbo 1\nnbmp {n}\nnmat 1\nspx 0 4\nspy 0 4\nspz 0 4\ndcel 1\n"


def parse(m, text):
    return m.Deck.parse(text)


def one_point(x="1.5", extra="", mat="1 elas 1000 1e7 0.3"):
    return (HEAD.format(n=1) + extra + "mate\n" + mat + "\npart poin 1 1\n1 1 2.0 " + x + " 1.5 1.5\nendi\n")


def test_reals_are_read_as_float32(gpu_mod):
    d = parse(gpu_mod, one_point(x="0.1"))
    x = d.particles()["Xp"][0, 0]
    assert x == float(np.float32(0.1)) and x != 0.1


def test_fortran_d_exponent_and_comments_and_tabs(gpu_mod):
    txt = one_point(x="1.25d0").replace("spx 0 4", "spx\t0, 4   ! comment, 7 8")
    d = parse(gpu_mod, txt)
    assert d.particles()["Xp"][0, 0] == 1.25
    assert d.scalars()["spx1"] == 4.0


def test_keywords_case_insensitive_4_chars(gpu_mod):
    txt = one_point().replace("mate\n", "MATERIAL\n").replace("part poin", "Particle POINT")
    d = parse(gpu_mod, txt)
    assert d.nb_particle == 1


def test_musl_is_default_even_after_musl_off(gpu_mod):
    d = parse(gpu_mod, one_point(extra="musl off\n"))
    assert d.flags["MUSL"]
    d = parse(gpu_mod, one_point(extra="usf on\n"))
    assert d.flags["USF"] and not d.flags["MUSL"]


def test_cutoff_uses_float_literal(gpu_mod):
    d = parse(gpu_mod, one_point())
    # CutOff = density * DCell**3 * REAL(1e-5) / nmat (DataIn.f90:524)
    assert d.scalars()["CutOff"] == 1000.0 * 1.0 * float(np.float32(1e-5)) / 1


def test_field_truncated_to_20_characters(gpu_mod):
    d = parse(gpu_mod, one_point(x="1.500000000000000000009"))
    assert d.particles()["Xp"][0, 0] == 1.5


def test_errors_are_reported_not_fatal(gpu_mod):
    with pytest.raises(gpu_mod.MpmError) as e:
        parse(gpu_mod, one_point(x="abc"))
    assert e.value.code == 3 and "non-numeric" in str(e.value)
    with pytest.raises(gpu_mod.MpmError) as e:
        parse(gpu_mod, one_point().replace("endi\n", ""))
    assert "end of file" in str(e.value)
    with pytest.raises(gpu_mod.MpmError) as e:
        parse(gpu_mod, "nmat 1\nmate\n1 elas 1 1 0.3\nendi\n")
    assert "nbmp" in str(e.value)
    with pytest.raises(gpu_mod.MpmError):
        parse(gpu_mod, one_point().replace("nmat 1", "nmat 1\nfoo 3"))
    with pytest.raises(gpu_mod.MpmError) as e:
        parse(gpu_mod, one_point(extra=" ".join(["spx 0 4"] * 6) + "\n"))
    assert "fields" in str(e.value)


def test_block_generator_positions_and_mass(gpu_mod):
    txt = (HEAD.format(n=24) + "mate\n1 elas 1000 1e7 0.3\npart bloc 1 1 1000 0.5 0 0 1 2 3 4\nendi\n")
    d = parse(gpu_mod, txt)
    p = d.particles()
    assert p["mass"][0] == 1000.0 * 0.5 ** 3
    assert np.allclose(p["Xp"][:, 0], [0.25, 0.25, 1.25])
    assert np.allclose(p["Xp"][:, -1], [0.75, 1.25, 2.75])


def test_sphere_and_disc_generators(gpu_mod):
    base = HEAD.replace("spx 0 4\nspy 0 4\nspz 0 4", "spx -4 4\nspy -4 4\nspz -4 4")
    n_sphere = sum(1 for i in range(-1, 3) for j in range(-1, 3) for k in range(-1, 3)
                   if ((i - 0.5) ** 2 + (j - 0.5) ** 2 + (k - 0.5) ** 2) * 0.25 < 1.0)
    txt = base.format(n=n_sphere) + "mate\n1 elas 1000 1e7 0.3\npart sphe 1 1 1000 0.5 0 0 0 2\nendi\n"
    assert parse(gpu_mod, txt).nb_particle == n_sphere
    n_disc = sum(1 for i in range(-1, 3) for j in range(-1, 3) if ((i - 0.5) ** 2 + (j - 0.5) ** 2) * 0.25 < 1.0)
    txt = base.format(n=n_disc) + "mate\n1 elas 1000 1e7 0.3\npart cicl 1 1 1000 0.5 0 0 0 2\nendi\n"
    assert parse(gpu_mod, txt).nb_particle == n_disc


def test_velocity_load_gravity_eos(gpu_mod):
    txt = one_point(mat="1 sjc 8930 1.17e11 0.35 1.57e8 4.25e8 1 0 1e-3\nseos 1 2 3940 1.49 1.96 0")
    txt = txt.replace("endi\n", "velo\nbody 1 0 0 -190\nendv\nload\npart 1 1 2 3\ngrav 1 0 0 -9.81\nendl\nendi\n")
    d = parse(gpu_mod, txt)
    p = d.particles()
    assert p["VXp"][2, 0] == -190.0 and list(p["FXp"][:, 0]) == [1.0, 2.0, 3.0]
    assert d.flags["Gravity"]


def test_library_exports_every_declared_symbol(gpu_mod):
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    names = set()
    for h in ("mpm3d_gpu.h", "mpm_deck.h"):
        txt = open(os.path.join(root, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"\b(mpm_[a-z0-9_]+)\s*\(", txt))
    lib = gpu_mod.library()
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert len(names) >= 25
