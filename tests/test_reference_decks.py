"""The reference's example decks as the parity tests run them.

Where the reference tree is present: each deck regenerated by
tests/reference_decks.py parses into exactly the reference deck's data --
every field of the parsed record (particles, bodies, materials and EOS
constants, grid, boundary codes, loads, velocities, time-step and output
settings), bit for bit. Independently of the library's reader, the real
numbers of the reference decks' particle lists are compared with their
decimal text rounded once to a 32-bit REAL (GetReal, FFI.f90:110-138), so a
wrong rounding in the reader, which the oracle shares, would show here.
Everywhere: the regenerated decks parse and hold their stated particle
counts.
"""
import os

import numpy as np
import pytest

from deck_struct import deck_record, diff_records
from reference_decks import REFERENCE_DECKS
from golden.make_reference_fixtures import read_point_list

EXPECTED_NP = {"Data/Deto1k.mpm": 4000, "Data/TNT3D.mpm": 27000, "Data/LeadHypervelocityImpact.mpm": 138278,
               "Data/Taylor.mpm": 21172, "Data/Slopefail.mpm": 19640}


@pytest.mark.parametrize("name", sorted(REFERENCE_DECKS))
def test_regenerated_deck_parses(gpu_mod, name):
    d = gpu_mod.Deck.parse(REFERENCE_DECKS[name]())
    if name in EXPECTED_NP:
        assert d.nb_particle == EXPECTED_NP[name]
    assert d.nb_particle > 0


@pytest.mark.parametrize("name", sorted(REFERENCE_DECKS))
def test_regenerated_deck_equals_reference(gpu_mod, reference_tree, name):
    a = gpu_mod.Deck.load(os.path.join(reference_tree, name))
    b = gpu_mod.Deck.parse(REFERENCE_DECKS[name]())
    bad = diff_records(deck_record(a), deck_record(b))
    assert not bad, (name, bad)


@pytest.mark.parametrize("name", ["Data/Taylor.mpm", "Data/Slopefail.mpm",
                                  "VolumetricLockingEx/Cook_membrane/SG23072p/Cookmo_SG0p5m.mpm"])
def test_point_lists_read_as_real4(gpu_mod, reference_tree, name):
    path = os.path.join(reference_tree, name)
    want = read_point_list(path)
    got = gpu_mod.Deck.load(path).particles()
    np.testing.assert_array_equal(got["mass"], want["mass"].astype(np.float64))
    for k, c in (("x", 0), ("y", 1), ("z", 2)):
        np.testing.assert_array_equal(got["Xp"][c], want[k].astype(np.float64), err_msg=k)
