"""Mixed-precision batched engine: accuracy against the FP64 GPU form, and the
identity of a scene's results whatever else shares its batch (alone, mixed
with other scenes, admitted mid-run, served by the serving runtime)."""
import time

import numpy as np
import pytest

from gpu_cases import CASES

pytestmark = pytest.mark.gpu

# Relative error bound of the mixed form against FP64 strict (max |a - b| /
# max |a| per field) after the case's step count: 1e-5, the bound the mixed
# form is held to. Where a case cannot meet it, the bound below says why, with
# the numbers measured on a GB300 beside it -- the mixed error and the spread
# of the FP64 strict form itself when its initial positions are perturbed by
# 1e-12 (relative, seeded), which measures how much the case amplifies any
# perturbation:
# * Johnson-Cook cases: the plastic threshold switches particles between
#   elastic and plastic steps, which amplifies rounding-size differences by
#   orders of magnitude. Taylor bar ('jcf', 100 steps): SD 5.4e-2 mixed, 6.8e-5
#   from a 1e-12 FP64 perturbation; the other fields 1.3e-5..5.6e-5.
#   Simplified Johnson-Cook + Gruneisen (80 steps): mixed 1.0e-3 / 4.0e-3 /
#   3.4e-3 (PXg / SM / SD), the 1e-12 FP64 perturbation 8.2e-4 / 4.9e-3 /
#   2.4e-3 -- the case is chaotic at any precision. With failure ('sjcf'),
#   rounding flips individual particles' failure flags: PXg 2.0e-2 mixed, 1.2e-3
#   from the FP64 perturbation.
# * Nearly incompressible neo-Hookean Cook membranes (nu = 0.499): the mean
#   stress is lamda ln J with lamda = 499 G, and the trace of the FP32 velocity
#   gradient that drives J cancels about 500:1, so SM keeps FP32 rounding
#   times ~500: 1.3e-5 after 300 B-spline steps (other fields <= 6e-7).
MIXED_TOL = {
    # the FP32 Johnson-Cook return moves SD by up to 5e-2 and, through it,
    # VXp by 6e-5 .. 1.4e-4 depending on the order of FP32 roundings (sort
    # keys, increments, the energy / DT partial sums)
    "taylor_small_usf_jcf_linear": {"SD": 0.1, "VXp": 2e-4, "*": 1e-4},
    "block_musl_sjc_gruneisen": {"*": 2e-2},
    "block_usf_sjcf_gruneisen": {"*": 5e-2},
}
DEFAULT_TOL = 1e-5
COOK_TOL = {"SM": 3e-5, "*": DEFAULT_TOL}
# Spre is SM smoothed through the grid: it carries SM's error and the FP32
# shape weights of the two transfers
SMOOTH_TOL = 1e-4


def _tol(table, field):
    return table.get(field, table.get("*", DEFAULT_TOL))


FIELDS = ["PXg", "Mg", "SM", "SD", "Xp", "VXp"]


def _rel(a, b):
    s = float(np.max(np.abs(a))) if a.size else 0.0
    d = float(np.max(np.abs(a - b))) if a.size else 0.0
    return d / s if s > 0 else d


@pytest.mark.parametrize("name", sorted(n for n in CASES if not n.startswith(("contact", "tl_"))))
def test_mixed_vs_fp64(built, name):
    from mpm3d_gb300 import Deck, MpmStep
    mk, steps = CASES[name]
    d = Deck.parse(mk())
    a = MpmStep(d, "fp64")
    a.run(steps)
    a.sync()
    b = MpmStep(d, "mixed")
    b.run(steps)
    b.sync()
    for f in FIELDS:
        tol = _tol(MIXED_TOL.get(name, {}), f)
        err = _rel(a.download(f), b.download(f))
        assert err <= tol, f"{name} {f}: mixed vs FP64 relative error {err:.3g} > {tol}"
    sa, sb = a.scalars(), b.scalars()
    assert sa["istep"] == sb["istep"] == steps


@pytest.mark.parametrize("variant", ["mpm", "gimp", "bimp", "sgmp"])
def test_mixed_cook_vs_fp64(built, variant):
    """Nearly incompressible neo-Hookean (nu = 0.499): the mixed form derives
    J - 1 and B - I from Fp - I without cancellation."""
    from mpm3d_gb300 import Deck, MpmStep, decks
    d = Deck.parse(decks.cook_membrane(variant))
    a = MpmStep(d, "fp64")
    b = MpmStep(d, "mixed")
    a.run(300)
    b.run(300)
    for f in FIELDS:
        err = _rel(a.download(f), b.download(f))
        assert err <= _tol(COOK_TOL, f), f"cook {variant} {f}: {err:.3g}"


MIX = ["slope_small_usf_dp_gimp", "beam_musl_neoh_sgmp", "block_usf_john", "dam_small_musl_null_bspline"]
PFIELDS = ["Xp", "VXp", "SM", "SD", "PXg"]


def _alone(deck, steps):
    from mpm3d_gb300 import Batch
    with Batch() as bt:
        sid = bt.add(deck, steps=steps)
        bt.run(steps)
        bt.sync()
        return {f: bt.download(sid, f) for f in PFIELDS}


def test_batch_alone_vs_mix_identity(built):
    """Four scenes of four shape families in one batch: each scene's state is
    bit-identical to the scene run alone; scenes stop at their step count."""
    from mpm3d_gb300 import Batch, Deck
    decks_ = {n: Deck.parse(CASES[n][0]()) for n in MIX}
    alone = {n: _alone(decks_[n], 30) for n in MIX}
    with Batch() as bt:
        ids = {n: bt.add(decks_[n], steps=30) for n in MIX}
        bt.run(45)
        bt.sync()
        for n in MIX:
            assert bt.scalars(ids[n])["istep"] == 30
            for f in PFIELDS:
                np.testing.assert_array_equal(bt.download(ids[n], f), alone[n][f], err_msg=f"{n} {f}")


def test_batch_admission_mid_run_identity(built):
    """Scenes admitted and retired while others run (the batch is re-laid out
    on the device each time) keep bit-identical results; eager and graph
    launches agree."""
    from mpm3d_gb300 import Batch, Deck
    decks_ = {n: Deck.parse(CASES[n][0]()) for n in MIX}
    alone = {n: _alone(decks_[n], 30) for n in MIX[:3]}
    with Batch() as bt:
        i0 = bt.add(decks_[MIX[0]], steps=30)
        bt.run(10)
        i1 = bt.add(decks_[MIX[1]], steps=30)
        bt.run(25, graph=False)
        i2 = bt.add(decks_[MIX[2]], steps=30)
        bt.remove(i0)
        bt.run(7)
        bt.run(33)
        bt.sync()
        for n, i in ((MIX[1], i1), (MIX[2], i2)):
            for f in PFIELDS:
                np.testing.assert_array_equal(bt.download(i, f), alone[n][f], err_msg=f"{n} {f}")


def test_batch_block_shape_invariance(built):
    """Launch shapes (the autotuner's knobs) change no result."""
    from mpm3d_gb300 import Batch, Deck
    d = Deck.parse(CASES[MIX[0]][0]())
    ref = _alone(d, 20)
    with Batch() as bt:
        sid = bt.add(d, steps=20)
        bt.set_blocks(128, 512)
        bt.run(20)
        for f in PFIELDS:
            np.testing.assert_array_equal(bt.download(sid, f), ref[f], err_msg=f)


def test_serving_runtime(built):
    """Sixteen serving scenes (Cook panels and soft beams, SGMP, MUSL,
    neo-Hookean) submitted from the host while earlier ones run: all finish
    their step count, latencies are reported, and a served scene's fields are
    bit-identical to the same scene run alone."""
    from mpm3d_gb300 import Deck, Server, decks
    rng = np.random.default_rng(3)
    scenes = [Deck.parse(decks.serving_scene(rng, 2000, 40000)[0]) for _ in range(16)]
    alone = _alone(scenes[5], 60)
    with Server(chunk_steps=16, autotune=True) as srv:
        tickets = []
        for d in scenes:
            tickets.append(srv.submit(d, 60, fields=["Xp", "SD", "VXp"]))
            time.sleep(0.005)
        for t in tickets:
            assert srv.wait(t, 300000)
        st = srv.stats()
        assert st["finished"] == 16 and st["resident"] == 0 and st["queued"] == 0
        # the autotuner timed its candidates on one composition and chose
        shape = srv.launch_shape()
        assert shape is not None and shape["scatter_blocks_per_sm"] in (8, 32, 64)
        for t in tickets:
            r = srv.result(t)
            assert r["istep"] == 60
            assert 0 <= r["queue_ms"] <= r["latency_ms"]
        for f in ["Xp", "SD", "VXp"]:
            np.testing.assert_array_equal(srv.field(tickets[5], f), alone[f], err_msg=f)
        srv.release(tickets[0])


def test_serving_budget_admission(built):
    """A budget that holds one scene at a time still runs every scene, and a
    scene larger than the budget fails alone instead of blocking the queue."""
    from mpm3d_gb300 import Batch, Deck, MpmError, Server, decks
    rng = np.random.default_rng(5)
    small = [Deck.parse(decks.serving_scene(rng, 3000, 6000)[0]) for _ in range(3)]
    big = Deck.parse(decks.serving_scene(rng, 50000, 60000)[0])
    budget = max(Batch.scene_bytes(d) for d in small) + 1
    assert Batch.scene_bytes(big) > budget
    with Server(hbm_budget_bytes=budget, chunk_steps=10) as srv:
        t_big = srv.submit(big, 10)
        ts = [srv.submit(d, 20) for d in small]
        with pytest.raises(MpmError):
            srv.wait(t_big, 60000)
        for t in ts:
            assert srv.wait(t, 60000)
        assert srv.stats()["peak_resident_bytes"] <= budget


def test_serving_shortest_first(built):
    """With one scene resident at a time, the shortest-work-first policy runs
    the small queued scenes before a larger one submitted earlier."""
    from mpm3d_gb300 import Deck, Server, decks
    rng = np.random.default_rng(9)
    first = Deck.parse(decks.serving_scene(rng, 20000, 20001, kind="beam")[0])
    big = Deck.parse(decks.serving_scene(rng, 30000, 30001, kind="beam")[0])
    small = [Deck.parse(decks.serving_scene(rng, 2000, 2001, kind="beam")[0]) for _ in range(2)]
    with Server(chunk_steps=10, policy="shortest", max_resident_particles=1) as srv:
        t0 = srv.submit(first, 300)
        tb = srv.submit(big, 20)
        ts = [srv.submit(d, 20) for d in small]
        for t in [t0, tb] + ts:
            assert srv.wait(t, 120000)
        done_big = srv.result(tb)["latency_ms"]
        for t in ts:
            assert srv.result(t)["latency_ms"] < done_big


@pytest.mark.parametrize("variant", ["mpm", "gimp", "bimp", "sgmp"])
def test_mixed_stress_smoothing(built, variant):
    """Spre of the mixed form (computed from the state after the last step
    when read) against the FP64 form, and the same alone or in a batch."""
    from mpm3d_gb300 import Batch, Deck, MpmStep, decks
    d = Deck.parse(decks.cook_membrane(variant, spacing=1.0))
    a = MpmStep(d, "fp64")
    b = MpmStep(d, "mixed")
    a.run(40)
    b.run(40)
    sa, sb = a.download("Spre"), b.download("Spre")
    assert np.all(np.isfinite(sb)) and np.any(sa != 0.0)
    err = _rel(sa, sb)
    assert err <= SMOOTH_TOL, f"cook {variant} Spre: {err:.3g}"
    # with a scene of another material (the batch then runs one stress
    # instantiation per material type): the same state and Spre
    other = Deck.parse(CASES["slope_small_usf_dp_gimp"][0]())
    with Batch() as bt:
        bt.add(other, steps=40)
        sid = bt.add(d, steps=40)
        bt.run(40)
        for f in ["Xp", "SD", "Spre"]:
            np.testing.assert_array_equal(bt.download(sid, f), b.download(f), err_msg=f)


def test_mixed_refuses_contact(built):
    """The batched engine keeps one grid per scene: decks with contact run
    in the FP64 forms only."""
    from mpm3d_gb300 import Deck, MpmError, MpmStep, decks
    with pytest.raises(MpmError):
        MpmStep(Deck.parse(decks.contact_blocks()), "mixed")


@pytest.mark.parametrize("name", ["slope_small_usf_dp_gimp", "beam_musl_neoh_sgmp", "block_usf_elastic_drda"])
def test_run_splitting_and_energies(built, name):
    """A step's energy / DT reduction overlaps the next step's sort on a
    second stream, and the last reduction of a run ends it: one run of n
    steps, n runs of one step and an eager run give the same state, energies,
    momentum and DT -- with dynamic relaxation, whose damping reads the
    kinetic energy of the step before."""
    from mpm3d_gb300 import Batch, Deck
    if name.endswith("_drda"):
        text = CASES[name[: -len("_drda")]][0]().replace("usf on\n", "usf on\ndrda\n")
        assert "drda" in text
    else:
        text = CASES[name][0]()
    d = Deck.parse(text)
    keys = ("istep", "CurrentTime", "DT", "EngKinetic", "EngInternal", "Momentum_x", "Momentum_y", "Momentum_z",
            "EngKinetic_prev")
    out = []
    for mode in ("one_run", "split", "eager"):
        with Batch() as bt:
            sid = bt.add(d, steps=24)
            if mode == "one_run":
                bt.run(24)
            elif mode == "split":
                for _ in range(24):
                    bt.run(1)
            else:
                bt.run(24, graph=False)
            bt.sync()
            sc = bt.scalars(sid)
            out.append(({k: sc[k] for k in keys}, {f: bt.download(sid, f) for f in PFIELDS}))
    for sc, fields in out[1:]:
        assert sc == out[0][0]
        for f in PFIELDS:
            np.testing.assert_array_equal(fields[f], out[0][1][f], err_msg=f"{name} {f}")


def _outlier_deck(outlier: bool) -> str:
    """A GIMP elastic block drifting at 0.05 m/s and, with outlier, one more
    particle of the same mass two cells above it moving at 5 m/s -- 100 times
    the block's speed, so that its momentum alone sets the scene's
    fixed-point bound for the momentum transfers. The two share no node."""
    from mpm3d_gb300.decks import DeckWriter, _grid_lines, f32s
    dp, h = 0.5, 1.0
    w = DeckWriter("elastic block with an outlier particle")
    w.kw("nmat 1")
    w.head += _grid_lines(((-2.0, 6.0), (-2.0, 4.0), (0.0, 9.0)), h)
    w.kw("dtsc 0.5")
    w.kw("endt 100.0")
    w.kw("usf on")
    w.kw("gimp")
    w.kw("fixe 0 0 0 0 1 0")
    w.kw("mate")
    w.kw("1 elas 1000 1e7 0.3")
    w.block(1, 1000.0, dp, (0.0, 0.0, h), (8, 4, 6))
    velo = ["velo", "body 1 0 0 %s" % f32s(-0.05)]
    if outlier:
        w.block(1, 1000.0, dp, (1.0, 1.0, 6.5), (1, 1, 1))
        velo.append("body 2 %s 0 0" % f32s(5.0))
    w.tail += velo + ["endv"]
    return w.text()


def test_mixed_outlier_particle(built):
    """The fixed-point scale of a scene's grid sums comes from its largest
    single contribution. One particle 100 times faster than the rest must not
    coarsen the others' sums: the block's particle fields keep the same
    error against FP64 with the outlier present as without it."""
    from mpm3d_gb300 import Deck, MpmStep
    errs = {}
    for outlier in (False, True):
        d = Deck.parse(_outlier_deck(outlier))
        a = MpmStep(d, "fp64")
        b = MpmStep(d, "mixed")
        a.run(60)
        b.run(60)
        nb = 8 * 4 * 6
        e = {}
        for f in ("SM", "SD", "VXp"):
            fa, fb = a.download(f), b.download(f)
            fa = fa.reshape(-1, d.nb_particle)[:, :nb]
            fb = fb.reshape(-1, d.nb_particle)[:, :nb]
            e[f] = _rel(fa, fb)
        errs[outlier] = e
        if outlier:  # the outlier really dominates the momentum bound
            v = a.download("VXp").reshape(3, -1)
            assert np.max(np.abs(v[:, nb:])) > 50 * np.max(np.abs(v[:, :nb]))
        a.close()
        b.close()
    # (the outlier also shortens DT by a few per cent, so the two runs do not
    # take the same steps: the bound is an order of magnitude, not equality)
    for f, e in errs[True].items():
        assert e <= 1e-5, f"{f}: {e:.3g} with the outlier"
        assert e <= 10 * max(errs[False][f], 1e-7), f"{f}: {e:.3g} with the outlier, {errs[False][f]:.3g} without"


def test_batch_device_loop(built):
    """The device-resident run loop: the device repeats steps until a scene
    takes its last step (or the step budget is spent, or the host interrupts
    it), with the same results as host-driven runs."""
    import threading
    from mpm3d_gb300 import Batch, Deck, decks
    dk = [Deck.parse(decks.soft_beam()), Deck.parse(decks.soil_slope(dp=0.5, width=2.0))]
    with Batch() as ref:
        a = ref.add(dk[0], steps=40)
        b = ref.add(dk[1], steps=25)
        ref.run(41)
        ref.sync()
        want = {s: {f: ref.download(s, f) for f in PFIELDS} for s in (a, b)}
    with Batch() as bt:
        a = bt.add(dk[0], steps=40)
        b = bt.add(dk[1], steps=25)
        assert bt.run_loop(7) == 7  # the budget
        # steps 8.. in one launch: the loop test after each pair of steps sees
        # scene b take its last step (25) in the pair (25, 26)
        assert bt.run_loop(1000) == 19
        assert bt.scalars(b)["istep"] == 25 and bt.scalars(a)["istep"] == 26
        assert bt.run_loop(1000) == 15  # scene a's last step (40) in the pair (40, 41)
        assert bt.scalars(a)["istep"] == 40
        assert bt.run_loop(1000) == 1  # nothing left to do: the first step only
        bt.sync()
        for s in (a, b):
            for f in PFIELDS:
                assert np.array_equal(bt.download(s, f), want[s][f]), (s, f)
    # the host interrupts a loop that would otherwise run for 10^6 steps
    with Batch() as bt:
        s = bt.add(dk[0], steps=1_000_000)
        bt.commit()
        got = {}
        th = threading.Thread(target=lambda: got.setdefault("n", bt.run_loop(1_000_000)))
        th.start()
        time.sleep(0.3)
        bt.interrupt()
        th.join(timeout=60)
        assert not th.is_alive() and 1 <= got["n"] < 1_000_000
        assert bt.scalars(s)["istep"] == got["n"]
        assert bt.run_loop(5) == 5  # the request was consumed


def _dense_deck() -> str:
    """An elastic block of ordinary density (8 particles per cell) beside a
    cluster of 22^3 = 10648 particles inside one cell: the counting sort's
    segments then have every length class -- up to 32 particles (one thread),
    33..8192 (a block in shared memory: the cluster's neighbouring keys) and
    beyond 8192 (a block in global memory: the cluster's own key)."""
    from mpm3d_gb300.decks import DeckWriter, _grid_lines, f32s
    h = 1.0
    w = DeckWriter("block and a dense cluster")
    w.kw("nmat 1")
    w.head += _grid_lines(((-2.0, 10.0), (-2.0, 4.0), (0.0, 6.0)), h)
    w.kw("dtsc 0.5")
    w.kw("endt 100.0")
    w.kw("usf on")
    w.kw("fixe 0 0 0 0 1 0")
    w.kw("mate")
    w.kw("1 elas 1000 1e7 0.3")
    w.block(1, 1000.0, 0.5, (0.0, 0.0, 1.0), (8, 4, 6))
    dp = h / 22
    w.block(1, 1000.0, dp, (6.0 + dp / 2, 1.0 + dp / 2, 2.0 + dp / 2), (22, 22, 22))
    w.tail += ["velo", "body 1 0 0 %s" % f32s(-1.0), "body 2 %s 0 0" % f32s(0.5), "endv"]
    return w.text()


def test_mixed_sort_long_segments(built):
    """Segments of every length sort into the same order each run (results
    bit-identical run to run and alone vs in a batch) and the step stays
    within the mixed form's bound of FP64."""
    from mpm3d_gb300 import Batch, Deck, MpmStep
    d = Deck.parse(_dense_deck())
    runs = []
    for _ in range(2):
        m = MpmStep(d, "mixed")
        m.run(30)
        runs.append({f: m.download(f) for f in PFIELDS})
        m.close()
    for f in PFIELDS:
        assert np.array_equal(runs[0][f], runs[1][f]), f
    with Batch() as bt:
        bt.add(Deck.parse(CASES["slope_small_usf_dp_gimp"][0]()), steps=30)  # another scene in the batch
        sid = bt.add(d, steps=30)
        bt.run(30)
        bt.sync()
        for f in ["Xp", "VXp", "SM", "SD"]:
            assert np.array_equal(bt.download(sid, f), runs[0][f]), f
    a = MpmStep(d, "fp64")
    a.run(30)
    for f in ["PXg", "SM", "SD", "VXp"]:
        err = _rel(a.download(f), runs[0][f])
        assert err <= DEFAULT_TOL, f"{f}: {err:.3g}"
    a.close()
