"""Admission decisions of the serving runtime (host logic, no GPU): the same
function the server thread calls at every admission point."""
import pytest


def test_fifo_stops_at_first_misfit(gpu_mod):
    from mpm3d_gb300 import serve_plan
    adm, rej = serve_plan([100, 100, 100], [10, 10, 10], [40, 70, 10], "fifo", budget=100)
    # scene 1 does not fit after scene 0; FIFO does not skip ahead to scene 2
    assert adm == [0] and rej == []


def test_shortest_orders_by_work(gpu_mod):
    from mpm3d_gb300 import serve_plan
    np_ = [5000, 100, 2000, 100]
    steps = [10, 500, 10, 10]  # work 50000, 50000, 20000, 1000
    adm, rej = serve_plan(np_, steps, [1, 1, 1, 1], "shortest")
    assert adm == [3, 2, 0, 1]  # ties keep submission order


def test_particle_cap_admits_a_lone_scene(gpu_mod):
    from mpm3d_gb300 import serve_plan
    adm, _ = serve_plan([500, 10], [1, 1], [1, 1], "fifo", max_resident_particles=100)
    assert adm == [0]  # over the cap but alone: admitted; the next waits
    adm, _ = serve_plan([10, 500], [1, 1], [1, 1], "fifo", max_resident_particles=100, resident=(1, 50, 1))
    assert adm == [0]
    adm, _ = serve_plan([60], [1], [1], "fifo", max_resident_particles=100, resident=(1, 50, 1))
    assert adm == []


def test_over_budget_scene_rejected_only_when_nothing_resident(gpu_mod):
    from mpm3d_gb300 import serve_plan
    adm, rej = serve_plan([10, 10], [1, 1], [500, 50], "fifo", budget=100)
    assert rej == [0] and adm == [1]
    adm, rej = serve_plan([10, 10], [1, 1], [500, 50], "fifo", budget=100, resident=(1, 10, 10))
    assert rej == [] and adm == []  # it might fit later... never, but the head blocks until residents retire


def test_scene_cap(gpu_mod):
    from mpm3d_gb300 import serve_plan
    adm, _ = serve_plan([1] * 10, [1] * 10, [1] * 10, "fifo", max_scenes=4, resident=(1, 1, 1))
    assert adm == [0, 1, 2]


def test_empty_queue(gpu_mod):
    from mpm3d_gb300 import serve_plan
    assert serve_plan([], [], [], "shortest") == ([], [])
