"""More than 128 solver colours.  A dynamic 20 x 0.5 x 20 m plate carrying
400 boxes is one body in 401 manifolds: the greedy colouring needs at least 401
colours, several windows of the per-body colour masks.  The reference solves
such a pile (sequential_impulse_solver.cpp:520-621 has no colour limit); so
must the GPU, bit for bit equal to the oracle fed the same colour order, in the
single-world engine and in the batched engine."""
import numpy as np
import pytest

from helpers import assert_bit_equal, assert_manifolds_equal, colors_valid
from oracle import cpu
from phys_gb300 import scenes

pytestmark = pytest.mark.gpu

DT = 1 / 60


def plate_scene(side=20, box=0.9):
    """A static 40 x 1 x 40 floor, a dynamic 20 x 0.5 x 20 plate resting on
    it, and side x side boxes of edge `box` on the plate, 1 m apart (no two
    boxes touch, so every box's only contact is the plate)."""
    f = np.float32
    pos = [[0.0, -0.5, 0.0], [0.0, 0.25, 0.0]]
    dims = [[40.0, 1.0, 40.0], [20.0, 0.5, 20.0]]
    for i in range(side):
        for k in range(side):
            pos.append([f(-9.5) + f(i), f(0.5) + f(box) * f(0.5), f(-9.5) + f(k)])
            dims.append([box, box, box])
    n = len(pos)
    static = np.zeros(n, np.uint8)
    static[0] = 1
    return scenes.Scene(shape=np.ones(n, np.uint8), is_static=static, dims=np.array(dims, f), pos=np.array(pos, f),
                        density=np.ones(n, f), restitution=np.zeros(n, f), friction=np.full(n, f(0.5)),
                        linvel=np.zeros((n, 3), f), spin=np.zeros((n, 3), f), hull_id=np.full(n, -1, np.int32),
                        mass=np.zeros(n, f), inv_inertia=np.zeros((n, 3), f))


def test_plate_world_more_than_128_colours_matches_oracle(gpu):
    sc = plate_scene()
    g = gpu.GpuWorld(algo=0, iterations=10, order=gpu.ORDER_COLOR)
    o = cpu.OracleWorld(algo=0, iterations=10, order_mode=1)
    g.load_scene(sc)
    o.load_scene(sc)
    statics = sc.is_static.astype(bool)
    for s in range(20):
        g.step(DT)
        o.step(DT)
        gb, ob = g.bodies(), o.bodies()
        for k in ("pos", "quat", "lin", "ang"):
            assert_bit_equal(gb[k], ob[k], f"step {s} {k}")
        assert_manifolds_equal(g.contacts(), o.contacts(), what=f"step {s}")
        order, colors = g.solve_order()
        oorder, ocolors = o.solve_order()
        assert np.array_equal(order, oorder) and np.array_equal(colors, ocolors), f"step {s} colour order"
        assert colors_valid(g.contacts(), colors, statics)
    assert int(g.stats()["color_count"]) == int(o.stats()["color_count"]) > 400


def test_plate_in_batched_engine_matches_oracle(gpu):
    """The same plate as one world of a batch beside two ordinary worlds; each
    world against the oracle every step."""
    sc = [scenes.generate(scenes.BOXES_ON_PLANE, 64, 5), plate_scene(), plate_scene(side=12)]
    batch = gpu.GpuBatch(sc, iterations=10)
    oracles = []
    for s in sc:
        ow = cpu.OracleWorld(algo=0, iterations=10, order_mode=1)
        ow.load_scene(s)
        oracles.append(ow)
    for step in range(15):
        batch.step(DT)
        for ow in oracles:
            ow.step(DT)
        for w, ow in enumerate(oracles):
            pos, rot, lin, ang = batch.world_bodies(w)
            ob = ow.bodies()
            for k, v in (("pos", pos), ("quat", rot), ("lin", lin), ("ang", ang)):
                assert_bit_equal(v, ob[k], f"step {step} world {w} {k}")
            assert_manifolds_equal(batch.contacts(w), ow.contacts(), what=f"step {step} world {w}")
    assert int(batch.stats(1)["color_count"]) == int(oracles[1].stats()["color_count"]) > 400
    assert 128 < int(batch.stats(2)["color_count"]) == int(oracles[2].stats()["color_count"])
