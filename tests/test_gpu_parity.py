"""GPU parity: the CUDA path through the C ABI against the reference's golden
fixtures and the oracle, bit for bit (integers and floats alike; the device
code mirrors the reference's operation order with contraction off)."""
import numpy as np
import pytest

from helpers import assert_bit_equal, assert_manifolds_equal, colors_valid
from oracle import cpu
from phys_gb300 import scenes

pytestmark = pytest.mark.gpu

WORLD_RUNS = ["spheres_floor_sap", "spheres_floor_grid", "mixed_volume_sap", "mixed_volume_grid", "pyramid_sap",
              "boxes_plane_sap", "mixed_volume_tree"]


def scene_from(g):
    n = len(g["shape"])
    return scenes.Scene(g["shape"], g["is_static"], g["dims"], g["pos"], g["density"], g["restitution"],
                        g["friction"], g["linvel"], g["spin"], np.full(n, -1, np.int32), np.zeros(n, np.float32),
                        np.zeros((n, 3), np.float32))


def compare_worlds(gw, ow, what, features=True):
    gb, ob = gw.bodies(), ow.bodies()
    for k in ("pos", "quat", "lin", "ang"):
        assert_bit_equal(gb[k], ob[k], f"{what} {k}")
    assert_bit_equal(gw.pairs(), ow.pairs(), f"{what} pairs")
    assert_manifolds_equal(gw.contacts(), ow.contacts(), features=features, what=what)


# ------------------------------------------------------------- broadphase ---
@pytest.mark.parametrize("algo", [0, 1])
def test_broadphase_golden(gpu, golden, algo):
    g = golden("broadphase")
    for k in range(int(g["count"])):
        c = g[f"aabb_{k}"]
        pairs, st = gpu.broadphase(c[:, 0], c[:, 1], algo)
        assert_bit_equal(pairs, g[f"pairs_{k}_{algo}"], f"case {k} pairs")
        got = np.array([st["x_window_comparisons"], st["aabb_pairs"], st["grid_comparisons"], st["grid_entries"],
                        st["grid_overflow_aabbs"]], np.uint64)
        assert np.array_equal(got, g[f"stats_{k}_{algo}"]), f"case {k}: {got} != {g[f'stats_{k}_{algo}']}"
        assert st["grid_cell_size"] == g[f"cell_{k}_{algo}"]


@pytest.mark.parametrize("algo", [0, 1])
def test_broadphase_random_large(gpu, algo):
    rng = np.random.default_rng(3)
    for n in (5000, 40000):
        c = rng.uniform(-60, 60, (n, 3)).astype(np.float32)
        h = rng.uniform(0.05, 1.5, (n, 3)).astype(np.float32)
        pairs, st = gpu.broadphase(c - h, c + h, algo)
        ref, rst = cpu.broadphase("oracle", c - h, c + h, algo)
        assert_bit_equal(pairs, ref, f"n={n}")
        assert st["aabb_pairs"] == rst["aabb_pairs"] and st["x_window_comparisons"] == rst["x_window_comparisons"]
        assert st["grid_comparisons"] == rst["grid_comparisons"] and st["grid_entries"] == rst["grid_entries"]


def test_broadphase_fixed_cell_same_pairs(gpu):
    rng = np.random.default_rng(4)
    c = rng.uniform(-30, 30, (20000, 3)).astype(np.float32)
    h = rng.uniform(0.1, 0.6, (20000, 3)).astype(np.float32)
    base, _ = gpu.broadphase(c - h, c + h, 0)
    for cell in (1.2, 2.5, 7.0):
        pairs, st = gpu.broadphase(c - h, c + h, 1, cell)
        assert_bit_equal(pairs, base, f"cell {cell}")
        assert st["grid_cell_size"] == cell


def test_broadphase_tree_rejected(gpu):
    with pytest.raises(ValueError):
        gpu.broadphase(np.zeros((2, 3)), np.ones((2, 3)), 2)


# ------------------------------------------------------------ narrowphase ---
def test_narrowphase_golden(gpu, golden):
    g = golden("narrowphase")
    for k in range(len(g["hits"])):
        args = (g["shapes"][k, 0], g["dims"][k, 0], g["pos"][k, 0], g["quat"][k, 0], g["shapes"][k, 1],
                g["dims"][k, 1], g["pos"][k, 1], g["quat"][k, 1])
        hit, m = gpu.generate_contact(*args)
        assert hit == bool(g["hits"][k]), f"case {k} hit"
        if hit:
            assert_manifolds_equal(np.array([m]), g["manifolds"][k:k + 1], features=False, what=f"case {k}")
            ohit, om = cpu.generate_contact("oracle", *args)
            assert_bit_equal(m["feature"], om["feature"], f"case {k} feature ids")


# ------------------------------------------------------------------ world ---
@pytest.mark.parametrize("run", WORLD_RUNS)
def test_world_manifold_order_matches_reference(gpu, golden, run):
    """In the reference's own manifold order the GPU step equals the reference
    PhysicsWorld::step, bit for bit, over the whole run."""
    g = golden(f"world_{run}")
    w = gpu.GpuWorld(algo=int(g["algo"]), order=gpu.ORDER_MANIFOLD)
    w.load_scene(scene_from(g))
    counts = []
    for _ in range(int(g["steps"])):
        w.step(g["dt"])
        counts.append(len(w.contacts()))
    b = w.bodies()
    for k in ("pos", "quat", "lin", "ang"):
        assert_bit_equal(b[k], g[f"final_{k}"], f"{run} {k}")
    assert_manifolds_equal(w.contacts(), g["contacts"], features=False, what=run)
    assert np.array_equal(np.array(counts, np.uint32), g["contacts_per_step"])
    assert_bit_equal(w.pairs(), g["last_pairs"], f"{run} pairs")
    st, ref = w.stats(), g["stats"][0]
    for f in ("possible_pairs", "candidate_pairs", "contact_count", "solved_contact_count", "x_window_comparisons",
              "aabb_pairs", "grid_comparisons", "grid_entries", "grid_overflow_aabbs", "prepared_points",
              "warm_start_comparisons", "warm_start_matches", "velocity_point_visits"):
        assert st[f] == ref[f], f"{run} {f}: {st[f]} != {ref[f]}"


@pytest.mark.parametrize("kind,n,algo,cell,iters,steps", [
    (scenes.SPHERES_ON_FLOOR, 1000, 0, 0.0, 10, 60),
    (scenes.MIXED_VOLUME, 6000, 1, 2.2, 10, 40),
    (scenes.MIXED_VOLUME, 6000, 0, 0.0, 10, 20),
    (scenes.PYRAMIDS_BOXES_ONLY, 2, 0, 0.0, 20, 40),
    (scenes.BOXES_ON_PLANE, 64, 1, 0.0, 8, 60),
    (scenes.MIXED_VOLUME, 6000, 2, 0.0, 10, 30),
    (scenes.PYRAMIDS_BOXES_ONLY, 2, 2, 0.0, 20, 30),
])
def test_world_color_order_matches_oracle_every_step(gpu, kind, n, algo, cell, iters, steps):
    sc = scenes.generate(kind, n, 42)
    gw = gpu.GpuWorld(algo=algo, cell_size=cell, iterations=iters, order=gpu.ORDER_COLOR)
    ow = cpu.OracleWorld(algo=algo, cell_size=cell, iterations=iters, order_mode=1)
    gw.load_scene(sc)
    ow.load_scene(sc)
    statics = sc.is_static.astype(bool)
    for s in range(steps):
        gw.step(1 / 60)
        ow.step(1 / 60)
        compare_worlds(gw, ow, f"step {s}")
        order, colors = gw.solve_order()
        oorder, ocolors = ow.solve_order()
        assert np.array_equal(order, oorder) and np.array_equal(colors, ocolors), f"step {s} colour order"
        assert colors_valid(gw.contacts(), colors, statics)
    st, ost = gw.stats(), ow.stats()
    for f in ("candidate_pairs", "contact_count", "prepared_points", "warm_start_matches", "np_candidates",
              "np_contacts", "color_count"):
        assert np.array_equal(st[f], ost[f]), f


def test_world_hulls_match_oracle(gpu):
    sc = scenes.generate(scenes.PYRAMIDS, 1, 9)
    # lower the hulls onto the pyramid so they collide within the run
    sc.pos[sc.shape == 2, 1] -= 20.0
    gw = gpu.GpuWorld(iterations=20, order=gpu.ORDER_COLOR)
    ow = cpu.OracleWorld(iterations=20, order_mode=1)
    gw.load_scene(sc)
    ow.load_scene(sc)
    hull_contacts = 0
    for s in range(120):
        gw.step(1 / 60)
        ow.step(1 / 60)
        compare_worlds(gw, ow, f"step {s}")
        hull_contacts += int(gw.stats()["np_contacts"][3])
    assert hull_contacts > 0


# ----------------------------------------------------------------- solver ---
def test_solver_known_answers(gpu, golden):
    g = golden("solver")
    for name in ("offcenter", "restitution"):
        w = gpu.GpuWorld(order=gpu.ORDER_MANIFOLD)
        w.create_body(1, [2, 2, 2], [0, 0, 0], 1.0, 1, 0.0, 0.0)
        h = w.create_body(1, [2, 2, 2], [0, 0, 0], 1.0, 0, float(g[f"{name}_rest"]), 0.0)
        st = w.get_body(gpu.Handle(int(h[0]), int(h[1])))
        st.linear_velocity[:] = [0.0, float(g[f"{name}_vel"]), 0.0]
        w.set_body(gpu.Handle(int(h[0]), int(h[1])), st)
        solved = w.solve(g[f"{name}_in"], 1 / 60)
        b = w.bodies()
        assert_manifolds_equal(solved, g[f"{name}_out"], features=False, what=name)
        assert_bit_equal(b["lin"], g[f"{name}_lin"], name)
        assert_bit_equal(b["ang"], g[f"{name}_ang"], name)


def test_standalone_solve_matches_oracle_with_stale_handles(gpu):
    sc = scenes.generate(scenes.PYRAMIDS_BOXES_ONLY, 1, 42)
    gw = gpu.GpuWorld(order=gpu.ORDER_COLOR)
    ow = cpu.OracleWorld(order_mode=1)
    gw.load_scene(sc)
    ow.load_scene(sc)
    gw.step(1 / 60)
    ow.step(1 / 60)
    cs = ow.contacts().copy()
    cs["normal_impulse"] = 0
    stale = cs[:3].copy()
    stale["body_b_generation"] += 1
    mixed = np.concatenate([stale, cs])
    order, _, _ = ow.color(mixed)
    got = gw.solve(mixed, 1 / 60)
    exp, est = ow.solve(mixed, 1 / 60, 8, order)
    assert_manifolds_equal(got, exp, features=False)
    for k in ("lin", "ang"):
        assert_bit_equal(gw.bodies()[k], ow.bodies()[k], k)
    assert gw.stats()["solved_contact_count"] == est["solved_contact_count"] == len(cs)


# ------------------------------------------------------------- edge cases ---
def test_empty_and_single_body_worlds(gpu):
    w = gpu.GpuWorld()
    w.step(1 / 60)
    assert len(w.contacts()) == 0 and w.stats()["candidate_pairs"] == 0
    h = w.create_body(0, [0.5, 0, 0], [0, 3, 0], 1.0, 0, 0.0, 0.5)
    for _ in range(10):
        w.step(1 / 60)
    o = cpu.OracleWorld()
    o.create_body(0, [0.5, 0, 0], [0, 3, 0], 1.0, 0, 0.0, 0.5)
    for _ in range(10):
        o.step(1 / 60)
    assert_bit_equal(w.bodies()["pos"], o.bodies()["pos"], "free fall")
    assert h[0] == 0


def test_removal_slot_reuse_and_stale_handles(gpu):
    sc = scenes.generate(scenes.SPHERES_ON_FLOOR, 120, 5)
    gw, ow = gpu.GpuWorld(order=gpu.ORDER_COLOR), cpu.OracleWorld(order_mode=1)
    hg, ho = gw.load_scene(sc), ow.load_scene(sc)
    assert np.array_equal(hg, ho)
    for s in range(40):
        gw.step(1 / 60)
        ow.step(1 / 60)
        if s == 10:
            for i in (5, 17, 60):
                gw.remove_body(hg[i, 0], hg[i, 1])
                ow.remove_body(ho[i, 0], ho[i, 1])
        if s == 20:
            a = gw.create_body(1, [0.6, 0.6, 0.6], [0.5, 4.0, 0.2], 1.0, 0, 0.0, 0.5)
            b = ow.create_body(1, [0.6, 0.6, 0.6], [0.5, 4.0, 0.2], 1.0, 0, 0.0, 0.5)
            assert np.array_equal(a, b) and a[1] == 1  # reused slot, bumped generation
        compare_worlds(gw, ow, f"step {s}")
    with pytest.raises(LookupError):
        gw.get_body(gpu.Handle(int(hg[5, 0]), int(hg[5, 1])))


def test_invalid_arguments_and_unsupported(gpu):
    w = gpu.GpuWorld()
    with pytest.raises(ValueError):
        w.create_body(0, [0.001, 0, 0], [0, 0, 0], 1.0, 0, 0, 0)  # Sphere is too small
    with pytest.raises(ValueError):
        w.create_body(1, [1, 1, 1], [0, 0, 0], 50.0, 0, 0, 0)  # Density is out of range
    with pytest.raises(ValueError):
        w.create_body(1, [100, 100, 1], [0, 0, 0], 1.0, 1, 0, 0)  # Box is too large
    with pytest.raises(ValueError):
        gpu.check(w.lib.pe_world_set_worker_counts(w.h, 0, 1, 1))


def test_pair_buffer_growth(gpu):
    """A dense pile overflows the initial pair capacity; the step is re-run
    from the untouched state with larger buffers and still matches."""
    n = 9000
    rng = np.random.default_rng(1)
    sc = scenes.generate(scenes.SPHERES_ON_FLOOR, n, 2)
    sc.pos[1:] = rng.uniform(-5, 5, (n, 3)).astype(np.float32) + np.float32([0, 6, 0])
    gw, ow = gpu.GpuWorld(order=gpu.ORDER_COLOR), cpu.OracleWorld(order_mode=1)
    gw.load_scene(sc)
    ow.load_scene(sc)
    for s in range(3):
        gw.step(1 / 60)
        ow.step(1 / 60)
        compare_worlds(gw, ow, f"step {s}")
    assert gw.stats()["candidate_pairs"] > 65536


def test_one_block_sweep_pair_overflow_reruns(gpu):
    """A world small enough for the one-block sweep whose raw pairs outgrow the
    sweep's own finalize (more than 8,192): the step is re-run with the
    separate finalize and still matches, step after step."""
    n = 2000
    rng = np.random.default_rng(3)
    sc = scenes.generate(scenes.SPHERES_ON_FLOOR, n, 5)
    sc.pos[1:] = (rng.uniform(-6, 6, (n, 3)) * np.float32([1, 0.25, 1])).astype(np.float32) + np.float32([0, 4, 0])
    gw, ow = gpu.GpuWorld(order=gpu.ORDER_COLOR), cpu.OracleWorld(order_mode=1)
    gw.load_scene(sc)
    ow.load_scene(sc)
    for s in range(3):
        gw.step(1 / 60)
        ow.step(1 / 60)
        compare_worlds(gw, ow, f"step {s}")
    assert gw.stats()["candidate_pairs"] > 8192


def test_world_read_poses_matches_bodies(gpu):
    """read_poses (positions packed on the device, rotations copied as they
    are) returns the state pe_world_read_bodies reports, and forces written
    through write_forces reach dynamic bodies only."""
    sc = scenes.generate(scenes.SPHERES_ON_FLOOR, 60, 3)
    gw = gpu.GpuWorld(order=gpu.ORDER_COLOR)
    gw.load_scene(sc)
    rng = np.random.default_rng(4)
    for _ in range(5):
        gw.write_forces(rng.normal(size=(sc.count, 3)).astype(np.float32) * 20)
        gw.step(1 / 60)
    pos = np.zeros((sc.count, 3), np.float32)
    rot = np.zeros((sc.count, 4), np.float32)
    gw.read_poses(pos, rot)
    b = gw.bodies()
    assert_bit_equal(pos, b["pos"], "read_poses positions")
    assert_bit_equal(rot, b["quat"], "read_poses rotations")
    static = sc.is_static.astype(bool)
    assert np.all(b["lin"][static] == 0)


# ------------------------------------------------------- sleeping islands ---
def _sleep_names():
    import sleep_scenarios as ss

    return list(ss.all_scenarios())


@pytest.mark.parametrize("name", _sleep_names())
def test_sleeping_scenarios_match_oracle(gpu, name):
    """Sleeping scenarios (settle, wake by every mutator, collisions, support
    and property changes, quiet-time thresholds, the 512-box profile scene) and
    multi-collider bodies: GPU graph-colour order against the oracle in the same
    order, bit for bit."""
    import sleep_scenarios as ss
    from test_oracle import assert_observations_equal

    ops, dt = ss.all_scenarios()[name]
    got = ss.run(gpu.GpuWorld(), ops, dt)
    want = ss.run(cpu.OracleWorld(order_mode=1), ops, dt)
    assert_observations_equal(got, want, name, features=True)


@pytest.mark.parametrize("name", ["opt_in", "mutator_0", "collision_wake", "remove_floor_collider", "stacks_512",
                                  "compound_drop", "compound_remove_collider"])
def test_sleeping_manifold_order_matches_reference(gpu, golden, name):
    """The GPU in the reference's manifold order against the reference's own
    observations (tests/golden/sleeping.npz)."""
    import sleep_scenarios as ss
    from test_oracle import _sleeping_golden, assert_observations_equal

    ops, dt = ss.all_scenarios()[name]
    got = ss.run(gpu.GpuWorld(order=gpu.ORDER_MANIFOLD), ops, dt)
    assert_observations_equal(got, _sleeping_golden(golden, name), name)


@pytest.mark.parametrize("algo,graphs", [(1, True), (0, False), (2, True)])
def test_sleeping_grid_and_direct_launches(gpu, algo, graphs):
    import sleep_scenarios as ss
    from test_oracle import assert_observations_equal

    for name in ("mutator_0", "replace_lower", "boxes_on_plane", "compound_drop"):
        ops, dt = ss.all_scenarios()[name]
        g = gpu.GpuWorld(algo=algo)
        g.set_graphs(graphs)
        assert_observations_equal(ss.run(g, ops, dt), ss.run(cpu.OracleWorld(algo=algo, order_mode=1), ops, dt),
                                  f"{name} algo {algo}", features=True)


def test_sleeping_write_forces_wakes(gpu):
    """Bulk forces wake their bodies like applyForce; zero forces do not."""
    import sleep_scenarios as ss

    ops, dt = ss.all_scenarios()["mutator_0"]
    g = gpu.GpuWorld()
    o = cpu.OracleWorld(order_mode=1)
    ss.run(g, ops[:-6], dt)
    ss.run(o, ops[:-6], dt)
    f = np.zeros((g.body_count(), 3), np.float32)
    g.write_forces(f)
    g.step(dt)
    o.step(dt)
    assert g.sleeping().tolist() == o.sleeping().tolist() == [False, True, True, True]
    f[ss.UPPER] = [0.1, 0, 0]
    g.write_forces(f)
    o.apply_force(ss.UPPER, f[ss.UPPER])
    assert not g.sleeping()[ss.UPPER]
    for _ in range(3):
        g.step(dt)
        o.step(dt)
    for k in ("pos", "quat", "lin", "ang"):
        assert_bit_equal(g.bodies()[k], o.bodies()[k], k)
    assert g.sleeping().tolist() == o.sleeping().tolist()


# ------------------------------------------------------------- world copy ---
def test_world_clone_is_independent_and_continues(gpu):
    """PhysicsWorld's copy constructor (physics_world.cpp:74-93): the copy
    carries bodies, contacts and the warm-start cache, so stepping it continues
    the original's trajectory bit for bit; editing or stepping one leaves the
    other unchanged."""
    sc = scenes.generate(scenes.MIXED_VOLUME, 3000, 9)
    g = gpu.GpuWorld(algo=1, iterations=10)
    o = cpu.OracleWorld(algo=1, iterations=10, order_mode=1)
    hg = g.load_scene(sc)
    o.load_scene(sc)
    for _ in range(30):
        g.step(1 / 60)
        o.step(1 / 60)
    c = g.clone()
    oc = o.clone()
    compare_worlds(c, o, "fresh copy")
    assert c.stats()["contact_count"] == g.stats()["contact_count"]
    for _ in range(20):
        g.step(1 / 60)
        o.step(1 / 60)
    compare_worlds(g, o, "original after 20 steps")
    compare_worlds(c, oc, "copy not stepped")
    for _ in range(20):
        c.step(1 / 60)
        oc.step(1 / 60)
    compare_worlds(c, o, "copy after 20 steps (warm-start cache carried)")
    c.remove_body(int(hg[5, 0]), int(hg[5, 1]))
    oc.remove_body(int(hg[5, 0]), int(hg[5, 1]))
    c.step(1 / 60)
    oc.step(1 / 60)
    g.step(1 / 60)
    o.step(1 / 60)
    compare_worlds(g, o, "original after the copy's edit")
    gb, ob = c.bodies(), oc.bodies()
    for k in gb:
        gb[k][5] = ob[k][5] = 0
        assert_bit_equal(gb[k], ob[k], f"edited copy {k}")
    assert_manifolds_equal(c.contacts(), oc.contacts(), what="edited copy")


def test_world_clone_sleeping_state(gpu):
    """Copies own independent sleeping state (sleeping_tests.cpp:330-343)."""
    import sleep_scenarios as ss

    ops, dt = ss.all_scenarios()["mutator_0"]
    g = gpu.GpuWorld()
    o = cpu.OracleWorld(order_mode=1)
    hg = ss.run(g, ops[:-6], dt)
    ss.run(o, ops[:-6], dt)
    c = g.clone()
    oc = o.clone()
    assert c.sleeping().tolist() == [False, True, True, True]
    c.wake_up(gpu.Handle(ss.UPPER, 0))
    oc.wake_body(ss.UPPER)
    for w in (c, oc, g, o):
        w.step(dt)
    assert c.sleeping().tolist() == oc.sleeping().tolist() == [False, False, False, True]
    assert g.sleeping().tolist() == [False, True, True, True]
    for k in ("pos", "quat", "lin", "ang"):
        assert_bit_equal(c.bodies()[k], oc.bodies()[k], k)
    assert c.stats()["solved_contact_count"] == oc.stats()["solved_contact_count"] == 2



# ------------------------------------------------------------ tree selector ---
def test_tree_pairs_equal_sweep_on_large_and_degenerate_sets(gpu):
    """The linear-BVH tree reports exactly the sweep-and-prune pair set: the
    100k-body workload, a pile of coincident spheres (equal Morton codes, ties
    broken by index), and worlds of zero, one and two bodies."""
    sc = scenes.generate(scenes.MIXED_VOLUME, 100_000, 42)
    worlds = {}
    for algo in (0, 2):
        w = gpu.GpuWorld(algo=algo, iterations=10)
        w.load_scene(sc)
        for _ in range(3):
            w.step(1 / 60)
        worlds[algo] = w
    assert len(worlds[0].pairs()) > 1000
    assert_bit_equal(worlds[2].pairs(), worlds[0].pairs(), "100k pairs")
    for k in ("pos", "quat", "lin", "ang"):
        assert_bit_equal(worlds[2].bodies()[k], worlds[0].bodies()[k], f"100k {k}")
    assert worlds[2].stats()["aabb_pairs"] == worlds[0].stats()["aabb_pairs"]
    assert worlds[2].stats()["x_window_comparisons"] == 0
    for n in (0, 1, 2, 64):
        g = gpu.GpuWorld(algo=2)
        o = cpu.OracleWorld(algo=2, order_mode=1)
        for i in range(n):
            for w in (g, o):
                w.create_body(0, [0.5, 0, 0], [0.0, 2.0 + 0.001 * (i % 3), 0.0], 1.0, 0, 0.0, 0.5)
        for _ in range(3):
            g.step(1 / 60)
            o.step(1 / 60)
        assert len(g.pairs()) == (n * (n - 1)) // 2 or n > 2
        compare_worlds(g, o, f"{n} coincident spheres")


@pytest.mark.parametrize("sleeping", [False, True])
def test_large_contact_counts_multikernel_solver(gpu, sleeping):
    """More than 4096 manifolds take the multi-kernel solver (cooperative
    colouring and sweeps, cache rebuilt in manifold order for one collider per
    body): 16 copies of the 512-box stack scene against the oracle, every step."""
    sc = scenes.box_stacks(4, 4)
    g = gpu.GpuWorld(algo=0, iterations=8)
    o = cpu.OracleWorld(algo=0, iterations=8, order_mode=1)
    for w in (g, o):
        w.set_sleeping_enabled(sleeping)
        w.load_scene(sc)
    for s in range(25):
        g.step(1 / 120)
        o.step(1 / 120)
        if s % 6 == 0 or s == 24:
            compare_worlds(g, o, f"step {s}")
    assert g.stats()["contact_count"] > 4096
    for f in ("solved_contact_count", "prepared_points", "warm_start_matches", "awake_body_count"):
        assert g.stats()[f] == o.stats()[f], f


def test_reference_benchmark_scene_matches_oracle(gpu):
    """The reference's own benchmark scene (mixed field over a floor, SAP,
    8 iterations, 120 Hz) against the oracle in colour order, every 10 steps."""
    sc = scenes.mixed_field(2000, 42)
    g = gpu.GpuWorld(algo=0, iterations=8)
    o = cpu.OracleWorld(algo=0, iterations=8, order_mode=1)
    g.load_scene(sc)
    o.load_scene(sc)
    for s in range(60):
        g.step(1 / 120)
        o.step(1 / 120)
        if s % 10 == 9:
            compare_worlds(g, o, f"step {s}")
    assert g.stats()["contact_count"] > 1000


def island_mix_scene(patch: int, patches: int, plate: bool = False):
    """A static floor with islands of the sizes the island sweeps tell apart:
    `patches` patches of patch x patch touching unit boxes (a 30 x 30 patch is
    one island of thousands of manifolds, a 10 x 10 one of 442), rows of 20
    and of 12 touching spheres (islands of 39 and 23 manifolds) and two-high
    box stacks (islands of two); with `plate`, a dynamic 8 x 0.5 x 8 plate
    carrying 64 spheres (a body with 65 manifolds)."""
    f = np.float32
    pos, shape, dims = [[0.0, -0.5, 0.0]], [1], [[64.0, 1.0, 64.0]]
    for p in range(patches):
        x0, z0 = f(-31.0) + f(11.0) * f(p % 4), f(-31.0) + f(11.0) * f(p // 4)
        for i in range(patch):
            for k in range(patch):
                pos.append([x0 + f(0.999) * f(i), 0.5, z0 + f(0.999) * f(k)])
                shape.append(1)
                dims.append([1.0, 1.0, 1.0])
    for row, count in enumerate([20] * 6 + [12] * 6):
        z0 = f(-31.0) if count == 20 else f(-8.0)
        for i in range(count):
            pos.append([f(16.0) + f(2.5) * f(row % 6), 0.499, z0 + f(0.998) * f(i)])
            shape.append(0)
            dims.append([0.5, 0.0, 0.0])
    for i in range(10):
        for level in range(2):
            pos.append([f(-31.0) + f(2.0) * f(i), f(0.5) + f(1.0) * f(level), 20.0])
            shape.append(1)
            dims.append([1.0, 1.0, 1.0])
    if plate:
        pos.append([20.0, 0.249, 14.0])
        shape.append(1)
        dims.append([8.0, 0.5, 8.0])
        for i in range(8):
            for k in range(8):
                pos.append([f(16.5) + f(i), 0.998, f(10.5) + f(k)])
                shape.append(0)
                dims.append([0.5, 0.0, 0.0])
    n = len(pos)
    static = np.zeros(n, np.uint8)
    static[0] = 1
    return scenes.Scene(shape=np.array(shape, np.uint8), is_static=static, dims=np.array(dims, f),
                        pos=np.array(pos, f), density=np.ones(n, f), restitution=np.zeros(n, f),
                        friction=np.full(n, f(0.5)), linvel=np.zeros((n, 3), f), spin=np.zeros((n, 3), f),
                        hull_id=np.full(n, -1, np.int32), mass=np.zeros(n, f), inv_inertia=np.zeros((n, 3), f))


@pytest.mark.parametrize("patch,patches,plate", [(30, 1, False), (10, 12, False), (10, 12, True)])
def test_island_sizes_match_oracle(gpu, patch, patches, plate):
    """Islands of two manifolds to thousands against the oracle in colour
    order: one island of thousands (every island in grid-wide sweeps), or
    twelve of 442 with smaller ones (per-warp and per-thread sweeps); a body
    with more manifolds than the colouring's per-body lists hold (colouring
    in rounds)."""
    sc = island_mix_scene(patch, patches, plate)
    g = gpu.GpuWorld(algo=0, iterations=8)
    o = cpu.OracleWorld(algo=0, iterations=8, order_mode=1)
    g.load_scene(sc)
    o.load_scene(sc)
    for s in range(12):
        g.step(1 / 120)
        o.step(1 / 120)
        if s % 4 == 3:
            compare_worlds(g, o, f"step {s}")
    assert g.stats()["solved_contact_count"] > 4096


def box_pile(nx: int):
    """nx x nx touching unit boxes (0.999 m apart) on a floor of 60 x 1 x 60
    static tiles: one island of about 5 nx^2 manifolds."""
    f = np.float32
    pos, shape, dims = [], [], []
    tiles = (nx + 59) // 60
    for tx in range(tiles):
        for tz in range(tiles):
            pos.append([f(60.0) * f(tx) - f(0.5), -0.5, f(60.0) * f(tz) - f(0.5)])
            shape.append(1)
            dims.append([60.0, 1.0, 60.0])
    n_static = len(pos)
    g = np.arange(nx, dtype=f)
    xs, zs = np.meshgrid(f(0.999) * g, f(0.999) * g, indexing="ij")
    for x, z in zip(xs.ravel(), zs.ravel()):
        pos.append([x, 0.5, z])
        shape.append(1)
        dims.append([1.0, 1.0, 1.0])
    n = len(pos)
    static = np.zeros(n, np.uint8)
    static[:n_static] = 1
    return scenes.Scene(shape=np.array(shape, np.uint8), is_static=static, dims=np.array(dims, f),
                        pos=np.array(pos, f), density=np.ones(n, f), restitution=np.zeros(n, f),
                        friction=np.full(n, f(0.5)), linvel=np.zeros((n, 3), f), spin=np.zeros((n, 3), f),
                        hull_id=np.full(n, -1, np.int32), mass=np.zeros(n, f), inv_inertia=np.zeros((n, 3), f))


def test_grid_wide_island_sweeps_match_oracle(gpu):
    """A pile of 57,600 boxes (about 270,000 manifolds, one island) through
    the grid-wide sweeps against the oracle in colour order."""
    sc = box_pile(240)
    g = gpu.GpuWorld(algo=0, iterations=8)
    o = cpu.OracleWorld(algo=0, iterations=8, order_mode=1)
    g.load_scene(sc)
    o.load_scene(sc)
    for s in range(3):
        g.step(1 / 120)
        o.step(1 / 120)
    compare_worlds(g, o, "step 2")
    assert int(g.stats()["solved_contact_count"]) > 250_000


def test_step_io_equals_separate_calls(gpu):
    """pe_world_step_io = write_forces + step + read_poses, bit for bit."""
    sc = scenes.generate(scenes.MIXED_VOLUME, 5000, 3)
    a = gpu.GpuWorld(algo=1, cell_size=2.2, iterations=10)
    b = gpu.GpuWorld(algo=1, cell_size=2.2, iterations=10)
    a.load_scene(sc)
    b.load_scene(sc)
    rng = np.random.default_rng(1)
    n = sc.count
    for s in range(12):
        f = rng.normal(size=(n, 3)).astype(np.float32) * (s % 3)
        pa, qa = np.zeros((n, 3), np.float32), np.zeros((n, 4), np.float32)
        pb, qb = np.zeros((n, 3), np.float32), np.zeros((n, 4), np.float32)
        a.step_io(1 / 60, f, pa, qa)
        b.write_forces(f)
        b.step(1 / 60)
        b.read_poses(pb, qb)
        assert_bit_equal(pa, pb, f"step {s} positions")
        assert_bit_equal(qa, qb, f"step {s} rotations")
    compare_worlds(a, b, "after step_io")


def test_step_io_in_place_with_pinned_arrays(gpu):
    """With pinned host arrays the step reads the forces and writes the poses in
    place (the pose kernel writes the caller's memory through the step's I/O
    descriptor, no copy operations); the results equal separate calls bit for
    bit, also on steps where one array is pageable or the rotation array is not
    16-byte aligned (those go through copies)."""
    torch = pytest.importorskip("torch")
    sc = scenes.generate(scenes.MIXED_VOLUME, 5000, 3)
    a = gpu.GpuWorld(algo=1, cell_size=2.2, iterations=10)
    b = gpu.GpuWorld(algo=1, cell_size=2.2, iterations=10)
    a.load_scene(sc)
    b.load_scene(sc)
    rng = np.random.default_rng(2)
    n = sc.count

    def pinned(count):
        return torch.zeros(count, dtype=torch.float32).pin_memory().numpy()

    for s in range(10):
        f = pinned(3 * n).reshape(n, 3)
        f[:] = rng.normal(size=(n, 3)).astype(np.float32) * (s % 3)
        pa = pinned(3 * n).reshape(n, 3)
        qa = pinned(4 * n).reshape(n, 4)
        if s == 4:
            pa = np.zeros((n, 3), np.float32)  # pageable: this step copies
        if s == 6:
            qa = pinned(4 * n + 1)[1:].reshape(n, 4)  # 4 bytes off 16-byte alignment
        pb, qb = np.zeros((n, 3), np.float32), np.zeros((n, 4), np.float32)
        a.step_io(1 / 60, f, pa, qa)
        b.write_forces(np.array(f))
        b.step(1 / 60)
        b.read_poses(pb, qb)
        assert_bit_equal(np.array(pa), pb, f"step {s} positions")
        assert_bit_equal(np.array(qa), qb, f"step {s} rotations")
    compare_worlds(a, b, "after in-place step_io")


# ------------------------------------------- benchmarked configurations ---
def _bench_cell(sc):
    """The benchmark's grid cell: 2 x the largest collider extent (sphere
    radius, box half diagonal)."""
    sph = sc.shape == 0
    ext = np.where(sph, sc.dims[:, 0], np.linalg.norm(sc.dims * 0.5, axis=1))
    return float(2.0 * ext.max())


def _run_pair(gw, ow, steps, dt, check, statics=None):
    for s in range(steps):
        gw.step(dt)
        ow.step(dt)
        if check(s):
            compare_worlds(gw, ow, f"step {s}")
            order, colors = gw.solve_order()
            oorder, ocolors = ow.solve_order()
            assert np.array_equal(order, oorder) and np.array_equal(colors, ocolors), f"step {s} colour order"
            if statics is not None:
                assert colors_valid(gw.contacts(), colors, statics)
            st, ost = gw.stats(), ow.stats()
            for f in ("candidate_pairs", "contact_count", "prepared_points", "warm_start_matches", "np_candidates",
                      "np_contacts", "color_count", "x_window_comparisons", "grid_comparisons"):
                assert np.array_equal(st[f], ost[f]), f"step {s} {f}: {st[f]} != {ost[f]}"


def test_mixed_100k_bench_config_matches_oracle(gpu):
    """The benchmark world itself: 100,000 spheres and boxes, the bench's grid
    cell (2 x the largest extent), 10 iterations, dt 1/60, against the oracle
    in colour order: every one of the first 5 steps, then every 10th step up
    to step 60 (pairs, manifolds with feature ids, poses, colour order,
    counters)."""
    import os

    sc = scenes.generate(scenes.MIXED_VOLUME, 100_000, 42)
    cell = _bench_cell(sc)
    assert abs(cell - 2.055892) < 1e-5
    gw = gpu.GpuWorld(algo=1, cell_size=cell, iterations=10, order=gpu.ORDER_COLOR)
    ow = cpu.OracleWorld(algo=1, cell_size=cell, iterations=10, order_mode=1, threads=os.cpu_count() or 1)
    gw.load_scene(sc)
    ow.load_scene(sc)
    _run_pair(gw, ow, 60, 1 / 60, lambda s: s < 5 or s % 10 == 9, sc.is_static.astype(bool))
    assert gw.stats()["contact_count"] > 200


def test_spheres_1000_all_300_steps_match_oracle(gpu):
    """Config 1 in full: 1,000 spheres dropped on a static floor, SAP, 10
    iterations, 300 steps at dt 1/60, every step against the oracle."""
    sc = scenes.generate(scenes.SPHERES_ON_FLOOR, 1000, 42)
    gw = gpu.GpuWorld(algo=0, iterations=10, order=gpu.ORDER_COLOR)
    ow = cpu.OracleWorld(algo=0, iterations=10, order_mode=1)
    gw.load_scene(sc)
    ow.load_scene(sc)
    _run_pair(gw, ow, 300, 1 / 60, lambda s: True, sc.is_static.astype(bool))
    assert gw.stats()["contact_count"] > 500


def _lowered_pyramids(per_side, drop):
    sc = scenes.generate(scenes.PYRAMIDS, per_side, 42)
    sc.pos[sc.shape == 2, 1] -= np.float32(drop)
    return sc


def test_stacking_convex_16_pyramids_match_oracle(gpu):
    """Config 3 at 16 pyramids (3,360 boxes) with the proportional 1,250
    hulls, lowered 28 m so that they reach the pyramids and the floor within
    the run (GJK/EPA contacts, deep first contacts included), 20 iterations
    with warm start, 40 steps against the oracle in colour order."""
    import os

    sc = _lowered_pyramids(4, 28.0)
    assert int((sc.shape == 2).sum()) == 1250
    gw = gpu.GpuWorld(algo=0, iterations=20, order=gpu.ORDER_COLOR)
    ow = cpu.OracleWorld(algo=0, iterations=20, order_mode=1, threads=os.cpu_count() or 1)
    gw.load_scene(sc)
    ow.load_scene(sc)
    hull_contacts = 0
    for s in range(40):
        gw.step(1 / 60)
        ow.step(1 / 60)
        hull_contacts += int(gw.stats()["np_contacts"][3])
        if s < 3 or s % 8 == 7:
            compare_worlds(gw, ow, f"step {s}")
            assert np.array_equal(gw.solve_order()[1], ow.solve_order()[1]), f"step {s} colours"
    assert hull_contacts > 100
    for f in ("contact_count", "prepared_points", "warm_start_matches", "np_contacts", "color_count"):
        assert np.array_equal(gw.stats()[f], ow.stats()[f]), f


def test_stacking_convex_full_config_matches_oracle(gpu):
    """Config 3 at its full size: 256 pyramids (53,760 boxes) and 20,000
    hulls, 20 iterations, the first 3 steps against the oracle in colour
    order (about 130,000 manifolds a step)."""
    import os

    sc = scenes.generate(scenes.PYRAMIDS, 16, 42)
    assert int((sc.shape == 1).sum() - sc.is_static.sum()) == 53_760 and int((sc.shape == 2).sum()) == 20_000
    gw = gpu.GpuWorld(algo=0, iterations=20, order=gpu.ORDER_COLOR)
    ow = cpu.OracleWorld(algo=0, iterations=20, order_mode=1, threads=os.cpu_count() or 1)
    gw.load_scene(sc)
    ow.load_scene(sc)
    _run_pair(gw, ow, 3, 1 / 60, lambda s: s == 0 or s == 2)
    assert gw.stats()["contact_count"] > 100_000
