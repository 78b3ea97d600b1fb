"""CPU checks of the FP64 evaluation of the differentiable rollout: its forward
steps equal the oracle's FP64 steps, and its hand-written adjoint matches
central finite differences (eps = 1e-4) of a loss computed through the oracle's
FP64 step, in contact-stable windows, within 1e-3 relative.  Contact-stable
means that no perturbation of the window crosses a discrete event: a contact
appearing or vanishing, a clamp switching, or a penetration crossing the
solver's 5 mm slop (where the position bias has a kink), or a sliding contact
sticking; bodies therefore start embedded 2 cm, slide at 1.5-2.5 m/s, and the
window is 20 steps at dt = 1/120 (8 steps for the impact case, which ends while
the boxes are in the air after bouncing)."""
import numpy as np
import pytest

from oracle import cpu
from phys_gb300 import rollout, scenes

DT = 1 / 120
ITERS = 10
TOL = 1e-3


def contact_scene(kind, impact=False):
    if kind == "boxes":
        sc = scenes.generate(scenes.BOXES_ON_PLANE, 6, 5)
    else:
        sc = scenes.generate(scenes.BOXES_ON_PLANE, 4, 7)
        sc.pos[1:, 1] -= np.float32(0.02)
        # two spheres on the floor, pressed against each other, and a sphere on a box
        extra = scenes.generate(scenes.SPHERES_ON_FLOOR, 3, 1)
        for f in ("shape", "is_static", "dims", "pos", "density", "restitution", "friction", "linvel", "spin",
                  "hull_id", "mass", "inv_inertia"):
            setattr(sc, f, np.concatenate([getattr(sc, f), getattr(extra, f)[1:]]))
        r = sc.dims[-3:, 0]
        sc.pos[-3] = [5.0, r[0] - 0.02, 5.0]
        sc.pos[-2] = [5.0 + r[0] + r[1] - 0.04, r[1] - 0.02, 5.0]
        top = sc.pos[1, 1] + sc.dims[1, 1] / 2
        sc.pos[-1] = [sc.pos[1, 0] + 0.05, top + r[2] - 0.02, sc.pos[1, 2]]
        sc.restitution[-3:] = [0.1, 0.2, 0.25]
    rng = np.random.default_rng(1)
    # sliding fast enough to keep slipping through the window (no stick/slip switch)
    ang = rng.uniform(0, 2 * np.pi, sc.count - 1)
    speed = rng.uniform(1.5, 2.5, sc.count - 1)
    sc.linvel[1:] = np.stack([speed * np.cos(ang), np.zeros_like(ang), speed * np.sin(ang)], 1).astype(np.float32)
    if kind == "boxes":
        sc.pos[1:, 1] -= np.float32(0.02)
    if impact:
        sc.linvel[1:, 1] = np.float32(-2.0)
    return sc


def setup(sc):
    ow = cpu.OracleWorld(fp64=True, algo=0, iterations=ITERS, order_mode=1)
    ow.load_scene(sc)
    b = ow.bodies_f64()
    state = [b["pos"], b["quat"], b["lin"], b["ang"]]
    mat = np.array([ow.material(i) for i in range(sc.count)])
    mass32, iinv, he = rollout.body_properties(sc)
    assert np.array_equal(mass32.astype(np.float64), mat[:, 0])
    return ow, state, mat[:, 0].copy(), mat[:, 1].copy(), mat[:, 2].copy(), iinv, he


def oracle_final(ow, steps):
    w = ow.clone()
    for _ in range(steps):
        w.step(DT)
    b = w.bodies_f64()
    return [b["pos"], b["quat"], b["lin"], b["ang"]]


@pytest.mark.parametrize("kind", ["boxes", "mixed"])
def test_fp64_forward_equals_oracle_fp64(kind):
    sc = contact_scene(kind)
    ow, state, mass, mu, rest, iinv, he = setup(sc)
    out, _ = rollout.fp64_rollout(sc.shape, sc.is_static, he, iinv, state, mass, mu, rest, 40, DT, ITERS)
    ref = oracle_final(ow, 40)
    for a, b in zip(out, ref):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("kind,impact", [("boxes", False), ("boxes", True), ("mixed", False)])
def test_fp64_adjoint_matches_oracle_finite_differences(kind, impact):
    sc = contact_scene(kind, impact)
    # an impact bounces the boxes off the floor: end the window before they land
    steps = 8 if impact else 20
    ow, state, mass, mu, rest, iinv, he = setup(sc)
    rng = np.random.default_rng(2)
    out, _ = rollout.fp64_rollout(sc.shape, sc.is_static, he, iinv, state, mass, mu, rest, steps, DT, ITERS)
    c = [rng.normal(size=o.shape) for o in out]
    _, grads = rollout.fp64_rollout(sc.shape, sc.is_static, he, iinv, state, mass, mu, rest, steps, DT, ITERS,
                                    d_final=c)
    loss = lambda o: sum(float((a * b).sum()) for a, b in zip(c, o))

    def fd(which, i, j=None, eps=1e-4):
        vals = []
        for sgn in (1.0, -1.0):
            w = ow.clone()
            if which in ("x", "v", "w"):
                vec = {"x": state[0], "v": state[2], "w": state[3]}[which][i].copy()
                vec[j] += sgn * eps
                if which == "x":
                    w.set_position_f64(i, vec)
                else:
                    w.set_velocity_f64(i, vec if which == "v" else state[2][i], vec if which == "w" else state[3][i])
            else:
                m, f, r = mass[i], mu[i], rest[i]
                if which == "m":
                    m += sgn * eps
                elif which == "f":
                    f += sgn * eps
                else:
                    r += sgn * eps
                w.set_material(i, m, f, r)
            for _ in range(steps):
                w.step(DT)
            b = w.bodies_f64()
            vals.append(loss([b["pos"], b["quat"], b["lin"], b["ang"]]))
        return (vals[0] - vals[1]) / (2 * eps)

    dx, dq, dv, dw, dm, df, dr = grads
    cases = [("v", 1, 0, dv[1, 0]), ("v", 2, 2, dv[2, 2]), ("v", 3, 1, dv[3, 1]), ("w", 1, 1, dw[1, 1]),
             ("x", 2, 1, dx[2, 1]), ("x", 3, 0, dx[3, 0]), ("m", 1, None, dm[1]), ("m", 4, None, dm[4]),
             ("f", 2, None, df[2]), ("f", 3, None, df[3]), ("r", 3, None, dr[3])]
    if impact:
        # positions of an impacting box sit at the restitution threshold (approach
        # speed -1 m/s) under a 1e-4 perturbation; the impact case checks the
        # restitution, velocity, mass and friction gradients
        cases = [x for x in cases if x[0] != "x"] + [("r", 1, None, dr[1]), ("r", 4, None, dr[4])]
    if kind == "mixed":
        n = sc.count
        cases += [("v", n - 1, 0, dv[n - 1, 0]), ("x", n - 2, 1, dx[n - 2, 1]), ("r", n - 3, None, dr[n - 3]),
                  ("m", n - 2, None, dm[n - 2])]
    scale = max(abs(x[3]) for x in cases)
    for which, i, j, a in cases:
        ref = fd(which, i, j)
        # relative error (a true zero is held to 1e-9 of the largest gradient)
        assert abs(a - ref) <= TOL * max(abs(ref), 1e-6 * scale), (which, i, j, a, ref)
