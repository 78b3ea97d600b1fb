"""GPU tests of the differentiable rollout: the forward pass equals the batched
engine bit for bit; the FP32 adjoint matches the FP64 CPU adjoint within 1e-3
relative (entries below a millionth of the largest gradient, true zeros, are
held to 1e-9 of it); the torch.autograd.Function harness gives the gradients of
a centre-of-mass loss — initial velocities, masses, frictions and, on worlds
with impacts, restitutions — that match central finite differences through the
oracle's FP64 step within 1e-3 relative.  (Measured: at most 2.2e-4 against the
FP64 adjoint, at most 1e-5 against finite differences.)"""
import numpy as np
import pytest

from helpers import assert_bit_equal
from oracle import cpu
from phys_gb300 import rollout, scenes

pytestmark = pytest.mark.gpu

DT = 1 / 120
ITERS = 10


def sliding_boxes(n, seed, embed=0.02, impact=False):
    sc = scenes.generate(scenes.BOXES_ON_PLANE, n, seed)
    rng = np.random.default_rng(seed)
    ang = rng.uniform(0, 2 * np.pi, n)
    speed = rng.uniform(1.5, 2.5, n)
    sc.linvel[1:] = np.stack([speed * np.cos(ang), np.zeros(n), speed * np.sin(ang)], 1).astype(np.float32)
    sc.pos[1:, 1] -= np.float32(embed)
    if impact:
        sc.linvel[1:, 1] = np.float32(-2.0)
    return sc


def mixed_world(seed):
    sc = sliding_boxes(4, seed)
    extra = scenes.generate(scenes.SPHERES_ON_FLOOR, 3, seed)
    for f in ("shape", "is_static", "dims", "pos", "density", "restitution", "friction", "linvel", "spin", "hull_id",
              "mass", "inv_inertia"):
        setattr(sc, f, np.concatenate([getattr(sc, f), getattr(extra, f)[1:]]))
    r = sc.dims[-3:, 0]
    sc.pos[-3] = [5.0, r[0] - 0.02, 5.0]
    sc.pos[-2] = [5.0 + r[0] + r[1] - 0.04, r[1] - 0.02, 5.0]
    sc.linvel[-3:] = 0
    sc.linvel[-1] = [0.5, 0.0, 0.0]
    sc.pos[-1] = [-5.0, r[2] - 0.02, -5.0]
    sc.restitution[-3:] = [0.1, 0.2, 0.25]
    return sc


def torch_state(roll):
    import torch

    x0, q0, v0, w0 = roll.initial_state()
    t = lambda a: torch.tensor(a, device="cuda:0")
    return t(x0), t(q0), t(v0), t(w0), t(roll.mass), t(roll.friction), t(roll.restitution)


def test_rollout_forward_matches_batch_engine(gpu):
    sc = [sliding_boxes(6, 1), mixed_world(2), scenes.generate(scenes.MIXED_VOLUME, 40, 3)]
    steps = 30
    roll = rollout.GpuRollout(sc, steps, DT, iterations=ITERS, checkpoint_every=7)
    outs = roll.forward(*torch_state(roll))
    batch = gpu.GpuBatch(sc, iterations=ITERS)
    batch.step(DT, steps)
    ref = batch.bodies()
    for k, (o, r) in enumerate(zip(outs, ref)):
        assert_bit_equal(o.cpu().numpy(), r, f"state {k}")


def test_rollout_gradients_match_fp64_adjoint(gpu):
    import torch

    sc = [sliding_boxes(6, 1), mixed_world(2), sliding_boxes(5, 4, impact=True)]
    steps = [20, 20, 8]
    rng = np.random.default_rng(5)
    for w, s in enumerate(sc):
        roll = rollout.GpuRollout([s], steps[w], DT, iterations=ITERS, checkpoint_every=6)
        state = torch_state(roll)
        outs = roll.forward(*state)
        d = [rng.normal(size=tuple(o.shape)).astype(np.float32) for o in outs]
        grads = roll.backward(*[torch.tensor(a, device="cuda:0") for a in d])
        mass32, iinv, he = rollout.body_properties(s)
        x0, q0, v0, w0 = roll.initial_state()
        _, ref = rollout.fp64_rollout(s.shape, s.is_static, he, iinv, [x0, q0, v0, w0], roll.mass, roll.friction,
                                      roll.restitution, steps[w], DT, ITERS, d_final=d)
        dyn = ~s.is_static.astype(bool)
        for name, g, r in zip(("x0", "q0", "v0", "w0", "mass", "friction", "restitution"), grads, ref):
            g = g.cpu().numpy()[dyn]
            r = r[dyn]
            scale = np.abs(r).max()
            if scale == 0:
                assert np.abs(g).max() < 1e-5, (w, name)
                continue
            err = np.abs(g - r) / np.maximum(np.abs(r), 1e-6 * scale)
            assert err.max() <= 1e-3, (w, name, float(err.max()), g.ravel()[:6], r.ravel()[:6])


def test_rollout_autograd_com_loss_matches_oracle_fd(gpu):
    import torch

    # boxes (half extents U[0.2,0.5], friction U[0.2,0.8], restitution U[0,0.3])
    # on a plane, sliding, two worlds; loss = |COM_final - target|^2
    sc = [sliding_boxes(8, 11), sliding_boxes(8, 12)]
    steps = 24
    roll = rollout.GpuRollout(sc, steps, DT, iterations=ITERS, checkpoint_every=10)
    fn = rollout.rollout_function()
    x0, q0, v0, w0, m, f, r = (t.requires_grad_(True) for t in torch_state(roll))
    xT, qT, vT, wT = fn.apply(roll, x0, q0, v0, w0, m, f, r)
    target = torch.tensor([[1.0, 0.5, -2.0], [-3.0, 0.2, 1.0]], device="cuda:0")
    loss = 0
    dyn = torch.tensor(~np.concatenate([s.is_static for s in sc]).astype(bool), device="cuda:0")
    for w in range(2):
        s0, s1 = int(roll.starts[w]), int(roll.starts[w + 1])
        mw = m[s0:s1] * dyn[s0:s1]
        com = (mw[:, None] * xT[s0:s1]).sum(0) / mw.sum()
        loss = loss + ((com - target[w]) ** 2).sum()
    loss.backward()

    def oracle_loss(w, which, i, j, eps):
        s = sc[w]
        ow = cpu.OracleWorld(fp64=True, algo=0, iterations=ITERS, order_mode=1)
        ow.load_scene(s)
        mat = np.array([ow.material(k) for k in range(s.count)])
        if which == "v":
            b = ow.bodies_f64()
            v = b["lin"][i].copy()
            v[j] += eps
            ow.set_velocity_f64(i, v, b["ang"][i])
        elif which in ("m", "f", "r"):
            mm, ff, rr = mat[i]
            mm, ff, rr = mm + eps * (which == "m"), ff + eps * (which == "f"), rr + eps * (which == "r")
            ow.set_material(i, mm, ff, rr)
            mat[i] = (mm, ff, rr)
        for _ in range(steps):
            ow.step(DT)
        x = ow.bodies_f64()["pos"]
        mw = mat[:, 0] * (~s.is_static.astype(bool))
        com = (mw[:, None] * x).sum(0) / mw.sum()
        return float(((com - target[w].cpu().numpy().astype(np.float64)) ** 2).sum())

    def fd(w, which, i, j=0, eps=1e-4):
        return (oracle_loss(w, which, i, j, eps) - oracle_loss(w, which, i, j, -eps)) / (2 * eps)

    gv, gm, gf, gr = v0.grad.cpu().numpy(), m.grad.cpu().numpy(), f.grad.cpu().numpy(), r.grad.cpu().numpy()
    checks = []
    for w in range(2):
        base = int(roll.starts[w])
        for i in (1, 3, 6):
            checks += [(w, "v", i, 0, gv[base + i, 0]), (w, "v", i, 2, gv[base + i, 2]),
                       (w, "m", i, 0, gm[base + i]), (w, "f", i, 0, gf[base + i])]
    scale = max(abs(c[4]) for c in checks)
    for w, which, i, j, a in checks:
        ref = fd(w, which, i, j)
        assert abs(a - ref) <= 1e-3 * max(abs(ref), 1e-6 * scale), (w, which, i, j, a, ref)


def com_loss_and_oracle(sc, steps, roll, target):
    """Centre-of-mass loss of every world through the autograd harness, and the
    same loss of one world through the oracle's FP64 step with one input
    perturbed (velocity component j of body i, or its mass / friction /
    restitution)."""
    import torch

    fn = rollout.rollout_function()
    x0, q0, v0, w0, m, f, r = (t.requires_grad_(True) for t in torch_state(roll))
    xT, qT, vT, wT = fn.apply(roll, x0, q0, v0, w0, m, f, r)
    dyn = torch.tensor(~np.concatenate([s.is_static for s in sc]).astype(bool), device="cuda:0")
    loss = 0
    for w in range(len(sc)):
        s0, s1 = int(roll.starts[w]), int(roll.starts[w + 1])
        mw = m[s0:s1] * dyn[s0:s1]
        com = (mw[:, None] * xT[s0:s1]).sum(0) / mw.sum()
        loss = loss + ((com - target[w]) ** 2).sum()
    loss.backward()

    def oracle_loss(w, which, i, j, eps):
        s = sc[w]
        ow = cpu.OracleWorld(fp64=True, algo=0, iterations=ITERS, order_mode=1)
        ow.load_scene(s)
        mat = np.array([ow.material(k) for k in range(s.count)])
        if which == "v":
            b = ow.bodies_f64()
            v = b["lin"][i].copy()
            v[j] += eps
            ow.set_velocity_f64(i, v, b["ang"][i])
        else:
            mm, ff, rr = mat[i]
            mm, ff, rr = mm + eps * (which == "m"), ff + eps * (which == "f"), rr + eps * (which == "r")
            ow.set_material(i, mm, ff, rr)
            mat[i] = (mm, ff, rr)
        for _ in range(steps):
            ow.step(DT)
        x = ow.bodies_f64()["pos"]
        mw = mat[:, 0] * (~s.is_static.astype(bool))
        com = (mw[:, None] * x).sum(0) / mw.sum()
        return float(((com - target[w].cpu().numpy().astype(np.float64)) ** 2).sum())

    grads = {"v": v0.grad.cpu().numpy(), "m": m.grad.cpu().numpy(), "f": f.grad.cpu().numpy(),
             "r": r.grad.cpu().numpy()}
    return grads, oracle_loss


def test_rollout_autograd_restitution_matches_oracle_fd(gpu):
    """Restitution enters only through an approach faster than 1 m/s
    (sequential_impulse_solver.cpp:101-214): boxes driven into the plane at
    2 m/s, 8 steps, two worlds; the gradients of the centre-of-mass loss with
    respect to every dynamic box's restitution, mass and vertical velocity
    against central differences (eps 1e-4) through the oracle's FP64 step."""
    import torch

    sc = [sliding_boxes(6, 13, impact=True), sliding_boxes(6, 14, impact=True)]
    steps = 8
    roll = rollout.GpuRollout(sc, steps, DT, iterations=ITERS, checkpoint_every=4)
    target = torch.tensor([[1.0, 0.5, -2.0], [-3.0, 0.2, 1.0]], device="cuda:0")
    grads, oracle_loss = com_loss_and_oracle(sc, steps, roll, target)
    checks = []
    for w in range(2):
        base = int(roll.starts[w])
        for i in range(1, 7):
            checks += [(w, "r", i, 1, grads["r"][base + i]), (w, "m", i, 1, grads["m"][base + i]),
                       (w, "v", i, 1, grads["v"][base + i, 1])]
    assert max(abs(c[4]) for c in checks if c[1] == "r") > 1e-3  # restitution matters here
    scale = max(abs(c[4]) for c in checks)
    eps = 1e-4
    for w, which, i, j, a in checks:
        ref = (oracle_loss(w, which, i, j, eps) - oracle_loss(w, which, i, j, -eps)) / (2 * eps)
        assert abs(a - ref) <= 1e-3 * max(abs(ref), 1e-6 * scale), (w, which, i, a, ref)


def test_rollout_uneven_mixed_batch_matches_batch_engine(gpu):
    """Worlds of the uneven batched workload (mixed spheres and boxes, 16 to
    2,048 bodies, each sized by its own slot of the device arena): the forward
    rollout equals the batched engine bit for bit, and the adjoint gives finite
    gradients for every world."""
    import torch

    sizes = [2048, 16, 700, 37, 1500, 120, 300]
    sc = [scenes.generate(scenes.MIXED_VOLUME, n, 42 + w) for w, n in enumerate(sizes)]
    steps = 24
    roll = rollout.GpuRollout(sc, steps, 1 / 60, iterations=ITERS, checkpoint_every=10, manifolds_per_body=0.25)
    outs = roll.forward(*torch_state(roll))
    batch = gpu.GpuBatch(sc, iterations=ITERS)
    batch.step(1 / 60, steps)
    for k, (o, r) in enumerate(zip(outs, batch.bodies())):
        assert_bit_equal(o.cpu().numpy(), r, f"state {k}")
    assert roll.device_bytes() > 0
    rng = np.random.default_rng(3)
    d = [torch.tensor(rng.normal(size=tuple(o.shape)).astype(np.float32), device="cuda:0") for o in outs]
    grads = roll.backward(*d)
    for g in grads:
        assert bool(torch.isfinite(g).all())
    # the velocity gradient of a body reaches its own initial velocity
    assert float(grads[2].abs().max()) > 0
