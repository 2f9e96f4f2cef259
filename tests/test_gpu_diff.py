"""Gradients of the differentiable rollout (hand-written adjoint with
checkpointing and recomputation) against central finite differences: of the
same GPU forward in FP32 (h = 1e-3) and of the FP64 oracle (h = 1e-6, the
FP64 reference gradient).  Loss: squared distance of the final centre of mass
to (0.7, 0.5, 0.5); parameters: per-particle initial velocity v0 and Young's
modulus E (perturbed relatively: E (1 + h r), r in [0.5, 1.5]).  The block is
thrown at the floor: 64 substeps take it into contact, where its stiffness
moves the centre of mass (a free block's centre of mass does not depend on E)."""
import numpy as np
import pytest

from zeno_gb300 import scenes as S

pytestmark = pytest.mark.gpu

TARGET = np.array([0.7, 0.5, 0.5])


def _directions(n, k):
    """k-th direction of the directional checks: dv (n x 3) for v0 and
    relative factors rE in [0.5, 1.5] for E, from independent seeds."""
    base = [[1.0, 0.5, -0.3], [-0.4, 1.0, 0.6], [0.7, -0.8, 1.0]][k % 3]
    dv = np.tile([base], (n, 1)) + 0.5 * S.normal(5 + 10 * k, 0, n * 3).reshape(-1, 3)
    rE = 0.5 + S.uniform(6 + 10 * k, 0, n)
    return dv, rE


def _problem(cells=(16, 8, 8)):
    scene, parts = S.diff_scene(cells=cells)
    nu = scene.materials[0].nu
    E = parts.mu.astype(np.float64) * 2.0 * (1.0 + nu)
    v0 = S.diff_velocity(parts.n)
    dv, rE = _directions(parts.n, 0)
    return scene, parts, E, v0, dv, rE


def _gpu_grads(scene, parts, E, v0, steps, ckpt):
    import torch
    from zeno_gb300 import diff
    sim = diff.Rollout(scene, parts, steps, ckpt)
    v = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
    e = torch.tensor(E, dtype=torch.float64, device="cuda", requires_grad=True)
    L = diff.com_loss(sim.rollout(v, e), TARGET)
    L.backward()
    return sim, float(L.detach()), v.grad.double().cpu().numpy(), e.grad.double().cpu().numpy()


def _gpu_loss(sim, v0, E):
    import torch
    from zeno_gb300 import diff
    with torch.no_grad():
        x = sim.rollout(torch.tensor(v0, dtype=torch.float32, device="cuda"),
                        torch.tensor(E, dtype=torch.float64, device="cuda"))
        return float(diff.com_loss(x, TARGET))


def _oracle_loss(oracle_mod, scene, parts, v0, E, steps):
    p = parts.copy(dtype=np.float64)
    p.v = np.asarray(v0, np.float64)
    mu, lam = S.lame(np.asarray(E, np.float64), scene.materials[0].nu)
    p.mu, p.lam = mu, lam
    out, st = oracle_mod.run(scene, p, steps, "f64")
    assert st["status"] == 0
    return float(((out.x.mean(axis=0) - TARGET) ** 2).sum())


@pytest.mark.parametrize("k", [0, 1, 2])
def test_gradients_against_fp32_finite_differences(zsmpm_mod, k):
    """Three independent directions of v0 and of E."""
    scene, parts, E, v0, _, _ = _problem()
    dv, rE = _directions(parts.n, k)
    steps = 64
    sim, L, gv, gE = _gpu_grads(scene, parts, E, v0, steps, 16)
    h = 1e-3
    fd_v = (_gpu_loss(sim, v0 + h * dv, E) - _gpu_loss(sim, v0 - h * dv, E)) / (2 * h)
    ad_v = float((gv * dv).sum())
    assert abs(ad_v - fd_v) <= 2e-3 * abs(fd_v), (ad_v, fd_v)
    h = 1e-2  # the loss moves by ~1e-6 per percent of E: a larger step than for v0
    fd_E = (_gpu_loss(sim, v0, E * (1 + h * rE)) - _gpu_loss(sim, v0, E * (1 - h * rE))) / (2 * h)
    ad_E = float((gE * E * rE).sum())
    assert abs(ad_E - fd_E) <= 5e-2 * abs(fd_E) + 1e-12, (ad_E, fd_E)


@pytest.mark.parametrize("k", [0, 1, 2])
def test_gradients_against_fp64_reference(zsmpm_mod, oracle_mod, k):
    """Three independent directions of v0 and of E against central
    differences of the FP64 oracle."""
    scene, parts, E, v0, _, _ = _problem()
    dv, rE = _directions(parts.n, k)
    steps = 64
    _, L, gv, gE = _gpu_grads(scene, parts, E, v0, steps, 16)
    h = 1e-6
    ref_v = (_oracle_loss(oracle_mod, scene, parts, v0 + h * dv, E, steps) -
             _oracle_loss(oracle_mod, scene, parts, v0 - h * dv, E, steps)) / (2 * h)
    ad_v = float((gv * dv).sum())
    assert abs(ad_v - ref_v) <= 1e-3 * abs(ref_v), (ad_v, ref_v)
    ref_E = (_oracle_loss(oracle_mod, scene, parts, v0, E * (1 + h * rE), steps) -
             _oracle_loss(oracle_mod, scene, parts, v0, E * (1 - h * rE), steps)) / (2 * h)
    ad_E = float((gE * E * rE).sum())
    assert abs(ad_E - ref_E) <= 1e-2 * abs(ref_E) + 1e-12, (ad_E, ref_E)


def _entries(n, count=16):
    """(particle, component) entries spread over the particle index range."""
    idx = np.linspace(0, n - 1, count).round().astype(int)
    return idx, np.arange(count) % 3


def test_per_entry_gradients_against_fp64_reference(zsmpm_mod, oracle_mod):
    """The gradient entry by entry: 16 (particle, component) entries of v0
    and the E of 16 particles, each against a central difference of the FP64
    oracle on that single entry (v0: h = 3e-4 absolute; E: h = 1e-4
    relative; at these steps the FP64 differences agree with steps 3x
    larger and smaller to ~1e-5).  Tolerance per entry: 1e-3 of the entry
    for v0, 1e-2 for E (entries below 10 % of the largest sampled one are
    held to the same bound relative to that 10 % floor)."""
    scene, parts, E, v0, _, _ = _problem()
    steps = 64
    _, _, gv, gE = _gpu_grads(scene, parts, E, v0, steps, 16)
    idx, comp = _entries(parts.n)
    ref_v = []
    h = 3e-4
    for i, c in zip(idx, comp):
        vp, vm = v0.copy(), v0.copy()
        vp[i, c] += h
        vm[i, c] -= h
        ref_v.append((_oracle_loss(oracle_mod, scene, parts, vp, E, steps) -
                      _oracle_loss(oracle_mod, scene, parts, vm, E, steps)) / (2 * h))
    ref_v = np.array(ref_v)
    ad_v = gv[idx, comp]
    floor_v = 0.1 * np.abs(ref_v).max()
    err_v = np.abs(ad_v - ref_v) / np.maximum(np.abs(ref_v), floor_v)
    assert err_v.max() <= 1e-3, (err_v, ad_v, ref_v)
    ref_E = []
    h = 1e-4
    for i in idx:
        Ep, Em = E.copy(), E.copy()
        Ep[i] *= 1 + h
        Em[i] *= 1 - h
        ref_E.append((_oracle_loss(oracle_mod, scene, parts, v0, Ep, steps) -
                      _oracle_loss(oracle_mod, scene, parts, v0, Em, steps)) / (2 * h * E[i]))
    ref_E = np.array(ref_E)
    ad_E = gE[idx]
    floor_E = 0.1 * np.abs(ref_E).max()
    err_E = np.abs(ad_E - ref_E) / np.maximum(np.abs(ref_E), floor_E)
    assert err_E.max() <= 1e-2, (err_E, ad_E, ref_E)


def test_checkpoint_interval_does_not_change_gradients(zsmpm_mod):
    scene, parts, E, v0, _, _ = _problem(cells=(8, 8, 8))
    a = _gpu_grads(scene, parts, E, v0, 24, 4)
    b = _gpu_grads(scene, parts, E, v0, 24, 24)
    np.testing.assert_array_equal(a[2], b[2])
    np.testing.assert_array_equal(a[3], b[3])


def test_forward_matches_plain_substeps(zsmpm_mod):
    """The rollout's forward is the plain substep (the same sorted store and
    kernels): bit for bit the same positions."""
    import torch
    from zeno_gb300 import diff
    scene, parts, E, v0, _, _ = _problem(cells=(8, 8, 8))
    sim = diff.Rollout(scene, parts, 20, 5)
    with torch.no_grad():
        x = sim.rollout(torch.tensor(v0, dtype=torch.float32, device="cuda"),
                        torch.tensor(E, device="cuda")).cpu().numpy()
    p = parts.copy()
    p.v = v0.astype(np.float32)
    # the rollout's own mu, lam (torch divides by a scalar through its
    # reciprocal, so numpy's quotients can differ by an ulp)
    mu, lam = sim.lame(torch.tensor(E, device="cuda"))
    p.mu, p.lam = mu.float().cpu().numpy(), lam.float().cpu().numpy()
    with zsmpm_mod.Context(scene, max_particles=p.n) as ctx:
        ctx.upload(p)
        ctx.substep(scene.dt, 20)
        ref = ctx.download()["x"]
    np.testing.assert_array_equal(x, ref)


# ---- sand: StVK-Hencky stress with the Drucker-Prager projection ----

def _sand_problem():
    scene, parts = S.sand_column(dx=1.0 / 128, cells=(8, 16, 8))
    E = np.full(parts.n, float(scene.materials[0].E))
    v0 = S.sand_velocity(parts.n)
    dv = np.tile([[1.0, 0.5, -0.3]], (parts.n, 1)) + 0.5 * S.normal(5, 0, parts.n * 3).reshape(-1, 3)
    rE = 0.5 + S.uniform(6, 0, parts.n)
    return scene, parts, E, v0, dv, rE


def test_sand_gradients_against_fp32_finite_differences(zsmpm_mod):
    """v0 gradient of a sand column thrown at the floor (projection active)."""
    scene, parts, E, v0, dv, _ = _sand_problem()
    steps = 48
    sim, L, gv, gE = _gpu_grads(scene, parts, E, v0, steps, 8)
    h = 1e-3
    fd_v = (_gpu_loss(sim, v0 + h * dv, E) - _gpu_loss(sim, v0 - h * dv, E)) / (2 * h)
    ad_v = float((gv * dv).sum())
    assert abs(ad_v - fd_v) <= 5e-3 * abs(fd_v), (ad_v, fd_v)


def test_sand_gradients_against_fp64_reference(zsmpm_mod, oracle_mod):
    """v0 and E gradients of the sand column against central differences of
    the FP64 oracle (h = 1e-6)."""
    scene, parts, E, v0, dv, rE = _sand_problem()
    steps = 48
    _, L, gv, gE = _gpu_grads(scene, parts, E, v0, steps, 8)
    h = 1e-6
    ref_v = (_oracle_loss(oracle_mod, scene, parts, v0 + h * dv, E, steps) -
             _oracle_loss(oracle_mod, scene, parts, v0 - h * dv, E, steps)) / (2 * h)
    ad_v = float((gv * dv).sum())
    assert abs(ad_v - ref_v) <= 2e-3 * abs(ref_v), (ad_v, ref_v)
    ref_E = (_oracle_loss(oracle_mod, scene, parts, v0, E * (1 + h * rE), steps) -
             _oracle_loss(oracle_mod, scene, parts, v0, E * (1 - h * rE), steps)) / (2 * h)
    ad_E = float((gE * E * rE).sum())
    assert abs(ad_E - ref_E) <= 5e-2 * abs(ref_E), (ad_E, ref_E)
