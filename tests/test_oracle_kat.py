"""Known-answer tests that pin the FP64 oracle (the reference ships no tests or
golden vectors, so the pins come from the mathematics of the reference step):

1. cubic B-spline partition of unity, linear reproduction, derivative consistency
   (interpolation.cpp:9-33);
2. particle weights: sum w = 1, sum w x_i = x_p, sum grad w = 0,
   sum x_i (grad w)^T = I for full stencils (HybridSolver.cpp:30-79);
3. 3x3 SVD contract of Eigen::JacobiSVD (HS:308,620): A = U S V^T, orthogonal
   U and V, S >= 0 sorted;
4. Gram-Schmidt QR (geometry.cpp:31-62): Q orthonormal, R upper triangular;
5. snow clamp (HS:626-631) and Drucker-Prager projection (HS:632-674): elastic
   points unchanged, projected points on the yield cone, tension to the apex,
   idempotence;
6. P2G conserves mass and momentum; an affine velocity field survives the APIC
   P2G -> G2P round trip exactly (zero stiffness, no gravity);
7. fixed cloth vertices (HS:513-550): a fixed vertex keeps its position and has
   zero velocity after steps (its whole stencil is zeroed, and the weights
   reproduce linear fields).
"""
import numpy as np
import pytest

from anisotropicelastoplasticity_gb300 import capi, make_params
from anisotropicelastoplasticity_gb300.solver import LevelSet, ParticleSystem, RegularGrid
from oracle.oracle import Oracle, cubic, dcubic, gram_schmidt, particle_weights, return_map, svd3


def test_spline_partition_of_unity_and_linear_reproduction():
    for x in np.linspace(-0.99, 0.99, 57):
        nodes = np.arange(-3, 4)
        w = np.array([cubic(x - i) for i in nodes])
        assert abs(w.sum() - 1.0) < 1e-14
        assert abs((w * nodes).sum() - x) < 1e-14
        dw = np.array([dcubic(x - i) for i in nodes])
        assert abs(dw.sum()) < 1e-13


def test_spline_derivative_matches_finite_differences():
    for x in np.linspace(-1.95, 1.95, 41):
        fd = (cubic(x + 1e-6) - cubic(x - 1e-6)) / 2e-6
        assert abs(fd - dcubic(x)) < 1e-7
    assert cubic(2.0) == 0.0 and cubic(-2.5) == 0.0 and dcubic(2.0) == 0.0


def test_particle_weights_reproduce_constants_and_linear_fields():
    grid = RegularGrid([0, 0, 0], [1, 1, 1], [16, 16, 16])
    prm = make_params()
    rng = np.random.default_rng(0)
    pos_nodes = grid.positions()
    for _ in range(20):
        xp = 0.2 + 0.6 * rng.random(3)
        node, w, g = particle_weights(grid, prm, xp)
        assert len(node) == 64
        xi = pos_nodes[node]
        assert abs(w.sum() - 1.0) < 1e-13
        assert np.abs((w[:, None] * xi).sum(0) - xp).max() < 1e-13
        assert np.abs(g.sum(0)).max() < 1e-10
        assert np.abs(xi.T @ g - np.eye(3)).max() < 1e-10


def test_weights_drop_nodes_outside_the_grid():
    grid = RegularGrid([0, 0, 0], [1, 1, 1], [16, 16, 16])
    node, w, _ = particle_weights(grid, make_params(), [0.01, 0.51, 0.52])
    assert len(node) == 48  # the x = -1 layer is dropped (HybridSolver.cpp:44-46)
    assert w.sum() < 1.0


@pytest.mark.parametrize("seed", range(6))
def test_svd_contract(seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((3, 3))
    if seed == 4:
        A[:, 2] = A[:, 0] * 2.0  # singular
    if seed == 5:
        A = np.diag([1.0, 1.0, 1.0]) + 1e-9 * rng.standard_normal((3, 3))  # near-degenerate
    U, s, V = svd3(A)
    assert np.abs(U @ np.diag(s) @ V.T - A).max() < 1e-13
    assert np.abs(U.T @ U - np.eye(3)).max() < 1e-13
    assert np.abs(V.T @ V - np.eye(3)).max() < 1e-13
    assert np.all(s >= 0) and s[0] >= s[1] >= s[2]
    assert np.allclose(s, np.linalg.svd(A, compute_uv=False), atol=1e-13)


def test_gram_schmidt_qr():
    rng = np.random.default_rng(3)
    D = np.eye(3) + 0.3 * rng.standard_normal((3, 3))
    Q, R = gram_schmidt(D)
    assert np.abs(Q @ R - D).max() < 1e-14
    assert np.abs(Q.T @ Q - np.eye(3)).max() < 1e-14
    assert np.allclose(np.tril(R, -1), 0) and np.all(np.diag(R) > 0)


def test_snow_clamp_and_idempotence():
    prm = make_params()
    lo, hi = 1 - prm.snow.theta_c, 1 + prm.snow.theta_s
    s, q = return_map(prm, capi.AEP_SNOW, [1.05, 1.0, 0.9], 0.0)
    assert np.allclose(s, [hi, 1.0, lo])
    s2, _ = return_map(prm, capi.AEP_SNOW, s, 0.0)
    assert np.array_equal(s, s2)


def _dp_yield(prm, s, q):
    E, nu = prm.sand.E, prm.sand.nu
    lam = E * nu / (1 + nu) / (1 - 2 * nu)
    mu = E / 2 / (1 + nu)
    phi = (prm.sand.h0 + (prm.sand.h1 * q - prm.sand.h3) * np.exp(-prm.sand.h2 * q)) * np.pi / 180
    alpha = np.sqrt(2 / 3) * 2 * np.sin(phi) / (3 - np.sin(phi))
    ln = np.log(s)
    dev = ln - ln.mean()
    return np.linalg.norm(dev) + (3 * lam + 2 * mu) / (2 * mu) * ln.sum() * alpha


def test_drucker_prager_projection_lands_on_the_cone():
    prm = make_params()
    rng = np.random.default_rng(5)
    on_cone = 0
    for _ in range(200):
        s0 = np.exp(rng.normal(0, 0.02, 3) - 0.01)
        q0 = rng.random() * 0.5
        f0 = _dp_yield(prm, s0, q0)
        s, q = return_map(prm, capi.AEP_SAND, s0, q0)
        if f0 <= 0:
            assert np.array_equal(s, s0) and q == q0  # elastic: unchanged
        elif np.log(s0).sum() > 0:
            assert np.allclose(s, 1.0) and q > q0  # tension: apex
        else:
            on_cone += 1
            # projected with the hardening state before the update (HS:646-672)
            assert abs(_dp_yield(prm, s, q0)) < 1e-12
            assert abs((np.log(s).sum()) - np.log(s0).sum()) < 1e-12  # trace preserved
            assert q > q0
            s2, q2 = return_map(prm, capi.AEP_SAND, s, q0)  # idempotent at the same state
            assert np.allclose(s2, s, atol=1e-12) and q2 == pytest.approx(q0, abs=1e-12)
    assert on_cone > 20


def _scene(n=400, seed=1, mat=capi.AEP_SNOW, E=None):
    rng = np.random.default_rng(seed)
    x = 0.35 + 0.3 * rng.random((n, 3))
    ps = ParticleSystem(positions=x, velocities=rng.standard_normal((n, 3)), masses=0.5 + rng.random(n),
                        volumes=np.full(n, 1e-4), elastic_deformation_gradients=np.tile(np.eye(3), (n, 1, 1)),
                        material=np.full(n, mat, np.uint8))
    kw = dict(gravity=[0.0, 0.0, 0.0])
    if E is not None:
        kw.update(snow_E=E)
    return RegularGrid([0, 0, 0], [1, 1, 1], [32, 32, 32]), ps, make_params(**kw)


def test_p2g_conserves_mass_and_momentum():
    grid, ps, prm = _scene()
    ps.affine_momenta = 0.01 * np.random.default_rng(2).standard_normal((len(ps), 3, 3))
    o = Oracle(grid, prm)
    o.set_particle_system(ps)
    o.init(volumes=False)
    g = o.get_grid()
    assert abs(g["masses"].sum() - ps.masses.sum()) < 1e-12 * ps.masses.sum()
    p_grid = (g["masses"][:, None] * g["velocities"]).sum(0)
    p_part = (ps.masses[:, None] * ps.velocities).sum(0)
    assert np.abs(p_grid - p_part).max() < 1e-11 * np.abs(p_part).max()


def test_apic_round_trip_of_an_affine_field_is_exact():
    grid, ps, prm = _scene(E=0.0)
    h = float(grid.h[0])
    a = np.array([0.3, -0.2, 0.1])
    Cm = np.array([[0.1, 0.2, -0.1], [0.0, -0.3, 0.2], [0.15, 0.05, 0.1]])
    ps.velocities = a + ps.positions @ Cm.T
    ps.affine_momenta = np.tile(Cm * h * h / 3.0, (len(ps), 1, 1))  # B = C D, D = h^2/3 I (HS:177)
    o = Oracle(grid, prm)
    o.set_particle_system(ps)
    o.set_level_set(LevelSet.ground(-10.0))
    o.init(volumes=False)
    o.step(1e-5)
    r = o.get_particles()
    assert np.abs(r["velocities"] - ps.velocities).max() < 1e-12
    assert np.abs(r["affine_momenta"] - ps.affine_momenta).max() < 1e-14
    assert np.abs(r["positions"] - (ps.positions + 1e-5 * ps.velocities)).max() < 1e-15 + 1e-12


def test_fixed_vertices_stay_put():
    from anisotropicelastoplasticity_gb300 import LagrangianMesh, scenes

    rng = np.random.default_rng(1)
    V, F = scenes.sheet(12, 0.4, (0.5, 0.5), 0.6, 1e-4, rng)
    mesh = LagrangianMesh.from_triangles(V, F, density=6.4, thickness=1 / 32, youngs_modulus=5.0, poisson_ratio=0.3,
                                         shear_stiffness=1e3, stiffness=1e3, friction_coeff=0.3)
    mesh.vertex_velocities = 0.2 * rng.standard_normal((len(V), 3))
    grid = RegularGrid([0, 0, 0], [1, 1, 1], [32, 32, 32])
    o = Oracle(grid, make_params())
    o.set_lagrangian_mesh(mesh)
    o.set_level_set(LevelSet.ground(0.05))
    fixed = np.zeros(len(V))
    fixed[[0, 11, 60]] = 1.0
    o.set_fixed_vertices(fixed)
    o.init(volumes=False)
    for _ in range(5):
        o.step(2e-5)
    m = o.get_mesh()
    f = fixed > 0
    assert np.abs(m["vertex_positions"][f] - V[f]).max() < 1e-14
    assert np.abs(m["vertex_velocities"][f]).max() == 0.0
    assert np.abs(m["vertex_positions"][~f] - V[~f]).max() > 1e-6  # the others move
    with pytest.raises(ValueError):
        o.set_fixed_vertices(np.ones(5))


def test_scene_factories_follow_the_reference_rules():
    from anisotropicelastoplasticity_gb300 import scenes

    b = scenes.snow_ball([0.5, 0.5, 0.5], 0.1, 4000, seed=1)
    assert len(b) == 4000 and np.all(b.material == capi.AEP_SNOW)
    assert np.linalg.norm(b.positions - 0.5, axis=1).max() <= 0.1
    assert abs(b.masses.sum() - 100 * 3.14 * 1e-3) < 1e-12
    s = scenes.sand_block([0, 0, 0], [0.4, 0.4, 0.4], 0.15, 5000, seed=2)
    assert np.linalg.norm(s.positions - [0, 0, 0.2], axis=1).min() >= 0.15
    with pytest.raises(ValueError):
        scenes.sand_block([0, 0, 0], [1, 1, 0.2], 0.1, 10)
    c = scenes.sand_cylinder([0.5, 0.5, 0.1], 0.1, 0.3, 3000, seed=3)
    assert np.all(c.velocities[:, 2] == -1.0) and c.positions[:, 2].min() >= 0.1
    assert np.linalg.norm(c.positions[:, :2] - 0.5, axis=1).max() <= 0.1
    assert abs(c.masses.sum() - 1300 * np.pi * 0.01 * 0.3) < 1e-9
    sb = scenes.sand_ball([0, 0, 0], 0.2, 100, seed=4)
    assert abs(sb.masses.sum() - 1300 * 3.14 * 0.008) < 1e-12
