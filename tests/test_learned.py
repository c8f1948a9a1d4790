"""The learned return map: the numpy oracle of the network is pinned by finite
differences (CPU); the GPU's tensor-core forward and backward kernels match the
oracle on the same parameters and records; training on harvested (trial,
projected) pairs reduces the loss; the learned G2P path stays within its stated
tolerance of the FP64 oracle step; and the trained network is compared with an
untrained one (what training gains: accepted predictions and error)."""
import numpy as np
import pytest

from anisotropicelastoplasticity_gb300 import HybridSolver, scenes
from oracle import mlp_oracle as mo

NP = 9928


def random_records(n, seed=0):
    rng = np.random.default_rng(seed)
    rec = np.zeros((n, 8), np.float32)
    ln = np.sort(rng.normal(0, 0.02, (n, 3)), axis=1)[:, ::-1]
    rec[:, 0:3] = ln
    rec[:, 3] = rng.random(n) * 0.5
    rec[:, 4] = rng.integers(0, 3, n)  # snow, sand, cloth rows
    rec[:, 5:8] = -0.3 * np.maximum(ln, 0) + 0.01 * rng.normal(size=(n, 3))
    return rec


def random_params(seed=1):
    rng = np.random.default_rng(seed)
    p = np.zeros(NP, np.float32)
    d = mo.unpack(p.astype(np.float64))
    d["w1t"][:, :7] = rng.normal(0, np.sqrt(2 / 7), (64, 7))
    d["w2t"][:] = rng.normal(0, np.sqrt(2 / 64), (64, 64))
    d["w3t"][:] = rng.normal(0, np.sqrt(2 / 64), (64, 64))
    d["w4t"][:3] = rng.normal(0, 0.1 * np.sqrt(2 / 64), (3, 64))
    for b in ("b1", "b2", "b3"):
        d[b][:] = 0.1 * rng.normal(size=64)
    d["b4"][:3] = 0.1 * rng.normal(size=3)
    return mo.pack(d).astype(np.float32)


def test_bf16_rounding_known_values():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-3], np.float32)
    r = mo.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125 and r[3] == -2.5
    assert abs(r[4] - 3.0e-3) / 3.0e-3 < 2 ** -8


def test_oracle_backward_matches_finite_differences():
    rec = random_records(24, seed=3)
    p = random_params(4).astype(np.float64)
    loss, g = mo.loss_and_grad(p, rec, bf=False)
    rng = np.random.default_rng(5)
    idx = np.concatenate([rng.choice(np.arange(0, 64 * 16).reshape(64, 16)[:, :7].ravel(), 10),
                          rng.integers(1024, 9728, 40), rng.integers(9728, 9728 + 195, 10)])
    for i in idx:
        h = 1e-6 * max(1.0, abs(p[i]))
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mo.loss_and_grad(pp, rec, bf=False)[0] - mo.loss_and_grad(pm, rec, bf=False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(abs(g).max(), 1e-12) + 1e-5 * abs(g[i]), (i, fd, g[i])


@pytest.mark.gpu
def test_gpu_gradient_matches_oracle():
    torch = pytest.importorskip("torch")
    from anisotropicelastoplasticity_gb300.learned import ReturnMapMLP

    rec = random_records(300, seed=7)  # several blocks of 64 rows, a partial last block
    p = random_params(8)
    m = ReturnMapMLP(seed=0)
    m.set_params(p)
    d = torch.from_numpy(rec).cuda()
    g_gpu, loss_gpu = m.gradient(d.data_ptr(), len(rec))
    loss_o, g_o = mo.loss_and_grad(p.astype(np.float64), rec, bf=True)
    assert abs(loss_gpu - loss_o) / loss_o < 1e-4
    go, gg = mo.unpack(g_o), mo.unpack(g_gpu.astype(np.float64))
    for name, _ in mo.LAYOUT:
        ref = go[name]
        if name == "w1t":
            ref, got = ref[:, :7], gg[name][:, :7]
        elif name in ("w4t", "b4"):
            ref, got = ref[:3], gg[name][:3]
        else:
            got = gg[name]
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        print(f"{name}: relative gradient difference {err:.2e}")
        # the two round to bfloat16 at the same points; an activation or gradient
        # whose FP32 value lands on the other side of a rounding boundary (the
        # accumulation orders differ) moves by 2^-9 of itself.  Measured on GB300:
        # at most 2.7e-6 (the biases of layers 1 and 2), 1e-7..8e-7 for the weights
        assert err < 5e-5, (name, err)


@pytest.mark.gpu
def test_gpu_adam_steps_match_fp64_adam():
    """Three Adam steps of aep_mlp_train (one batch = every record, so each step's
    gradient is the one aep_mlp_gradient returns for the same parameters) against
    FP64 Adam applied to those gradients: the parameters agree to FP32 rounding."""
    torch = pytest.importorskip("torch")
    from anisotropicelastoplasticity_gb300.learned import ReturnMapMLP

    rec = random_records(2048, seed=12)
    d = torch.from_numpy(rec).cuda()
    m = ReturnMapMLP(seed=0)
    m.set_params(random_params(13))
    p = m.get_params().astype(np.float64)
    mo_m, mo_v = np.zeros(NP), np.zeros(NP)
    lr = 2e-3
    for t in (1, 2, 3):
        g, _ = m.gradient(d.data_ptr(), len(rec))
        m.train(d.data_ptr(), len(rec), steps=1, batch=len(rec), lr=lr, lr_final=lr)
        got = m.get_params().astype(np.float64)
        p_want, mo_m, mo_v = mo.adam_step(p, g, mo_m, mo_v, t, lr)
        err = np.abs(got - p_want)
        # FP32 update arithmetic: a few units of FP32 spacing of the parameter, or
        # 1e-5 of the step for parameters near zero
        bound = 4 * np.spacing(np.abs(p_want).astype(np.float32)).astype(np.float64) + 1e-5 * lr
        assert np.all(err <= bound), (t, float((err / bound).max()))
        p = got


@pytest.mark.gpu
def test_gpu_forward_matches_oracle():
    torch = pytest.importorskip("torch")
    from anisotropicelastoplasticity_gb300.learned import ReturnMapMLP

    rec = random_records(1000, seed=9)
    p = random_params(10)
    m = ReturnMapMLP()
    m.set_params(p)
    d = torch.from_numpy(rec).cuda()
    out = torch.empty((len(rec), 3), dtype=torch.float32, device="cuda")
    m.forward(d.data_ptr(), len(rec), out.data_ptr())
    torch.cuda.synchronize()
    ref = mo.predict(p.astype(np.float64), rec, bf=True)
    assert np.abs(out.cpu().numpy() - ref).max() < 2e-4 * max(np.abs(ref).max(), 1e-3)
    # the step's arithmetic (its SiLU with the hardware tanh, relative error ~2^-11,
    # so a hidden activation is off by up to |z| 2^-12 before its bfloat16 rounding):
    # the same function to within the error that this feeds through two layers
    m.forward(d.data_ptr(), len(rec), out.data_ptr(), step_form=True)
    torch.cuda.synchronize()
    err = np.abs(out.cpu().numpy() - ref).max() / max(np.abs(ref).max(), 1e-3)
    print(f"step-form forward against the oracle: {err:.2e} of the largest output")
    assert err < 3e-3, err


def _strained(sc, seed):
    """The scene with +-1% random elastic strain: every state carries stress from the
    first step, and the plastic ones sit well above the FP32 resolution of ln s."""
    ps = sc.particles
    rng = np.random.default_rng(seed)
    ps.elastic_deformation_gradients = np.eye(3) + 0.01 * rng.standard_normal((len(ps), 3, 3))
    return sc


def _harvest_small(torch):
    from anisotropicelastoplasticity_gb300.learned import harvest_records

    # the snow block meets the ground after ~1,750 steps of 1e-4 s: harvest its impact
    recs = [harvest_records(scenes.snow_block(n=4096, res=32, seed=1), steps=200, capacity=100000, stride=1,
                            warm_steps=1650),
            harvest_records(_strained(scenes.sand_column(n=12000, res=32, seed=2), 7), steps=40, capacity=200000,
                            stride=1)]
    return torch.cat(recs)


def test_canonical_order_does_not_depend_on_the_input_order():
    """The harvest kernels append records in the order their atomics run; the
    canonical order (lexicographic by bit pattern) is the same for any permutation
    of one record set, duplicates included."""
    torch = pytest.importorskip("torch")
    from anisotropicelastoplasticity_gb300.learned import canonical_order

    rec = torch.from_numpy(random_records(5000, seed=21))
    rec = torch.cat([rec, rec[:100]])
    a = canonical_order(rec)
    b = canonical_order(rec[torch.randperm(len(rec), generator=torch.Generator().manual_seed(3))])
    assert torch.equal(a, b)
    bits = a.view(torch.int32).numpy()
    keys = [tuple(r) for r in bits[:200]]
    assert keys == sorted(keys)


@pytest.mark.gpu
def test_harvest_is_the_same_on_every_run():
    """Two harvests of the same scene give the same records in the same order, also
    when more records arrive than are kept (a seeded sample over all steps)."""
    torch = pytest.importorskip("torch")
    from anisotropicelastoplasticity_gb300.learned import harvest_records

    runs = [harvest_records(_strained(scenes.sand_column(n=12000, res=32, seed=2), 7), steps=20, capacity=50000,
                            stride=1) for _ in range(2)]
    assert len(runs[0]) == 50000
    assert torch.equal(runs[0], runs[1])


@pytest.mark.gpu
def test_training_reduces_loss_on_harvested_pairs():
    torch = pytest.importorskip("torch")
    from anisotropicelastoplasticity_gb300.learned import ReturnMapMLP

    rec = _harvest_small(torch)
    n = len(rec)
    assert n > 20000
    host = rec.cpu().numpy()
    assert np.all(np.isfinite(host))
    assert np.all(np.abs(host[:, 5:8]).max(axis=1) > 0)  # only projected (plastic) states are kept
    mat = host[:, 4].astype(int)
    assert (mat == 0).sum() > 1000 and (mat == 1).sum() > 1000
    # no sand apex (projection to ln s = 0, a constant the network never predicts)
    sand = host[mat == 1]
    assert np.all(np.abs(sand[:, 0:3] + sand[:, 5:8]).max(axis=1) > 0)
    m = ReturnMapMLP(seed=3)
    _, loss0 = m.gradient(rec.data_ptr(), n)
    loss1 = m.train(rec.data_ptr(), n, steps=1500, batch=4096, lr=2e-3, lr_final=2e-5)
    g_end, loss_end = m.gradient(rec.data_ptr(), n)
    assert loss_end < 0.05 * loss0, (loss0, loss1, loss_end)
    # the per-block gradients are summed in block order: training repeats bit for bit
    m2 = ReturnMapMLP(seed=3)
    assert m2.train(rec.data_ptr(), n, steps=1500, batch=4096, lr=2e-3, lr_final=2e-5) == loss1
    assert np.array_equal(m2.get_params(), m.get_params())
    g2, l2 = m2.gradient(rec.data_ptr(), n)
    assert np.array_equal(g2, g_end) and l2 == loss_end


def _learned_run(mlp, scene, steps, tol=1e-3):
    s = HybridSolver(scene.particles, scene.grid, scene.params)
    s.set_level_set(scene.levelset)
    s.init_volumes()
    s.set_return_map(mlp, tol)
    acc = fb = 0
    for _ in range(steps):
        s.step(scene.dt)
        st = s.stats()
        acc += st["learned_accepted"]
        fb += st["learned_fallbacks"]
    return s, acc, fb


@pytest.mark.gpu
def test_learned_step_matches_oracle_and_training_gains():
    torch = pytest.importorskip("torch")
    from anisotropicelastoplasticity_gb300.learned import ReturnMapMLP
    from oracle.oracle import Oracle

    rec = _harvest_small(torch)
    trained = ReturnMapMLP(seed=3)
    trained.train(rec.data_ptr(), len(rec), steps=2000, batch=4096, lr=2e-3, lr_final=2e-5)
    untrained = ReturnMapMLP(seed=3)
    strained = _strained(scenes.sand_column(n=12000, res=32, seed=5), 8)
    steps = 10
    # what training gains: the share of plastic states whose prediction passes the
    # in-kernel check against the exact projection (here within 1e-2 of its
    # magnitude) instead of falling back
    _, acc_tr, fb_tr = _learned_run(trained, strained, steps, tol=1e-2)
    _, acc_un, fb_un = _learned_run(untrained, strained, steps, tol=1e-2)
    rate_tr = acc_tr / max(acc_tr + fb_tr, 1)
    rate_un = acc_un / max(acc_un + fb_un, 1)
    assert acc_tr + fb_tr > 1000 and acc_un + fb_un > 1000
    assert rate_tr > rate_un + 0.3, (rate_tr, rate_un)
    # the learned path (default check, 1e-3) stays within its tolerance of the FP64
    # oracle step on the column at rest
    sc = scenes.sand_column(n=12000, res=32, seed=5)
    s_tr, acc, fb = _learned_run(trained, sc, steps)
    assert acc + fb > 0
    o = Oracle(sc.grid, sc.params)
    o.set_particle_system(sc.particles)
    o.set_level_set(sc.levelset)
    o.init(volumes=True)
    for _ in range(steps):
        o.step(sc.dt)
    gp, op = s_tr.get_particles(), o.get_particles()
    assert np.abs(gp["positions"] - op["positions"]).max() < 2e-6
    assert np.abs(gp["elastic_deformation_gradients"] - op["elastic_deformation_gradients"]).max() < 5e-4


@pytest.mark.gpu
@pytest.mark.parametrize("scene", ["mixed", "cloth"])
def test_learned_step_with_nothing_accepted_equals_the_plain_step(scene):
    """With an acceptance bound of zero every prediction falls back, and the learned
    pipeline (the trial check and queue in G2P, the exact projection in the finisher,
    the cloth elements' exact cap) must give the plain step's state bit for bit."""
    from anisotropicelastoplasticity_gb300.learned import ReturnMapMLP

    from .parity_util import perturbed, small_scene

    m = ReturnMapMLP(seed=5)
    if scene == "mixed":
        sc = perturbed(small_scene("mixed"), seed=31)
        _strained(sc, 9)
        mesh = None
    else:
        from .test_cloth_gpu import small_cloth

        grid, ps, mesh, ls, prm = small_cloth(True, seed=12, E=1e4, weighting=1)
        sc = type("S", (), {"particles": ps, "grid": grid, "params": prm, "levelset": ls, "dt": 2e-5})()
    outs = []
    for learned in (False, True):
        s = HybridSolver(sc.particles, sc.grid, sc.params)
        if mesh is not None:
            s.set_lagrangian_mesh(mesh)
        s.set_level_set(sc.levelset)
        s.init_volumes()
        if learned:
            s.set_return_map(m, 0.0, abs_tolerance=0.0)
        acc = fb = 0
        for _ in range(6):
            s.step(sc.dt)
            st = s.stats()
            acc += st["learned_accepted"]
            fb += st["learned_fallbacks"]
        outs.append((s.get_particles(), s.get_mesh() if mesh is not None else {}, acc, fb))
        s.close()
    (p0, m0, _, _), (p1, m1, acc, fb) = outs
    assert acc == 0 and fb > 0, (acc, fb)
    for k in p0:
        assert np.array_equal(p0[k], p1[k]), k
    for k in m0:
        assert np.array_equal(m0[k], m1[k]), k


@pytest.mark.gpu
def test_learned_cloth_return_map():
    """Cloth rows of the network: harvested (trial, projected) QR columns of plastic
    elements train the map; with it attached the elements' return mapping is
    predicted and checked, and the mesh stays within the cloth tolerances of the
    FP64 oracle."""
    torch = pytest.importorskip("torch")
    from anisotropicelastoplasticity_gb300.learned import ReturnMapMLP
    from oracle.oracle import Oracle

    from .test_cloth_gpu import _compare_mesh, pair, small_cloth

    grid, ps, mesh, ls, prm = small_cloth(False, seed=6, E=1e4, weighting=1)
    gpu, _ = pair(grid, ps, mesh, ls, prm)
    buf = torch.zeros((200000, 8), dtype=torch.float32, device="cuda")
    gpu.set_harvest(buf.data_ptr(), len(buf), 1)
    for _ in range(40):
        gpu.step(2e-5)
    nrec = min(gpu.harvest_count(), len(buf))
    gpu.set_harvest(0, 0, 1)
    rec = buf[:nrec].contiguous()
    assert nrec > 500 and torch.all(rec[:, 4] == 2)
    m = ReturnMapMLP(seed=4)
    _, loss0 = m.gradient(rec.data_ptr(), nrec)
    m.train(rec.data_ptr(), nrec, steps=1500, batch=4096, lr=2e-3, lr_final=2e-5)
    _, loss1 = m.gradient(rec.data_ptr(), nrec)
    assert loss1 < 0.2 * loss0
    g2, orc = pair(grid, ps, mesh, ls, prm)
    g2.set_return_map(m, 1e-3)
    acc = fb = 0
    orc.init(volumes=False)
    for _ in range(10):
        g2.step(2e-5)
        orc.step(2e-5)
        st = g2.stats()
        acc += st["learned_accepted"]
        fb += st["learned_fallbacks"]
    assert acc + fb > 0
    # an accepted prediction may differ from the exact projection by up to the
    # tolerance (1e-3) relative to the projected (r13, r23, r33 - 1), whose size is
    # at most ~1, in each of the 10 steps: the directions get 10 x 1e-3, the rest
    # keeps the exact-path tolerances
    _compare_mesh(g2.get_mesh(), orc.get_mesh(), 2e-6, 1e-3, 1e-2, 5e-3)


@pytest.mark.gpu
def test_scene_runner_with_the_learned_return_map(capsys):
    """python -m anisotropicelastoplasticity_gb300.run_scene ... --learned STEPS trains
    the network on the scene's own exact mappings and runs the learned step."""
    import json

    from anisotropicelastoplasticity_gb300 import run_scene

    assert run_scene.main(["snow_sand_collision", "--arg", "n=8192", "--arg", "res=32", "--steps", "2",
                           "--warmup", "1", "--learned", "200"]) == 0
    out = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert out["return_map"] == "learned"
    assert out["ms_per_step"] > 0 and out["phases_ms_per_step"]["mlp"] >= 0
