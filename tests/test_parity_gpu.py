"""GPU step (libaep.so through the C-ABI) against the FP64 oracle on identical
seeded inputs: grid state after P2G, after the force scatter and after the grid
update + collision, particle state after 1 and 10 steps, first-P2G volumes,
bit-for-bit repeatability, exact mass conservation, and edge cases.

Tolerances are FP32-vs-FP64: the bulk arithmetic is FP32 with int64
fixed-point grid sums; each bound is stated at its assertion."""
import numpy as np
import pytest

from anisotropicelastoplasticity_gb300 import AepError, HybridSolver, capi, scenes

from .parity_util import make_pair, mass_weighted_rel, max_rel, perturbed, small_scene

pytestmark = pytest.mark.gpu

KINDS = ["snow", "sand", "mixed", "boundary"]


@pytest.mark.parametrize("kind", KINDS)
def test_p2g_grid_matches_oracle(kind):
    sc = perturbed(small_scene(kind), seed=11)
    gpu, orc = make_pair(sc)
    gpu.step_stage(sc.dt, capi.AEP_STAGE_P2G)
    g = gpu.get_grid()
    orc.init(volumes=False)
    o = orc.get_grid()
    # node masses: FP32 contributions summed exactly in fixed point -> ~1e-7 relative
    assert max_rel(g["masses"], o["masses"]) < 2e-6
    # total grid mass (the boundary scene loses the weight of out-of-grid nodes, as the reference does)
    assert abs(g["masses"].sum() - o["masses"].sum()) / o["masses"].sum() < 1e-6
    # APIC momentum / mass: mass-weighted relative error
    assert mass_weighted_rel(g["velocities"], o["velocities"], o["masses"]) < 2e-5


@pytest.mark.parametrize("n", [1, 33, 127, 129, 4097, 100003])
def test_p2g_grid_matches_oracle_at_chunk_boundaries(n):
    """P2G picks its particles per warp (32 to 128) from the particle count, and
    each block's grid tile from its middle particle: particle counts around a
    warp, a block and an uneven last chunk give the oracle's grid."""
    sc = perturbed(scenes.sand_column(n=n, res=32, seed=n), seed=n + 1)
    gpu, orc = make_pair(sc)
    gpu.step_stage(sc.dt, capi.AEP_STAGE_P2G)
    g = gpu.get_grid()
    orc.init(volumes=False)
    o = orc.get_grid()
    assert max_rel(g["masses"], o["masses"]) < 2e-6
    assert abs(g["masses"].sum() - o["masses"].sum()) / o["masses"].sum() < 1e-6
    assert mass_weighted_rel(g["velocities"], o["velocities"], o["masses"]) < 2e-5
    gpu.close()


@pytest.mark.parametrize("kind", KINDS)
def test_force_scatter_matches_oracle(kind):
    sc = perturbed(small_scene(kind), seed=12)
    gpu, orc = make_pair(sc)
    gpu.step_stage(sc.dt, capi.AEP_STAGE_FORCES)
    g = gpu.get_grid()
    orc.init(volumes=False)
    orc.step(sc.dt, stage=capi.AEP_STAGE_FORCES)
    o = orc.get_grid()
    grav = np.array(list(sc.params.gravity))
    f_orc = o["forces"] - o["masses"][:, None] * grav  # the GPU reports f without gravity
    # FP32 SVD + stress relative to the largest nodal force
    assert max_rel(g["forces"], f_orc) < 2e-4


@pytest.mark.parametrize("kind", KINDS)
def test_grid_update_collision_matches_oracle(kind):
    sc = perturbed(small_scene(kind), seed=13)
    gpu, orc = make_pair(sc)
    gpu.step_stage(sc.dt, capi.AEP_STAGE_GRID)
    g = gpu.get_grid()
    orc.init(volumes=False)
    orc.step(sc.dt, stage=capi.AEP_STAGE_GRID)
    o = orc.get_grid()
    assert mass_weighted_rel(g["velocities"], o["velocities"], o["masses"]) < 1e-4
    assert mass_weighted_rel(g["velocities_before_friction"], o["velocities_before_friction"], o["masses"]) < 1e-4


def _compare_particles(gp, op, pos_tol, vel_tol, F_tol, B_tol, q_tol, h):
    assert np.abs(gp["positions"] - op["positions"]).max() < pos_tol
    assert max_rel(gp["velocities"], op["velocities"]) < vel_tol
    assert np.abs(gp["elastic_deformation_gradients"] - op["elastic_deformation_gradients"]).max() < F_tol
    # B ~ v h: relative to max(|B|, max|v| h) so that an exactly affine-free field (B = 0) is measurable
    bscale = max(np.abs(op["affine_momenta"]).max(), np.abs(op["velocities"]).max() * h)
    assert np.abs(gp["affine_momenta"] - op["affine_momenta"]).max() / bscale < B_tol
    assert np.abs(gp["plastic"] - op["plastic"]).max() < q_tol


@pytest.mark.parametrize("kind", KINDS)
def test_one_step_matches_oracle(kind):
    sc = perturbed(small_scene(kind), seed=14)
    gpu, orc = make_pair(sc)
    gpu.step(sc.dt)
    orc.init(volumes=False)
    orc.step(sc.dt)
    _compare_particles(gpu.get_particles(), orc.get_particles(), pos_tol=5e-7, vel_tol=1e-4, F_tol=2e-6,
                       B_tol=1e-3, q_tol=2e-6, h=float(sc.grid.h.min()))


@pytest.mark.parametrize("kind", ["snow", "sand", "mixed"])
def test_ten_steps_match_oracle(kind):
    sc = small_scene(kind, seed=3)
    gpu, orc = make_pair(sc)
    gpu.init_volumes()
    orc.init(volumes=True)
    for _ in range(10):
        gpu.step(sc.dt)
        orc.step(sc.dt)
    _compare_particles(gpu.get_particles(), orc.get_particles(), pos_tol=1e-6, vel_tol=2e-4, F_tol=1e-5,
                       B_tol=2e-3, q_tol=1e-5, h=float(sc.grid.h.min()))


@pytest.mark.parametrize("kind", ["snow", "sand"])
def test_init_volumes_match_oracle(kind):
    sc = small_scene(kind)
    gpu, orc = make_pair(sc)
    gpu.init_volumes()
    orc.init(volumes=True)
    assert max_rel(gpu.get_particles()["volumes"], orc.get_particles()["volumes"]) < 1e-5


def test_repeatable_bit_for_bit():
    sc = perturbed(small_scene("mixed"), seed=21)
    outs = []
    for _ in range(2):
        gpu = HybridSolver(sc.particles, sc.grid, sc.params)
        gpu.set_level_set(sc.levelset)
        for _ in range(5):
            gpu.step(sc.dt)
        outs.append((gpu.get_particles(), gpu.get_grid()))
    for k in ("positions", "velocities", "affine_momenta", "elastic_deformation_gradients", "plastic"):
        assert np.array_equal(outs[0][0][k], outs[1][0][k]), k
    assert np.array_equal(outs[0][1]["velocities"], outs[1][1]["velocities"])


def test_mass_conserved_exactly_over_run():
    sc = small_scene("sand")
    gpu = HybridSolver(sc.particles, sc.grid, sc.params)
    gpu.set_level_set(sc.levelset)
    gpu.init_volumes()
    m0 = None
    for _ in range(30):
        gpu.step(sc.dt)
        s = gpu.stats()
        m0 = s["total_mass"] if m0 is None else m0
        assert s["total_mass"] == m0  # exact: the grid mass is sum_p T_p in fixed point every step
        assert s["overflow"] == 0
    assert abs(m0 - sc.particles.masses.sum()) / sc.particles.masses.sum() < 1e-7


def test_plastic_F_tracking_matches_oracle():
    sc = perturbed(small_scene("snow"), seed=15)
    sc.params.track_plastic_F = 1
    gpu, orc = make_pair(sc)
    for _ in range(3):
        gpu.step(sc.dt)
    orc.init(volumes=False)
    for _ in range(3):
        orc.step(sc.dt)
    gp = gpu.get_particles(want_fp=True)
    op = orc.get_particles()
    assert np.abs(gp["plastic_deformation_gradients"] - op["plastic_deformation_gradients"]).max() < 1e-5


def test_invalid_arguments():
    sc = small_scene("snow")
    gpu = HybridSolver(None, sc.grid, sc.params)
    with pytest.raises(AepError):
        gpu.step(1e-4)  # no particles yet
    gpu.set_particle_system(sc.particles)
    with pytest.raises(AepError):
        gpu.step(-1.0)
    bad = sc.particles.copy()
    bad.masses[0] = np.nan
    with pytest.raises(AepError):
        gpu.set_particle_system(bad)


def test_out_of_domain_particles_are_counted_not_fatal():
    sc = small_scene("snow")
    ps = sc.particles.copy()
    ps.positions[:10] = [1.5, 0.5, 0.5]
    gpu = HybridSolver(ps, sc.grid, sc.params)
    gpu.set_level_set(sc.levelset)
    gpu.step(sc.dt)
    assert gpu.stats()["out_of_domain"] == 10
    assert np.all(np.isfinite(gpu.get_particles()["positions"]))


def _upload_raw(solver, ps, state):
    """aep_set_particles with the state read back from the device, Fp = NULL so that the
    snow J_P travels in `plastic`."""
    import ctypes as C

    from anisotropicelastoplasticity_gb300.solver import mats_to_ref, rows_to_ref, vec_to_ref

    arrs = [vec_to_ref(state["positions"]), vec_to_ref(state["velocities"]), rows_to_ref(state["affine_momenta"]),
            mats_to_ref(state["elastic_deformation_gradients"]), None, np.ascontiguousarray(ps.masses, float),
            np.ascontiguousarray(state["volumes"], float), np.ascontiguousarray(state["plastic"], float)]
    dp = [None if a is None else a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs]
    mat = np.ascontiguousarray(ps.material, np.uint8)
    solver._check(solver._lib.aep_set_particles(solver._h, len(ps), *dp, mat.ctypes.data_as(C.POINTER(C.c_uint8))))


def test_reupload_keeps_state_and_order():
    """set -> step -> get -> set (same n) keeps every value and the device order, so the
    next step is bit-identical to a solver that never re-uploaded."""
    sc = perturbed(small_scene("mixed"), seed=23)
    a = HybridSolver(sc.particles, sc.grid, sc.params)
    b = HybridSolver(sc.particles, sc.grid, sc.params)
    for s in (a, b):
        s.set_level_set(sc.levelset)
        s.init_volumes()
        for _ in range(3):
            s.step(sc.dt)
    st = b.get_particles()
    _upload_raw(b, sc.particles, st)
    again = b.get_particles()
    for k in ("positions", "velocities", "affine_momenta", "elastic_deformation_gradients", "volumes", "plastic"):
        assert np.array_equal(again[k], st[k]), k
    a.step(sc.dt)
    b.step(sc.dt)
    ra, rb = a.get_particles(), b.get_particles()
    for k in ("positions", "velocities", "affine_momenta", "elastic_deformation_gradients", "plastic"):
        assert np.array_equal(ra[k], rb[k]), k


def test_incremental_ordering_matches_full_sort():
    """The incremental ordering (movers partitioned out, ranked, merged) against the
    full radix sort every step: same particles, results equal up to the FP32
    rounding of the per-run sums (equal keys may be ordered differently)."""
    sc = perturbed(scenes.sand_column(n=40000, res=32, seed=12), seed=13, vscale=2.0)
    runs = {}
    for full in (0, 1):
        prm = capi.aep_params.from_buffer_copy(sc.params)
        prm.full_sort = full
        prm.reorder_interval = 1
        s = HybridSolver(sc.particles, sc.grid, prm)
        s.set_level_set(sc.levelset)
        s.init_volumes()
        movers = []
        for _ in range(12):
            s.step(sc.dt)
            movers.append(s.stats()["sort_movers"])
        runs[full] = (s.get_particles(), movers, s.stats()["total_mass"])
    inc, full = runs[0], runs[1]
    assert inc[1][0] == -1 and all(0 <= m < 40000 // 4 for m in inc[1][1:])  # first step: full sort
    assert any(m > 0 for m in inc[1][1:]) and all(m == -1 for m in full[1])
    assert inc[2] == full[2]  # exact fixed-point mass
    assert np.abs(inc[0]["positions"] - full[0]["positions"]).max() < 1e-6
    assert max_rel(inc[0]["velocities"], full[0]["velocities"]) < 1e-4


def test_reorder_interval_keeps_order_between_orderings():
    """reorder_interval = 4: three of every four steps keep the particles in their
    slots, and the particles that changed cell meanwhile are scattered and
    gathered out of order.  Against ordering every step: the same particles, exact
    fixed-point mass, results equal up to the FP32 rounding of the per-run sums;
    against the FP64 oracle at the usual step tolerances; and a checkpoint taken
    between two orderings resumes bit for bit."""
    from oracle.oracle import Oracle

    sc = perturbed(scenes.sand_column(n=40000, res=32, seed=14), seed=15, vscale=2.0)
    runs = {}
    for interval in (1, 4):
        prm = capi.aep_params.from_buffer_copy(sc.params)
        prm.reorder_interval = interval
        s = HybridSolver(sc.particles, sc.grid, prm)
        s.set_level_set(sc.levelset)
        s.init_volumes()
        movers = []
        for _ in range(10):
            s.step(sc.dt)
            movers.append(s.stats()["sort_movers"])
        runs[interval] = (s, movers, s.stats()["total_mass"])
    every, kept = runs[1], runs[4]
    # steps 1 (a full sort: the particles are still in the upload order), 5 and 9
    # order, the others keep the order
    assert kept[1][0] == -1 and kept[1][4] > 0 and kept[1][8] > 0
    assert all(kept[1][k] == 0 for k in (1, 2, 3, 5, 6, 7, 9))
    assert every[2] == kept[2]
    a, b = every[0].get_particles(), kept[0].get_particles()
    assert np.abs(a["positions"] - b["positions"]).max() < 1e-6
    assert max_rel(a["velocities"], b["velocities"]) < 1e-4
    o = Oracle(sc.grid, sc.params)
    o.set_particle_system(sc.particles)
    o.set_level_set(sc.levelset)
    o.init(volumes=True)
    for _ in range(10):
        o.step(sc.dt)
    op = o.get_particles()
    assert np.abs(b["positions"] - op["positions"]).max() < 2e-6
    assert max_rel(b["velocities"], op["velocities"]) < 2e-3
    # resume between orderings (one step after the ordering of step 9)
    s = kept[0]
    blob = s.checkpoint()
    for _ in range(4):
        s.step(sc.dt)
    ref = s.get_particles()
    s.load_checkpoint(blob)
    for _ in range(4):
        s.step(sc.dt)
    again = s.get_particles()
    for k in ("positions", "velocities", "elastic_deformation_gradients"):
        assert np.array_equal(ref[k], again[k])
    for s, _, _ in runs.values():
        s.close()


@pytest.mark.parametrize("where", ["pinned", "device"])
def test_upload_and_readback_from_pinned_and_device_memory(where):
    """aep_set_particles / aep_get_particles read and write page-locked host memory
    and device memory directly (no staging copy); the results equal the pageable
    path bit for bit, including a re-upload that keeps the device order."""
    import ctypes as C

    torch = pytest.importorskip("torch")
    from anisotropicelastoplasticity_gb300.solver import mats_to_ref, rows_to_ref, vec_to_ref

    sc = perturbed(scenes.snow_sand_collision(n=12000, res=32, seed=21), seed=22)
    ps = sc.particles
    n = len(ps)
    ref = HybridSolver(ps, sc.grid, sc.params)
    ref.set_level_set(sc.levelset)
    ref.init_volumes()
    for _ in range(3):
        ref.step(sc.dt)
    want = ref.get_particles()

    def buf(a):
        t = torch.from_numpy(np.ascontiguousarray(a))
        return t.pin_memory() if where == "pinned" else t.cuda()

    host = [vec_to_ref(ps.positions), vec_to_ref(ps.velocities), rows_to_ref(ps.affine_momenta),
            mats_to_ref(ps.elastic_deformation_gradients), mats_to_ref(ps.plastic_deformation_gradients),
            np.ascontiguousarray(ps.masses, float), np.ascontiguousarray(ps.volumes, float),
            np.ascontiguousarray(ps.plastic_amount, float)]
    bufs = [buf(a) for a in host]
    mat = buf(np.ascontiguousarray(ps.material, np.uint8))
    s = HybridSolver(None, sc.grid, sc.params)
    s._np = n
    lib, h = s._lib, s._h
    dp = lambda t: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))
    assert lib.aep_set_particles(h, n, *[dp(t) for t in bufs], C.cast(C.c_void_p(mat.data_ptr()),
                                                                     C.POINTER(C.c_uint8))) == 0
    s.set_level_set(sc.levelset)
    s.init_volumes()
    for _ in range(3):
        s.step(sc.dt)
    outs = [buf(np.zeros(k * n)) for k in (3, 3, 9, 9, 1, 1)]
    assert lib.aep_get_particles(h, n, dp(outs[0]), dp(outs[1]), dp(outs[2]), dp(outs[3]), None, dp(outs[4]),
                                 dp(outs[5])) == 0
    torch.cuda.synchronize()
    got = [o.cpu().numpy() for o in outs]
    wants = [vec_to_ref(want["positions"]), vec_to_ref(want["velocities"]), rows_to_ref(want["affine_momenta"]),
             mats_to_ref(want["elastic_deformation_gradients"]), want["volumes"], want["plastic"]]
    for g, w in zip(got, wants):
        assert np.array_equal(g, np.ravel(w))
    # re-upload of the read-back state (keeps the device order) and one more step
    for t, g in zip((bufs[0], bufs[1], bufs[2], bufs[3], bufs[6], bufs[7]), outs):
        t.view(-1).copy_(g)
    assert lib.aep_set_particles(h, n, *[dp(t) for t in bufs[:5]], dp(bufs[5]), dp(bufs[6]), dp(bufs[7]),
                                 C.cast(C.c_void_p(mat.data_ptr()), C.POINTER(C.c_uint8))) == 0
    s.step(sc.dt)
    ref.set_particle_system(ps.__class__(want["positions"], want["velocities"], ps.masses, want["volumes"],
                                         want["elastic_deformation_gradients"], ps.plastic_deformation_gradients,
                                         want["affine_momenta"], want["plastic"], ps.material))
    ref.step(sc.dt)
    a, b = s.get_particles(), ref.get_particles()
    assert np.array_equal(a["positions"], b["positions"]) and np.array_equal(a["velocities"], b["velocities"])


@pytest.mark.parametrize("kind", ["snow", "sand"])
def test_fp64_fallbacks_match_oracle(kind):
    """Near-degenerate deformation gradients (a singular value at 1% of the largest)
    take the FP64 path: in the force pass a separate kernel (k_force_fp64) redoes
    their stress and scatters it, in G2P the return mapping is redone in FP64.
    Forces and the stepped particles match the oracle at the usual tolerances."""
    sc = perturbed(small_scene(kind), seed=31)
    ps = sc.particles
    rng = np.random.default_rng(32)
    sel = rng.random(len(ps)) < 0.05
    q, _ = np.linalg.qr(rng.standard_normal((int(sel.sum()), 3, 3)))
    ps.elastic_deformation_gradients[sel] = q @ np.diag([1.0, 0.9, 0.01]) @ q.transpose(0, 2, 1)
    gpu, orc = make_pair(sc)
    gpu.step_stage(sc.dt, capi.AEP_STAGE_FORCES)
    assert gpu.stats()["fp64_fallbacks"] >= sel.sum()
    g = gpu.get_grid()
    orc.init(volumes=False)
    orc.step(sc.dt, stage=capi.AEP_STAGE_FORCES)
    o = orc.get_grid()
    f_orc = o["forces"] - o["masses"][:, None] * np.array(list(sc.params.gravity))
    assert max_rel(g["forces"], f_orc) < 2e-4
    gpu2, orc2 = make_pair(sc)
    gpu2.step(sc.dt)
    assert gpu2.stats()["fp64_fallbacks"] >= sel.sum()
    orc2.init(volumes=False)
    orc2.step(sc.dt)
    _compare_particles(gpu2.get_particles(), orc2.get_particles(), pos_tol=5e-7, vel_tol=1e-4, F_tol=2e-6,
                       B_tol=1e-3, q_tol=2e-6, h=float(sc.grid.h.min()))
