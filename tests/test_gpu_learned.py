"""Learned relaxation: the tcgen05 GEMM and MLP kernels against numpy, the
feature pass against a numpy restatement of its message sums, the fallback
path against the plain step (bit for bit), and training plus the learned
step against the plain relaxation."""
import numpy as np
import pytest

from conftest import bits_equal
from sph_gb300 import LearnedModel, Simulation, gemm_check, scenes

pytestmark = pytest.mark.gpu


def bf16(x):
    """Round-to-nearest-even float32 -> bfloat16, returned as float32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) & 0xFFFF0000).astype(np.uint32).view(np.float32)


def act_bf16(z):
    """The network's activation, 2 GELU (tanh form), evaluated step by step
    in BF16 arithmetic as the kernels evaluate it (each fused multiply-add
    rounded once)."""
    r = lambda v: bf16(np.asarray(v, np.float32)).astype(np.float64)  # noqa: E731
    c0, c1 = r(0.7978846), r(0.0356774)
    x = r(z)
    x2 = r(x * x)
    t = r(x2 * c1 + c0)
    u = r(x * t)
    th = r(np.tanh(u))
    return r(x * th + x)


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (200, 48, 96), (5, 16, 20), (300, 130, 130),
                                   (16, 128, 4096)])
def test_gemm_matches_numpy(cuda_lib, M, N, K):
    rng = np.random.default_rng(M * 1000 + N + K)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    C = gemm_check(A, B)
    ref = bf16(A).astype(np.float64) @ bf16(B).astype(np.float64).T
    # FP32 accumulation of exact BF16 products
    assert np.abs(C - ref).max() <= 1e-5 * np.sqrt(K) * np.abs(ref).max() + 1e-5


def numpy_mlp(w, x):
    """Inference form: the constant feature 31 carries the first bias, the
    second bias is added in BF16."""
    p = LearnedModel.unpack(w)
    W1 = p["W1"].astype(np.float32).copy()
    W1[:, 31] = W1[:, 31] + p["b1"]
    xb = bf16(x).astype(np.float64)
    z1 = xb @ bf16(W1).astype(np.float64).T
    h1 = act_bf16(z1)
    z2 = h1 @ bf16(p["W2"]).astype(np.float64).T + bf16(p["b2"])
    h2 = act_bf16(z2)
    return h2 @ bf16(p["W3"]).astype(np.float64).T + p["b3"]


def test_mlp_forward_matches_numpy(cuda_lib):
    rng = np.random.default_rng(5)
    with LearnedModel(0, seed=11) as m:
        w = m.get_params()
        w += rng.normal(0.0, 0.02, w.shape).astype(np.float32)  # non-zero biases
        m.set_params(w)
        assert np.array_equal(m.get_params(), w)
        x = rng.standard_normal((1000, LearnedModel.IN)).astype(np.float32)
        x[:, 31] = 1.0  # the constant feature
        y = m.forward(x)
        ref = numpy_mlp(w, x)
        # tanh.approx against tanh: an occasional BF16 ulp in an activation
        # (any layout or indexing fault gives errors of the order of the outputs)
        d = y[:, :3] - ref[:, :3]
        assert np.abs(d).max() <= 1.5e-2 * np.abs(ref[:, :3]).max(), np.abs(d).max()
        assert np.sqrt(np.mean(d ** 2)) <= 1e-2 * np.sqrt(np.mean(ref[:, :3] ** 2))
        assert np.all(y[:, 3:] == 0.0)
        # rows are independent: a prefix gives the same rows
        assert np.array_equal(m.forward(x[:130]), y[:130])


def random_blob(n, seed, vel=0.0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(5.0, 35.0, n).astype(np.float32)
    y = rng.uniform(5.0, 35.0, n).astype(np.float32)
    vx = rng.uniform(-vel, vel, n).astype(np.float32)
    vy = rng.uniform(-vel, vel, n).astype(np.float32)
    p = scenes.Params(g=0.0, sigma=0.0, beta=0.0)
    p.node_start_x, p.node_end_x = 0.0, 40.0
    return scenes.Scene(name="blob", x=x, y=y, vx=vx, vy=vy, box=(0.0, 40.0, 0.0, 40.0),
                        params=p, spacing=1.0, size_x=40, size_y=40)


def numpy_features(sc):
    """The feature rows (before BF16 rounding) of the predicted state of a
    scene without gravity or viscosity: x* = x + v dt."""
    P = sc.params
    dt = np.float32(P.time_step)
    px = (sc.x + sc.vx * dt).astype(np.float32)
    py = (sc.y + sc.vy * dt).astype(np.float32)
    vx = ((px - sc.x) / dt).astype(np.float64)
    vy = ((py - sc.y) / dt).astype(np.float64)
    h = float(P.smoothing_radius)
    n = sc.n
    out = np.zeros((n, 32))
    cnt = np.zeros(n, np.int64)
    k, kn, ks, rest = P.k, P.k_near, P.k_spring, P.rest_density
    ak, an, as_ = k / (k + kn + ks), kn / (k + kn + ks), ks / (k + kn + ks)
    # every particle's neighbours and densities first: the messages carry
    # the neighbours' densities and near densities
    nbs, ws, us = [], [], []
    rho, rhon = np.zeros(n), np.zeros(n)
    for i in range(n):
        dx = (px - px[i]).astype(np.float32)
        dy = (py - py[i]).astype(np.float32)
        r2 = (dx * dx + dy * dy).astype(np.float32)
        nb = np.nonzero(r2 <= np.float32(h * h))[0]
        nb = nb[nb != i]
        r = np.sqrt(r2[nb].astype(np.float64))
        q = r / h
        w = np.where(q < 1, 1.0 - q, 0.0)
        nbs.append(nb)
        ws.append(w)
        us.append((dx[nb] / r, dy[nb] / r))
        rho[i], rhon[i] = np.sum(w * w), np.sum(w ** 3)
    for i in range(n):
        nb, w, (ux, uy) = nbs[i], ws[i], us[i]
        cnt[i] = len(nb)
        a, b = rho[i], rhon[i]
        dvx = (vx[nb] - vx[i]) * dt / h
        dvy = (vy[nb] - vy[i]) * dt / h
        V1 = (np.sum(w * ux), np.sum(w * uy))
        V2 = (np.sum(w * w * ux), np.sum(w * w * uy))
        pr = w * (rho[nb] - rest)
        prn = w * w * rhon[nb]
        R1 = (np.sum(pr * ux), np.sum(pr * uy))
        R2 = (np.sum(prn * ux), np.sum(prn * uy))
        f = [a / 4, b / 2, V1[0] / 4, V1[1] / 4, V2[0] / 2, V2[1] / 2, np.sum(w) / 8,
             min(len(nb), 48) / 48, np.sum(w * dvx) * 2.5, np.sum(w * dvy) * 2.5,
             np.sum(w * ux * ux) / 4, np.sum(w * ux * uy) / 4, np.sum(w * uy * uy) / 4,
             ak, an, as_, rest / 4,
             ak * (a - rest) * V1[0] / 4, ak * (a - rest) * V1[1] / 4,
             an * b * V2[0] / 2, an * b * V2[1] / 2, as_ * V1[0] / 2, as_ * V1[1] / 2,
             ak * R1[0] / 4, ak * R1[1] / 4, an * R2[0] / 2, an * R2[1] / 2]
        f += [0.0] * (31 - len(f)) + [1.0]
        out[i] = f
    return out, cnt


@pytest.mark.parametrize("vel", [0.0, 0.6])
def test_features_match_numpy(cuda_lib, vel):
    sc = random_blob(1500, seed=21 + int(vel * 10), vel=vel)
    with Simulation.from_scene(sc) as s:
        f, c = s.learned_features()
    ref, rc = numpy_features(sc)
    assert np.array_equal(c, rc)
    assert c.max() < 48
    scale = np.abs(ref).max(axis=0) + 1e-3
    err = np.abs(f - ref) / scale
    # BF16 rounding of each feature (2^-8 relative) plus FP32 sums
    assert err.max() < 1.2e-2, (err.max(axis=0))


def dam_break(n=16384):
    return scenes.config2(n)


def test_fallback_only_is_the_plain_step(cuda_lib):
    sc = dam_break()
    with Simulation.from_scene(sc) as plain, Simulation.from_scene(sc) as learned, \
            LearnedModel(0, seed=3) as m:
        learned.set_learned(m, threshold=-1.0)
        for t in range(0, 30, 10):
            sched = [sc.params_at(t + i).as_dict() for i in range(10)]
            plain.step_schedule(sched)
            learned.step_schedule(sched)
        a, b = plain.download(), learned.download()
        for f in ("x", "y", "v_x", "v_y", "density", "density_near"):
            assert bits_equal(a[f], b[f]), f
        used, fell = learned.learned_counts()
        assert used == 0 and fell == 30 * sc.n
        times = learned.kernel_times()
        assert list(times)[4:8] == ["features", "mlp", "relax_learned", "relax_fallback"]
        assert learned.launches_per_step() == 11


@pytest.mark.parametrize("long_masks", [False, True])
def test_fallback_only_is_the_plain_step_in_dense_cells(cuda_lib, long_masks):
    """Cells of 25 particles: stencil rows of ~75 candidates, longer than a
    stored hit mask, so the plain relaxation searches the whole stencil (or,
    with long-row masks, walks two masks per row) and the fallback pass
    walks the rows 64 candidates at a time -- the same neighbours in the same
    order, bit for bit; and long-row masks change no bit of the plain step."""
    sc = scenes.dam_break(6400, 80, 64.0, 64.0, seed=77, name="dense", lattice=0.2,
                          x0=0.1, y0=0.1)
    gx = np.floor(sc.x / sc.spacing).astype(np.int64)
    gy = np.floor(sc.y / sc.spacing).astype(np.int64)
    assert 3 * np.bincount(gy * sc.size_x + gx).max() > 64
    P = sc.params.as_dict()
    with Simulation.from_scene(sc) as plain, Simulation.from_scene(sc) as learned, \
            Simulation.from_scene(sc) as ref, LearnedModel(0, seed=5) as m:
        for s in (plain, learned):
            s.set_long_row_masks(long_masks)
            assert s.long_row_masks() == long_masks
        for s in (plain, learned, ref):
            s.step(P, 2)
        learned.set_learned(m, threshold=-1.0)
        for s in (plain, learned, ref):
            s.step(P, 4)
        a, b, c = plain.download(), learned.download(), ref.download()
        for f in ("x", "y", "v_x", "v_y", "density", "density_near"):
            assert bits_equal(a[f], b[f]), f
            assert bits_equal(a[f], c[f]), f


def test_long_row_masks_leave_the_features_as_they_are(cuda_lib):
    """The message walk over two masks per long row visits the same
    neighbours in the same order as the whole-stencil walk."""
    sc = scenes.dam_break(6400, 80, 64.0, 64.0, seed=78, name="dense", lattice=0.2,
                          x0=0.1, y0=0.1)
    P = sc.params.as_dict()
    with Simulation.from_scene(sc) as a, Simulation.from_scene(sc) as b:
        b.set_long_row_masks(True)
        a.step(P, 3)
        b.step(P, 3)
        fa, ca = a.learned_features()
        fb, cb = b.learned_features()
    assert np.array_equal(ca, cb)
    assert bits_equal(fa, fb)


def rms_density_error(sc, model, state_steps, threshold):
    """One step from the same state with and without the model: RMS of the
    density difference (by particle) in units of the rest density, and the
    fraction of particles that used the network."""
    with Simulation.from_scene(sc) as a, Simulation.from_scene(sc) as b:
        sched = [sc.params_at(i).as_dict() for i in range(state_steps)]
        a.step_schedule(sched)
        b.step_schedule(sched)
        b.set_learned(model, threshold)
        p = sc.params_at(state_steps).as_dict()
        a.step(p)
        b.step(p)
        ra, _ = a.probe_density(p)
        rb, _ = b.probe_density(p)
        used, fell = b.learned_counts()
        return float(np.sqrt(np.mean((ra - rb) ** 2)) / sc.params.rest_density), used / sc.n


@pytest.fixture(scope="module")
def trained(cuda_lib):
    """A model trained on one 16,384-particle dam break (samples every 8
    steps over 240 steps), with the first and last training losses."""
    sc = dam_break()
    m = LearnedModel(400_000, seed=7)
    with Simulation.from_scene(sc) as s:
        for t in range(0, 240, 8):
            s.step_schedule([sc.params_at(t + i).as_dict() for i in range(8)])
            m.collect(s, 0.6)
    n = m.num_samples
    first = m.train(1, 2048, 1e-3)
    last = m.train(12, 2048, 1e-3)
    with Simulation.from_scene(sc) as s:
        s.step_schedule([sc.params_at(i).as_dict() for i in range(200)])
        m.calibrate(s, epochs=4)
    yield m, n, first, last
    m.close()


def test_training_and_learned_step(trained):
    m, n, first, last = trained
    sc = dam_break()
    assert n > 100_000
    assert last < 0.5 * first, (first, last)
    err, frac = rms_density_error(sc, m, 200, 0.01)
    err_all, frac_all = rms_density_error(sc, m, 200, 1e9)
    assert frac_all > 0.7
    assert err <= err_all + 1e-6
    assert err <= 0.01, (err, frac, err_all)


def test_params_round_trip_gives_the_same_steps(trained):
    m = trained[0]
    sc = dam_break()
    w = m.get_params()
    with LearnedModel(0, seed=99) as m2:
        m2.set_params(w)
        outs = []
        for model in (m, m2):
            with Simulation.from_scene(sc) as s:
                s.step_schedule([sc.params_at(i).as_dict() for i in range(20)])
                s.set_learned(model, 0.01)
                s.step_schedule([sc.params_at(20 + i).as_dict() for i in range(5)])
                outs.append(s.download())
        for f in ("x", "y", "v_x", "v_y"):
            assert bits_equal(outs[0][f], outs[1][f]), f


def test_skewed_ensemble_learned(trained):
    """Config-5 scenes (settled piles + Gaussian blobs), batched, with the
    network: one step against the plain ensemble from the same state."""
    from sph_gb300 import Ensemble
    m = trained[0]
    scs = scenes.settle_and_drop(scenes.config5(12), 60)
    n = sum(s.n for s in scs)
    a, b = Ensemble(scs), Ensemble(scs)
    try:
        for e in (a, b):
            e.upload_scenes()
            e.step(None, 30)
        b.set_learned(m, 0.01)
        a.step(None, 1)
        b.step(None, 1)
        ra, _ = a.probe_density()
        rb, _ = b.probe_density()
        used, fell = b.learned_counts()
        assert used + fell == n and used > 0.5 * n
        rms = float(np.sqrt(np.mean((ra.astype(np.float64) - rb) ** 2)) / 1.3)
        assert rms <= 0.01, rms
        # every scene stays in its box
        st = b.download()
        for k, sc in enumerate(scs):
            sl = b.scene_slice(k)
            assert st["x"][sl].min() >= 0 and st["x"][sl].max() <= sc.box[1]
    finally:
        a.close()
        b.close()


def test_bounded_wait_gives_up(cuda_lib):
    """A tensor-core wait on an mbarrier that nothing arrives at ends with a
    recorded error status (no hang), and the context stays usable."""
    import ctypes
    from sph_gb300 import _lib
    flag = ctypes.c_int(-1)
    _lib.check(cuda_lib.sph_learned_wait_selftest(ctypes.byref(flag)))
    assert flag.value == 1
    # the device still works afterwards
    A = np.ones((128, 32), np.float32)
    assert np.allclose(gemm_check(A, A[:16]), 32.0)
