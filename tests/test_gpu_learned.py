"""The learned search radius: training/inference kernels against an
independent float64 computation, exactness of the learned search against
the plain search, and what the trained network gains over a radius that is
not learned."""
import numpy as np
import pytest

import helpers as H
from oracle import mlp_oracle as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _nb():
    import libnabo_gb300 as nb
    return nb


@pytest.fixture(scope="module")
def lidar():
    from libnabo_gb300 import synthetic as S
    cloud = S.lidar_scan(n_azimuth=2400)
    q = S.lidar_queries(cloud)
    return cloud, q


@pytest.fixture(scope="module")
def lidar_model(lidar):
    """A model trained on another frame of the scene (fresh range noise, the
    same pose change): held-out queries, disjoint from every query the tests
    evaluate it on."""
    nb = _nb()
    from libnabo_gb300 import synthetic as S
    cloud, q = lidar
    s = nb.NearestNeighbourSearch(cloud, creationOptionFlags=nb.TOUCH_STATISTICS)
    frame = S.lidar_queries(S.lidar_scan(n_azimuth=2400, noise_seed=99))
    rng = np.random.default_rng(0)
    train = frame[rng.choice(frame.shape[0], 40000, replace=False)]
    m = nb.RadiusModel(s, train, k=10, maxRadius=1.0, epochs=12)
    return s, m


def test_inference_matches_float64_forward(lidar, lidar_model):
    s, m = lidar_model
    _, q = lidar
    sample = q[:3001]
    params, meta = m.get_params()
    X = m.features(sample).cpu().numpy()
    y_cpu, _ = M.forward(params, X)
    radii, raw = m.predict(sample, raw=True)
    raw = raw.cpu().numpy().astype(np.float64)
    err = np.abs(raw - y_cpu)
    assert err.max() < 2e-2 and err.mean() < 2e-3, (err.max(), err.mean())
    r_cpu = meta[2] * np.exp(meta[0] + meta[1] * (raw + meta[7]))
    np.testing.assert_allclose(radii.cpu().numpy(), r_cpu.astype(np.float32), rtol=2e-5)


def test_gradients_match_float64(lidar, lidar_model):
    _, m = lidar_model
    _, q = lidar
    rng = np.random.default_rng(1)
    sample = q[rng.choice(q.shape[0], 777, replace=False)]  # not a multiple of the 32-sample tile
    X = m.features(sample).cpu().numpy()
    Y = rng.normal(size=777).astype(np.float32)
    params, _ = m.get_params()
    g_gpu, loss_gpu = m.gradients(X, Y)
    g_cpu, loss_cpu = M.gradients(params, X, Y)
    rel = np.linalg.norm(g_gpu - g_cpu) / np.linalg.norm(g_cpu)
    assert rel < 5e-3, rel
    assert abs(loss_gpu - loss_cpu) <= 1e-3 * loss_cpu
    # every parameter block agrees, not just the norm
    for lo, hi in ((M.OFF_W1, M.OFF_B1), (M.OFF_B1, M.OFF_W2), (M.OFF_W2, M.OFF_B2), (M.OFF_B2, M.OFF_W3),
                   (M.OFF_W3, M.OFF_B3)):
        blk = np.linalg.norm(g_gpu[lo:hi] - g_cpu[lo:hi]) / max(np.linalg.norm(g_cpu[lo:hi]), 1e-12)
        assert blk < 2e-2, (lo, blk)


def test_training_reduces_loss(lidar, lidar_model):
    _, m = lidar_model
    meta = m.meta
    assert meta["train_samples"] > 30000
    # standardised targets have unit variance; a trained network explains most of it
    assert meta["train_loss"] < 0.5, meta


@pytest.mark.parametrize("k,radius", [(10, 1.0), (10, np.inf), (1, 1.0), (5, 0.3)])
def test_learned_search_equals_plain_search(lidar, lidar_model, k, radius):
    nb = _nb()
    cloud, q = lidar
    s, m = lidar_model
    pi, pd = s.knn(q, k, 0.0, 0, radius)
    plain_touched = s.touched
    li, ld = m.knn(q, k, 0.0, 0, radius)
    H.assert_identical(li, ld, pi, pd, f"learned k={k} r={radius}")
    assert 0 <= m.fallbacks < q.shape[0]
    assert m.touched > 0 and plain_touched > 0


def test_learned_search_device_api(lidar, lidar_model):
    import torch
    cloud, q = lidar
    s, m = lidar_model
    tq = torch.from_numpy(q).cuda()
    fb = torch.zeros(1, dtype=torch.int32, device="cuda")
    di, dd = m.knn_device(tq, 10, 0.0, 0, 1.0, fallbacks=fb)
    hi, hd = m.knn(q, 10, 0.0, 0, 1.0)
    torch.cuda.synchronize()
    H.assert_identical(di.cpu().numpy(), dd.cpu().numpy(), hi, hd, "device vs host")
    assert int(fb.item()) == m.fallbacks


def test_trained_network_gains_over_a_fixed_radius(lidar, lidar_model):
    """What the network buys: against the best radius that is not learned --
    one radius for every query, set to the same safety factor times the
    median k-th distance of the training queries -- the learned radii send
    far fewer queries back to the unbounded search, and the bounded search
    with them examines fewer points than the unbounded one."""
    cloud, q = lidar
    s, m = lidar_model
    k = 10
    _, pd = s.knn(q, k, 0.0, 0, 1.0)
    plain_touched = s.touched
    m.knn(q, k, 0.0, 0, 1.0)
    learned_rate = m.fallbacks / q.shape[0]
    learned_touched = m.touched
    dk = np.sqrt(pd[:, -1])
    fixed = np.float32(1.2 * np.median(dk[np.isfinite(dk)]))
    fi, fd = s.knn(q, k, 0.0, 0, 1.0, maxRadii=np.full(q.shape[0], min(fixed, 1.0), np.float32))
    fixed_rate = float(np.mean((fi[:, -1] < 0) & (fixed < 1.0)))
    assert learned_rate < 0.5 * fixed_rate, (learned_rate, fixed_rate)
    assert learned_rate < 0.2, learned_rate
    assert learned_touched < plain_touched * (1.0 + learned_rate), (learned_touched, plain_touched)


def test_save_and_load_give_the_same_radii(lidar, lidar_model, tmp_path):
    nb = _nb()
    cloud, q = lidar
    s, m = lidar_model
    path = str(tmp_path / "radius_model.npz")
    m.save(path)
    m2 = nb.RadiusModel(s, q[:2000], k=10, maxRadius=1.0, epochs=1, seed=99)
    r_before = m2.predict(q[:5000]).cpu().numpy()
    m2.load(path)
    r_after = m2.predict(q[:5000]).cpu().numpy()
    r_orig = m.predict(q[:5000]).cpu().numpy()
    assert np.array_equal(r_after, r_orig) and not np.array_equal(r_before, r_orig)


@pytest.mark.parametrize("dtype,d", [(np.float64, 3), (np.float32, 8), (np.float64, 8)])
def test_learned_search_other_types_and_dims(dtype, d):
    nb = _nb()
    from libnabo_gb300 import synthetic as S
    cloud, centres, sig = S.clusters(60000, d, seed=77, dtype=dtype)
    q, _, _ = S.clusters(20000, d, seed=78, dtype=dtype, centres=centres, sigmas=sig)
    s = nb.NearestNeighbourSearch(cloud)
    m = nb.RadiusModel(s, q[:10000], k=8, epochs=6)
    assert m.meta["inputs"] == (11 if d == 3 else d)
    pi, pd = s.knn(q, 8)
    li, ld = m.knn(q, 8)
    H.assert_identical(li, ld, pi, pd, f"learned {dtype.__name__} d={d}")
    ei, ed = m.knn(q, 8, 0.5)  # approximate: within the (1+eps) bound of the exact search
    assert (ed <= (np.asarray(1.5, dtype) ** 2) * pd * (1 + 1e-6)).all()
