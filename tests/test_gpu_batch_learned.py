"""The learned radius on batches of clouds: one network per (dimension,
scalar type) serving every cloud of a batch, trained on the GPU from exact
batched results, with per-query radii searched through the reference's
per-query radius seam (nabo/nabo.h:351). Results must equal the plain
batched search's exactly at epsilon 0 (and the oracle's), stay within the
(1 + epsilon) bound at epsilon 0.5, and the training kernel's gradients
must match the float64 restatement."""
import numpy as np
import pytest

from oracle import mlp_oracle as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu

K = 32


def _clouds(dtype, seed, n_clouds=6):
    from libnabo_gb300 import synthetic as S
    sizes = S.log_uniform_sizes(n_clouds, 20000, 80000, seed)
    clouds, train, evalq = [], [], []
    for i, n in enumerate(sizes):
        c, centres, sig = S.clusters(int(n), 8, seed + 10 + i, dtype=dtype)
        t, _, _ = S.clusters(3000, 8, seed + 1000 + i, dtype=dtype, centres=centres, sigmas=sig)
        e, _, _ = S.clusters(2500, 8, seed + 2000 + i, dtype=dtype, centres=centres, sigmas=sig)
        clouds.append(c)
        train.append(t)
        evalq.append(e)
    return clouds, train, evalq


@pytest.fixture(scope="module", params=[np.float32, np.float64], ids=["f32", "f64"])
def trained(request):
    import torch

    import libnabo_gb300 as nb
    dtype = request.param
    clouds, train, evalq = _clouds(dtype, seed=77)
    b = nb.BatchSearch([c.shape[0] for c in clouds], dim=8, dtype=dtype, maxLevels=64)
    tc = torch.from_numpy(np.concatenate(clouds)).cuda()
    b.set_queries([t.shape[0] for t in train], K)
    b.build(tc)
    tt = torch.from_numpy(np.concatenate(train)).cuda()
    _, td2 = b.knn(tt)
    model = b.train_radius_model(tt, td2, epochs=20)
    b.set_queries([e.shape[0] for e in evalq], K)
    te = torch.from_numpy(np.concatenate(evalq)).cuda()
    return dict(b=b, model=model, clouds=clouds, evalq=evalq, te=te, dtype=dtype)


def test_batched_learned_search_equals_plain_and_oracle(trained):
    import torch
    b, model, te = trained["b"], trained["model"], trained["te"]
    pi, pd = b.knn(te)
    fb = torch.zeros(1, dtype=torch.int32, device="cuda")
    li, ld = b.knn_learned(model, te, fallbacks=fb)
    torch.cuda.synchronize()
    assert torch.equal(pi, li) and torch.equal(pd, ld)
    # the fallback rule is exercised but rare (calibrated to ~1 % of training queries)
    assert 0 <= int(fb.item()) < 0.05 * te.shape[0], int(fb.item())
    bi, bd = b.split(li.cpu().numpy()), b.split(ld.cpu().numpy())
    for c in (0, len(trained["clouds"]) - 1):
        oi, od, _ = O.OracleTree(trained["clouds"][c]).knn(trained["evalq"][c][:800], K, mode=O.MODE_CANONICAL)
        assert np.array_equal(bi[c][:800], oi) and np.array_equal(bd[c][:800], od), c


def test_batched_learned_search_epsilon_bound(trained):
    import torch
    b, model, te = trained["b"], trained["model"], trained["te"]
    _, ld = b.knn_learned(model, te, epsilon=0.5)
    _, pd = b.knn(te)
    torch.cuda.synchronize()
    ad = ld.cpu().numpy()
    ed = pd.cpu().numpy()
    # every rank's squared distance within (1 + eps)^2 of the exact one
    assert (ad <= (1.5 ** 2) * ed * (1 + 1e-6)).all()


def test_batched_model_predicts_kth_distance(trained):
    """The network's radius tracks each query's own k-th distance across
    clouds of very different densities (it sees the query's home leaf, not
    its coordinates), and inference matches the float64 forward pass."""
    import torch
    b, model, te = trained["b"], trained["model"], trained["te"]
    meta = model.meta
    assert meta["inputs"] == 8 and meta["train_samples"] > 10000
    assert meta["train_loss"] < 0.3, meta
    _, pd = b.knn(te)
    radii, raw = b.predict_radii(model, te, raw=True)
    X = b.radius_features(model, te).cpu().numpy()
    torch.cuda.synchronize()
    dk = np.sqrt(np.concatenate([d[:, -1] for d in b.split(pd.cpu().numpy())]).astype(np.float64))
    r = radii.cpu().numpy().astype(np.float64)
    ratio = r / dk
    assert np.mean(ratio >= 1.0) > 0.95, np.mean(ratio >= 1.0)  # few fallbacks
    assert np.median(ratio) < 2.5, np.median(ratio)              # and a useful bound
    params, _ = model.get_params()
    y_cpu, _ = M.forward(params, X)
    err = np.abs(raw.cpu().numpy().astype(np.float64) - y_cpu)
    assert err.max() < 2e-2 and err.mean() < 2e-3, (err.max(), err.mean())


def test_batched_model_gradients_match_float64(trained):
    model = trained["model"]
    rng = np.random.default_rng(3)
    X = np.zeros((555, 16), np.float32)
    X[:, :8] = rng.uniform(-1.5, 1.5, (555, 8))
    Y = rng.normal(size=555).astype(np.float32)
    params, _ = model.get_params()
    g_gpu, loss_gpu = model.gradients(X, Y)
    g_cpu, loss_cpu = M.gradients(params, X, Y)
    rel = np.linalg.norm(g_gpu - g_cpu) / np.linalg.norm(g_cpu)
    assert rel < 5e-3, rel
    assert abs(loss_gpu - loss_cpu) <= 1e-3 * loss_cpu
