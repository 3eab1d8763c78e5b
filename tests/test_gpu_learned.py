"""The learned range surrogate: tensor-core GEMM, gradients against a CPU
restatement, training on rays from the exact marcher, and the learned query."""
import numpy as np
import pytest

from range_libc_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def bf16(x):
    """Round float32 to bfloat16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


@pytest.mark.parametrize("M,N,K,a_t,b_t", [(128, 256, 64, 0, 0), (256, 512, 192, 0, 0), (256, 256, 128, 1, 0),
                                           (128, 256, 256, 0, 1), (256, 512, 640, 1, 1)])
def test_tensor_core_gemm(rl, M, N, K, a_t, b_t):
    rng = np.random.default_rng(M + N + K + a_t * 2 + b_t)
    a = bf16(rng.standard_normal((M, K)).astype(np.float32))
    b = bf16(rng.standard_normal((N, K)).astype(np.float32))
    dev = torch.device("cuda:0")
    ta = torch.from_numpy(np.ascontiguousarray(a.T if a_t else a)).to(dev).to(torch.bfloat16)
    tb = torch.from_numpy(np.ascontiguousarray(b.T if b_t else b)).to(dev).to(torch.bfloat16)
    c = rl.tc_gemm(ta, tb, M, N, K, bool(a_t), bool(b_t))
    torch.cuda.synchronize()
    exp = (a.astype(np.float64) @ b.astype(np.float64).T)
    got = c.cpu().numpy()
    assert np.allclose(got, exp, rtol=1e-4, atol=1e-3), np.abs(got - exp).max()


KHID, KFEAT = 256, 512


def _layers(p):
    """(W [out, in], b) of the 4 hidden layers and the output (w, b) from the flat parameters."""
    out, off = [], 0
    for l in range(4):
        fin = KFEAT if l == 0 else KHID
        w = p[off:off + KHID * fin].reshape(KHID, fin)
        off += KHID * fin
        b = p[off:off + KHID]
        off += KHID
        out.append((w, b))
    return out, p[off:off + KHID], p[off + KHID]


def _gelu(z):
    k0, k1 = np.float32(0.7978845608028654), np.float32(0.044715)
    return np.float32(0.5) * z * (np.float32(1) + np.tanh(k0 * (z + k1 * z * z * z)))


def _gelu_grad(z):
    k0, k1 = np.float32(0.7978845608028654), np.float32(0.044715)
    th = np.tanh(k0 * (z + k1 * z * z * z))
    return np.float32(0.5) * (1 + th) + np.float32(0.5) * z * (1 - th * th) * k0 * (1 + 3 * k1 * z * z)


def cpu_gradients(p, X, t):
    """The GPU's forward and backward restated in numpy with the same bf16 rounding points."""
    layers, w_out, b_out = _layers(p)
    n = X.shape[0]
    h, zs, hs = X.astype(np.float32), [], [X.astype(np.float32)]
    for w, b in layers:
        z = (h.astype(np.float64) @ bf16(w).astype(np.float64).T).astype(np.float32) + b
        zb = bf16(z)
        h = bf16(_gelu(zb))
        zs.append(zb)
        hs.append(h)
    y = (h.astype(np.float64) @ w_out.astype(np.float64)).astype(np.float32) + b_out
    e = y - t
    loss = np.mean(np.where(np.abs(e) <= 1, 0.5 * e * e, np.abs(e) - 0.5))
    dy = (np.where(np.abs(e) <= 1, e, np.sign(e)) / n).astype(np.float32)
    grads = []
    d_wout = (dy.astype(np.float64) @ h.astype(np.float64)).astype(np.float32)
    d_bout = np.float32(dy.sum())
    dz = bf16(dy[:, None] * w_out[None, :] * _gelu_grad(zs[3]))
    for l in range(3, -1, -1):
        w, _ = layers[l]
        dw = (dz.astype(np.float64).T @ hs[l].astype(np.float64)).astype(np.float32)
        db = dz.astype(np.float64).sum(0).astype(np.float32)
        grads.append((dw, db))
        if l > 0:
            dh = (dz.astype(np.float64) @ bf16(w).astype(np.float64)).astype(np.float32)
            dz = bf16(dh * _gelu_grad(zs[l - 1]))
    grads = grads[::-1]
    flat = np.concatenate([np.concatenate([dw.ravel(), db]) for dw, db in grads] + [d_wout, [d_bout]])
    return flat.astype(np.float32), loss


@pytest.fixture(scope="module")
def learned_setup(rl):
    occ = W.rect_disk_map(256, 91)
    m = rl.PyOMap(np.ascontiguousarray(occ.T))
    rm = rl.PyRayMarching(m, 100.0)
    return occ, m, rm


@pytest.mark.parametrize("n", [256, 2048])   # 2048 rays: the weight gradients use split-K
def test_gradients_match_cpu_restatement(rl, learned_setup, n):
    _, _, rm = learned_setup
    L = rl.PyLearnedRM(rm, seed=3)
    xyt, t, _ = L.sample_rays(n, seed=11)
    g, loss = L.gradients(xyt, t)
    X = L.features(xyt).float().cpu().numpy()
    exp, exp_loss = cpu_gradients(L.params(), X, t.cpu().numpy())
    assert abs(loss - exp_loss) <= 1e-3 * max(1.0, abs(exp_loss))
    layers, _, _ = _layers(np.arange(len(exp)))
    # compare per parameter block (relative L2 error)
    off = 0
    for l in range(4):
        fin = KFEAT if l == 0 else KHID
        for size in (KHID * fin, KHID):
            a, b = g[off:off + size], exp[off:off + size]
            assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b) + 1e-9, (l, size)
            off += size
    assert np.linalg.norm(g[off:] - exp[off:]) <= 1e-3 * np.linalg.norm(exp[off:]) + 1e-9


def test_gradients_match_fp64_autograd(rl, learned_setup):
    """Independent check: torch autograd of the unrounded fp64 model agrees in direction."""
    _, _, rm = learned_setup
    L = rl.PyLearnedRM(rm, seed=4)
    xyt, t, _ = L.sample_rays(512, seed=12)
    g, _ = L.gradients(xyt, t)
    X = torch.from_numpy(L.features(xyt).float().cpu().numpy()).double()
    p = torch.from_numpy(L.params().astype(np.float64)).requires_grad_(True)
    layers, w_out, b_out = [], None, None
    off = 0
    h = X
    for l in range(4):
        fin = KFEAT if l == 0 else KHID
        w = p[off:off + KHID * fin].view(KHID, fin)
        off += KHID * fin
        b = p[off:off + KHID]
        off += KHID
        z = h @ w.T + b
        h = 0.5 * z * (1 + torch.tanh(0.7978845608028654 * (z + 0.044715 * z ** 3)))
    y = h @ p[off:off + KHID] + p[off + KHID]
    e = y - torch.from_numpy(t.cpu().numpy()).double()
    loss = torch.where(e.abs() <= 1, 0.5 * e * e, e.abs() - 0.5).mean()
    loss.backward()
    ref = p.grad.numpy()
    cos = float(np.dot(g, ref) / (np.linalg.norm(g) * np.linalg.norm(ref)))
    assert cos > 0.99


def test_training_gains_over_untrained(rl, learned_setup):
    occ, m, rm = learned_setup
    trained = rl.PyLearnedRM(rm, seed=5)
    fresh = rl.PyLearnedRM(rm, seed=5)
    xyt, t, rng_exact = trained.sample_rays(32768, first_id=10_000_000, seed=99)   # held out
    loss = trained.train(steps=600, batch=4096, lr=2e-3, seed=21)
    e_fresh = (fresh.predict(xyt) - t).abs().cpu().numpy()
    e_trained = (trained.predict(xyt) - t).abs().cpu().numpy()
    assert np.isfinite(loss)
    assert np.median(e_trained) < 0.5 * np.median(e_fresh)
    # accept rate of the learned query, trained vs untrained
    fs = W.free_cell_queries(occ, 2000, 31)
    ins = torch.from_numpy(np.stack([fs[:, 1], fs[:, 0], fs[:, 2]], 1).astype(np.float32)).cuda()
    ang = torch.from_numpy(W.laser_angles(61)).cuda()
    outs = torch.empty(len(fs) * 61, dtype=torch.float32, device="cuda")
    n_tr = trained.calc_range_repeat_angles(ins, ang, outs)
    n_fr = fresh.calc_range_repeat_angles(ins, ang, outs)
    assert n_tr < n_fr


def test_learned_query_recasts_are_exact(rl, learned_setup):
    occ, m, rm = learned_setup
    L = rl.PyLearnedRM(rm, seed=6)
    L.train(steps=200, batch=4096, lr=2e-3, seed=22)
    fs = W.free_cell_queries(occ, 1500, 41)
    ins = torch.from_numpy(np.stack([fs[:, 1], fs[:, 0], fs[:, 2]], 1).astype(np.float32)).cuda()
    ang = torch.from_numpy(W.laser_angles(61)).cuda()
    outs = torch.empty(len(fs) * 61, dtype=torch.float32, device="cuda")
    acc = torch.empty(len(fs) * 61, dtype=torch.uint8, device="cuda")
    n_rec = L.calc_range_repeat_angles(ins, ang, outs, acc)
    exact = torch.empty_like(outs)
    rm.calc_range_repeat_angles(ins, ang, exact)
    torch.cuda.synchronize()
    a = acc.cpu().numpy().astype(bool)
    o, ex = outs.cpu().numpy(), exact.cpu().numpy()
    assert n_rec == int((~a).sum())
    assert np.array_equal(o[~a], ex[~a])           # recast rays are the exact ranges
    # a hit cell reached at t < max_range can have its corner up to sqrt(2) farther (as in the reference)
    assert np.all(np.isfinite(o)) and np.all(o <= 100.0 + 1.5)


@pytest.mark.parametrize("n", [1, 127, 128, 5000])
def test_fused_forward_matches_layered(rl, learned_setup, n):
    """The fused forward kernel (whole network per 128-ray tile on one SM) gives the layer-by-layer
    GEMM path's predictions bit for bit, for a trained and a ragged number of rays."""
    occ, m, rm = learned_setup
    L = rl.PyLearnedRM(rm, seed=8)
    L.train(steps=50, batch=4096, lr=2e-3, seed=23)
    xyt, _, _ = L.sample_rays(n, first_id=77_000_000, seed=5)
    a = L.predict(xyt).cpu().numpy()
    b = L.predict(xyt, layered=True).cpu().numpy()
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
