"""CPU tests of the proposal network's oracle: its hand-written backward against finite
differences and against torch autograd (float64), and its BF16 rounding helper."""
import numpy as np
import pytest

from oracle import cnn_oracle as CO


def _problem(n=4, seed=0):
    rng = np.random.default_rng(seed)
    p = CO.init_params(seed + 1).astype(np.float64)
    x0 = rng.normal(0, 1, (n, 31, 31, 2))
    t = rng.normal(0, 1, (n, 6)) * np.array([3, 3, .01, .01, .01, .01])
    return p, x0, t


def test_backward_matches_finite_differences():
    p, x0, t = _problem()
    _, g, _ = CO.loss_and_grad(p, x0, t, bf=False)
    rng = np.random.default_rng(9)
    for name, (o, size) in CO.LAYOUT.items():
        for idx in o + rng.choice(size, 2, replace=False):
            e = 1e-6
            pp, pm = p.copy(), p.copy()
            pp[idx] += e
            pm[idx] -= e
            fd = (CO.loss_and_grad(pp, x0, t, bf=False)[0] - CO.loss_and_grad(pm, x0, t, bf=False)[0]) / (2 * e)
            assert abs(fd - g[idx]) <= 1e-6 + 1e-5 * abs(g[idx]), (name, idx, fd, g[idx])


def test_backward_matches_torch_autograd():
    torch = pytest.importorskip("torch")
    p, x0, t = _problem(n=3, seed=2)
    loss, g, _ = CO.loss_and_grad(p, x0, t, bf=False)
    P = CO.unpack(p)
    names = [("w", 0), ("b", 0), ("w", 1), ("b", 1), ("w", 2), ("b", 2), ("w", 3), ("b", 3)]
    ts = [torch.tensor(P[k][i], dtype=torch.float64, requires_grad=True) for k, i in names]
    ts += [torch.tensor(P[k], dtype=torch.float64, requires_grad=True) for k in ("w5", "b5", "w6", "b6")]
    h = torch.tensor(x0).permute(0, 3, 1, 2)
    for l in range(4):
        h = torch.relu(torch.nn.functional.conv2d(h, ts[2 * l].permute(0, 3, 1, 2), ts[2 * l + 1], stride=2, padding=1))
    h = h.permute(0, 2, 3, 1).reshape(x0.shape[0], 128)
    h = torch.relu(h @ ts[8].T + ts[9])
    o = h @ ts[10].T + ts[11]
    L = ((o - torch.tensor(t * CO.SCALE)) ** 2).sum() / (x0.shape[0] * 6)
    L.backward()
    gt = CO.pack_grads({"w": [ts[i].grad.numpy() for i in (0, 2, 4, 6)], "b": [ts[i].grad.numpy() for i in (1, 3, 5, 7)],
                        "w5": ts[8].grad.numpy(), "b5": ts[9].grad.numpy(), "w6": ts[10].grad.numpy(),
                        "b6": ts[11].grad.numpy()})
    assert abs(L.item() - loss) < 1e-12 * max(1.0, loss)
    assert np.linalg.norm(gt - g) <= 1e-12 * np.linalg.norm(g)


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.0078125, 3.14159265, -2.5e-3, 65504.0], dtype=np.float32)
    r = CO.bf16(x)
    # values exactly representable stay; others round to the nearest BF16 (8 significant bits)
    assert r[0] == 1.0 and r[2] == 1.0078125
    assert r[1] in (1.0, 1.0078125)
    assert abs(r[3] - 3.140625) < 1e-12
    assert np.all(np.abs(r - x) <= np.abs(x) * 2 ** -8)
