"""GPU tests of the proposal network: forward and gradients against the float64 CPU oracle
(oracle/cnn_oracle.py, itself checked against torch autograd and finite differences in
tests/test_cnn_oracle.py), training on method-generated pairs, and the learned-seed pair
solve (parity with the CPU path, and what the network gains over FFTCC seeding)."""
import numpy as np
import pytest

import dic_checks as C

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_mod():
    return pytest.importorskip("torch")


def test_forward_and_gradient_match_oracle(dic, torch_mod):
    torch = torch_mod
    from fasticgn_gb300.proposal import ProposalNet, init_params
    from oracle import cnn_oracle as CO
    rng = np.random.default_rng(5)
    n = 96
    params = init_params(3)
    x0 = CO.bf16(rng.normal(0.0, 1.0, (n, 31, 31, 2)).astype(np.float32)).astype(np.float32)
    target = (rng.normal(0.0, 1.0, (n, 6)) * np.array([3, 3, .01, .01, .01, .01])).astype(np.float32)
    net = ProposalNet(0, params)
    xd = torch.from_numpy(x0).to(torch.bfloat16).cuda()
    td = torch.from_numpy(target).cuda()
    out = net.forward(xd).cpu().numpy()
    loss, g = net.gradient(xd, td)
    g = g.cpu().numpy().astype(np.float64)
    want_loss, want_g, want_out = CO.loss_and_grad(params, x0, target, bf=True)
    np.testing.assert_allclose(out[:, :6], want_out, rtol=2e-2, atol=2e-2 * np.abs(want_out).max())
    assert abs(loss - want_loss) <= 2e-3 * want_loss
    for name, (o, size) in CO.LAYOUT.items():
        a, b = g[o:o + size], want_g[o:o + size]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        assert rel < 3e-2, (name, rel)
    net.close()


def test_training_reduces_loss(dic, torch_mod):
    from fasticgn_gb300 import proposal
    x0, tg = proposal.training_set(proposal.synthetic_pairs(2, seed=500, size=512), step=4)
    assert x0.shape[0] > 10000
    net = proposal.ProposalNet(0, proposal.init_params(1))
    losses = proposal.train(net, x0, tg, steps=300, batch=1024, lr=2e-3)
    assert np.mean(losses[-20:]) < 0.5 * np.mean(losses[:5]), (losses[:5], losses[-20:])
    net.close()


def test_learned_seed_parity_and_gain(dic, oracle_mod, torch_mod):
    """With the trained weights: learned-seed results agree with the CPU path (FFTCC seed +
    IC-GN) within the parity gate, and the proposal cuts IC-GN iterations."""
    from fasticgn_gb300 import proposal, speckle
    if not proposal.WEIGHTS.exists():
        pytest.skip("no trained weights")
    O = oracle_mod
    pr = speckle.pair_bumps(seed=777, width=768, height=768)
    h, w = pr.ref.shape
    net = proposal.ProposalNet.load()
    e = dic.Engine(15)
    e.set_proposal(net)
    e.set_ref(pr.ref)
    e.set_tar(pr.tar)
    q = dic.grid_queue(w, h, 15, 6)
    ql, rep = e.process_pair_learned(q.copy())
    qf = q.copy()
    e.process_pair(qf)
    pois = O.grid_pois(w, h, 15, 6)
    O.run_pair(pr.ref.astype(np.float32), pr.tar.astype(np.float32), pois, 15)
    cpu = {"u": pois["p"][:, O.P_U], "v": pois["p"][:, O.P_V], "zncc": pois["r"][:, O.R_ZNCC]}
    res = C.compare_frame(cpu, {"u": ql["u"], "v": ql["v"], "zncc": ql["zncc"]})
    assert res["pass"], res
    ok = (ql["zncc"] >= 0.9) & (qf["zncc"] >= 0.9)
    it_learned = ql["iteration"][ok].mean()
    it_fftcc = qf["iteration"][ok].mean()
    assert rep["repaired_candidates"] < 0.05 * len(q), rep
    assert it_learned < it_fftcc, (it_learned, it_fftcc)


@pytest.mark.parametrize("drop", [0, 3])
def test_fused_inference_matches_layerwise(dic, torch_mod, drop):
    """The fused per-tile kernel (dic_cnn_seed; conv2 on tcgen05) gives the layer-by-layer
    GEMM path's outputs, also for an odd queue (a tile with one live POI, a partial MLP batch)."""
    torch = torch_mod
    from fasticgn_gb300 import proposal, speckle
    pr = speckle.pair_bumps(seed=31, width=320, height=320)
    q = dic.grid_queue(320, 320, 15, 9)
    q = q[:len(q) - drop].copy()
    n = len(q)
    net = proposal.ProposalNet(0, proposal.init_params(4))
    rf = torch.from_numpy(pr.ref.astype(np.float32)).cuda()
    tf = torch.from_numpy(pr.tar.astype(np.float32)).cuda()
    qd = torch.from_numpy(q.view(np.uint8).copy()).cuda()
    out = net.forward(net.inputs(rf, tf, qd, n)).cpu().numpy()
    net.seed(rf, tf, qd, n)
    s = qd.cpu().numpy().view(dic.POI_DTYPE)
    got = np.stack([s["u"], s["v"], 100 * s["ux"], 100 * s["uy"], 100 * s["vx"], 100 * s["vy"]], axis=1)
    scale = np.abs(out[:, :6]).max()
    assert np.max(np.abs(got - out[:, :6])) <= 2e-2 * scale, np.max(np.abs(got - out[:, :6]))
    assert np.median(np.abs(got - out[:, :6])) <= 2e-3 * scale


def test_proposal_product_timeout_is_reported(dic, monkeypatch):
    """conv2's tensor-core products never issued (the DIC_TEST_WAIT_FAULT hook) end in the
    kernel's bounded mbarrier wait: the learned pair fails with DIC_ERR_CUDA naming the
    products, TMEM is released, and a fresh engine on the same context solves normally."""
    from fasticgn_gb300 import proposal, speckle, _lib
    pr = speckle.pair_bumps(seed=41, width=320, height=320)
    net = proposal.ProposalNet(0, proposal.init_params(2))
    q = dic.grid_queue(320, 320, 15, 8)

    def run(fault):
        if fault:
            monkeypatch.setenv("DIC_TEST_WAIT_FAULT", "2")
        e = dic.Engine(15)
        monkeypatch.delenv("DIC_TEST_WAIT_FAULT", raising=False)
        e.set_proposal(net)
        e.set_ref(pr.ref)
        e.set_tar(pr.tar)
        try:
            return e.process_pair_learned(q.copy())
        finally:
            e.close()

    want, _ = run(False)
    with pytest.raises(_lib.DicError) as info:
        run(True)
    assert info.value.code == _lib.DIC_ERR_CUDA and "tensor-core product" in str(info.value)
    got, _ = run(False)
    np.testing.assert_array_equal(got.view(np.uint8), want.view(np.uint8))
    net.close()
