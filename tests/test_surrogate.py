"""The learned warm start: the GPU forward/backward kernels against the numpy
FP64 oracle (which itself is checked against finite differences), training,
and the warm-started solve keeping parity with the cold one."""
import types

import numpy as np
import pytest


def test_oracle_backward_matches_finite_differences(oracle):
    from oracle import cnn_oracle as co

    rng = np.random.default_rng(0)
    n = co.param_count()
    params = rng.normal(0, 0.3, n) / 3
    feats = rng.normal(0, 1, (2, 3, 33, 33))
    tgts = rng.normal(0, 0.1, (2, 4, 33, 33))
    loss, g = co.loss_and_grads(params, feats, tgts, bf16_mode=False)
    idx = rng.choice(n, 12, replace=False)
    for i in idx:
        e = np.zeros(n)
        e[i] = 1e-5
        lp, _ = co.loss_and_grads(params + e, feats, tgts, bf16_mode=False)
        lm, _ = co.loss_and_grads(params - e, feats, tgts, bf16_mode=False)
        fd = (lp - lm) / 2e-5
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def _fake_torch(current_stream_handle):
    """The few torch calls train() makes before its first step."""
    gen = types.SimpleNamespace(manual_seed=lambda seed: None)
    cuda = types.SimpleNamespace(
        current_stream=lambda: types.SimpleNamespace(cuda_stream=current_stream_handle))
    return types.SimpleNamespace(cuda=cuda, Generator=lambda device=None: gen)


@pytest.mark.parametrize("torch_stream, library_stream", [(0, 1), (0x5a5a00, 0x5a5a00)])
def test_training_runs_on_torchs_stream(pkg, torch_stream, library_stream):
    """train() points the library at torch's current stream for the training
    steps (the mini-batch gathers run there) and restores the previous stream.
    torch's legacy default stream (handle 0) must become cudaStreamLegacy (1):
    a NULL stream would leave the library on its own non-blocking stream, which
    does not wait for the gathers."""
    S = pkg.surrogate
    calls = []
    engine = types.SimpleNamespace(stream_handle=0, set_stream=calls.append)
    sur = types.SimpleNamespace(engine=engine)
    feats = types.SimpleNamespace(shape=(512, 3, 33, 33))
    hist = S.train(sur, feats, None, _fake_torch(torch_stream), epochs=0)
    assert hist == []
    assert calls == [library_stream, 0]
    assert pkg._abi.CUDA_STREAM_LEGACY == 1


def test_param_count_matches_library(built):
    from oracle import cnn_oracle as co

    lib = built._abi.load()
    assert lib.msfem_surrogate_param_count() == co.param_count()


@pytest.mark.gpu
def test_gpu_forward_and_gradients_match_oracle(pkg, engine):
    torch = pytest.importorskip("torch")
    from oracle import cnn_oracle as co

    sur = pkg.surrogate.Surrogate(engine, seed=7)
    rng = np.random.default_rng(1)
    params = (rng.normal(0, 1, sur.n_params) * 0.1).astype(np.float32)
    sur.set_params(params)
    feats = rng.normal(0, 1, (3, 3, 33, 33)).astype(np.float32)
    tgts = rng.normal(0, 0.05, (3, 4, 33, 33)).astype(np.float32)
    f_d = torch.from_numpy(feats).cuda()
    t_d = torch.from_numpy(tgts).cuda()
    out = torch.empty((3, 4, 33, 33), dtype=torch.float32, device="cuda")
    sur.predict(f_d, out)
    ref = co.forward(params.astype(np.float64), feats.astype(np.float64), bf16_mode=True)
    got = out.cpu().numpy()
    # FP32 vs FP64 accumulation can move a hidden activation across a bf16
    # rounding boundary (one bf16 ulp = 2^-8 relative), so single entries may
    # differ by ~1e-3 of the output scale; on average the agreement is ~1e-6
    err = np.abs(got - ref)
    assert err.max() <= 1e-2 * np.abs(ref).max()
    assert err.mean() <= 1e-4 * np.abs(ref).max()
    loss, g = sur.gradients(f_d, t_d)
    lref, gref = co.loss_and_grads(params.astype(np.float64), feats.astype(np.float64),
                                   tgts.astype(np.float64), bf16_mode=True)
    assert abs(loss - lref) <= 1e-3 * lref
    # per layer, relative to the layer's gradient scale (bf16 gradients between layers)
    off = 0
    for ws, bs in co.param_shapes():
        nw, nb = int(np.prod(ws)), int(np.prod(bs))
        for a, b in ((off, off + nw), (off + nw, off + nw + nb)):
            scale = np.abs(gref[a:b]).max()
            assert np.abs(g[a:b] - gref[a:b]).max() <= 2e-2 * scale + 1e-12, (a, b)
        off += nw + nb
    sur.close()


@pytest.mark.gpu
def test_training_reduces_loss_and_warm_start_saves_iterations(pkg, engine):
    torch = pytest.importorskip("torch")
    S = pkg.surrogate
    W = pkg.workloads
    feats, tgts = S.training_set(engine, torch, seeds=[(11, 12, 13), (21, 22, 23)], K=32)
    sur = S.Surrogate(engine, seed=3)
    hist = S.train(sur, feats, tgts, torch, epochs=4, batch=128, lr=1e-3)
    assert hist[-1] < 0.5 * hist[0]
    # warm-started solve on unseen cells: same answer, fewer iterations
    prob = W.fourier_square(K=16, N=32, seeds=(3, 30, 300))
    desc, keep = S.device_problem(engine, prob, torch)
    cold = S.solve_device(engine, desc, torch, tol=1e-10)
    sur.attach()
    warm = S.solve_device(engine, desc, torch, tol=1e-10, warm=pkg._abi.WARM_SURROGATE)
    sur.detach()
    assert warm["stats"]["cells_failed"] == 0
    assert warm["stats"]["max_rel_residual"] < 1e-10
    Mc, Mw = cold["M"].cpu().numpy(), warm["M"].cpu().numpy()
    assert np.abs(Mc - Mw).max() < 1e-10 * np.abs(Mc).max()
    assert warm["stats"]["iterations_total"] < cold["stats"]["iterations_total"]
    sur.close()


@pytest.mark.gpu
def test_predict_is_independent_per_image(pkg, engine):
    """Each image's prediction depends only on that image: a large batch
    (many work items per persistent CTA, prefetched windows, reused tensor
    memory) equals the same images predicted on their own, bit for bit."""
    torch = pytest.importorskip("torch")
    sur = pkg.surrogate.Surrogate(engine, seed=11)
    rng = np.random.default_rng(5)
    B = 1500
    feats = torch.from_numpy(rng.normal(0, 1, (B, 3, 33, 33)).astype(np.float32)).cuda()
    out = torch.empty((B, 4, 33, 33), dtype=torch.float32, device="cuda")
    sur.predict(feats, out)
    assert torch.isfinite(out).all()
    for lo, hi in ((0, 3), (700, 701), (B - 5, B)):
        part = torch.empty((hi - lo, 4, 33, 33), dtype=torch.float32, device="cuda")
        sur.predict(feats[lo:hi].contiguous(), part)
        assert torch.equal(part, out[lo:hi])
    sur.close()


@pytest.mark.gpu
def test_features_match_numpy(pkg, engine):
    """Network input (log a11, a12 / sqrt(a11 a22), log a22 of the tensor
    averaged over each node's fine cells and Gauss points) against a numpy
    restatement from the same tabulated coefficient; FP32 arithmetic on the
    device, so 1e-5 relative to the feature scale."""
    torch = pytest.importorskip("torch")
    S, W = pkg.surrogate, pkg.workloads
    prob = W.subset(W.fourier_square(K=64, N=32), [0, 5, 2047, 4095])
    desc, keep = S.device_problem(engine, prob, torch)
    got = S.features(engine, desc, torch).cpu().numpy()
    tab = engine.tabulate(prob, 3).reshape(4, 3, 4, 32, 32)  # [cell][comp][q][cy][cx]
    cellavg = tab.mean(axis=2)                              # [cell][comp][cy][cx]
    pad = np.zeros((4, 3, 34, 34))
    cnt = np.zeros((34, 34))
    pad[:, :, 1:33, 1:33] = cellavg
    cnt[1:33, 1:33] = 1.0
    # node (iy, ix) averages the fine cells (iy-1..iy, ix-1..ix) that exist
    s = pad[:, :, :-1, :-1] + pad[:, :, 1:, :-1] + pad[:, :, :-1, 1:] + pad[:, :, 1:, 1:]
    c = cnt[:-1, :-1] + cnt[1:, :-1] + cnt[:-1, 1:] + cnt[1:, 1:]
    a = s / c
    ref = np.stack([np.log(a[:, 0]), a[:, 1] / np.sqrt(a[:, 0] * a[:, 2]), np.log(a[:, 2])], axis=1)
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max())
