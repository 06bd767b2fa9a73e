"""Emulator MLP: the CPU oracle's mathematics (finite differences), the tensor-core kernels against
the oracle (bit for bit on small integers, to fp32 rounding on real values), AdamW, training, the
CUDA-graph query path and the fallback to the plain SAM."""

import numpy as np
import pytest

from oracle import mlp_oracle as MO


def _rand_layers(rng, dims, scale=1.0):
    return [(rng.normal(0, scale / np.sqrt(k), size=(n, k)).astype(np.float32),
             rng.normal(0, 0.1, size=n).astype(np.float32)) for k, n in zip(dims[:-1], dims[1:])]


def test_oracle_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.01171875, -3.0, 1e-20, 65504.0], dtype=np.float32)
    r = MO.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: ties to even gives 1; 1 + 3 * 2^-8 rounds up to 1 + 2^-6
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.015625) and r[3] == -3.0
    assert np.array_equal(MO.from_bf16_bits(MO.bf16_bits(x)), r)


def test_oracle_gradients_match_finite_differences(monkeypatch):
    """With the bf16 roundings switched off the oracle's backward is the exact gradient of its loss."""
    monkeypatch.setattr(MO, "bf16", lambda a: np.asarray(a, dtype=np.float64))
    monkeypatch.setattr(MO, "_sigmoid", lambda z: 1.0 / (1.0 + np.exp(-np.asarray(z, dtype=np.float64))))
    monkeypatch.setattr(MO, "silu", lambda z: z / (1.0 + np.exp(-z)))

    def sg(z):
        s = 1.0 / (1.0 + np.exp(-z))
        return s * (1.0 + z * (1.0 - s))

    monkeypatch.setattr(MO, "silu_grad", sg)
    rng = np.random.default_rng(0)
    dims = [5, 7, 6, 3]
    layers = [(w.astype(np.float64), b.astype(np.float64)) for w, b in _rand_layers(rng, dims)]
    x = rng.normal(size=(9, 5))
    t = rng.normal(size=(9, 3))

    def loss_of(ls):
        _, _, out = MO.forward(ls, x)
        return np.mean((out - t) ** 2)

    # forward and backward still compute in float32: the tolerance is one float32 arithmetic meets
    _, grads = MO.backward(layers, x, t)
    h = 1e-3
    for ll in range(len(layers)):
        for which in (0, 1):
            arr = layers[ll][which]
            num = np.zeros_like(arr)
            for idx in np.ndindex(arr.shape):
                old = arr[idx]
                arr[idx] = old + h
                up = loss_of(layers)
                arr[idx] = old - h
                dn = loss_of(layers)
                arr[idx] = old
                num[idx] = (up - dn) / (2 * h)
            got = grads[ll][which]
            assert np.allclose(got, num, rtol=2e-3, atol=2e-5), (ll, which)


def test_oracle_adamw_first_step():
    p = np.array([1.0, -2.0, 0.5], dtype=np.float32)
    g = np.array([0.1, -0.2, 0.0], dtype=np.float32)
    m1, m2 = np.zeros(3, np.float32), np.zeros(3, np.float32)
    MO.adamw(p, g, m1, m2, 1, 0.01, 0.9, 0.999, 1e-8, 0.1, np.array([True, True, False]))
    # first bias-corrected step moves each entry by lr * sign(g) (plus decay on decayed entries)
    assert np.allclose(p, [1.0 - 0.001 - 0.01, -2.0 + 0.002 + 0.01, 0.5], atol=1e-6)


# ---- GPU ------------------------------------------------------------------------------------------

def _ensemble(dims, members, seed=0):
    from holodeck_gb300.emulator import MLPEnsemble
    return MLPEnsemble(dims, members=members, seed=seed)


def _set_layers(net, layers_per_member):
    flat = np.zeros((net.members, net.n_params), dtype=np.float32)
    for m, layers in enumerate(layers_per_member):
        off = 0
        for w, b in layers:
            n, k = w.shape
            flat[m, off:off + n * k] = w.ravel()
            flat[m, off + n * k:off + n * k + n] = b
            off += n * k + n
    net.load_params(flat)


def _bf16_tensor(a):
    import torch
    return torch.as_tensor(np.asarray(a, dtype=np.float32), device="cuda").to(torch.bfloat16)


@pytest.mark.gpu
@pytest.mark.parametrize("dims,batch", [([16, 32], 200), ([256, 160], 129), ([16, 256], 128), ([64, 48, 32], 300),
                                        ([16, 160], 1)])
def test_forward_exact_on_small_integers(built_lib, dims, batch):
    """Integer weights, biases and inputs: every tensor-core sum is exact, so the output equals the
    oracle bit for bit (checks the TMA boxes, shared-memory layout, descriptors and TMEM read-back,
    including rows and columns the boxes fill with zeros)."""
    import torch
    rng = np.random.default_rng(len(dims) * 1000 + batch)
    E = 2
    net = _ensemble(dims, E)
    layers = [[(rng.integers(-3, 4, size=(n, k)).astype(np.float32), rng.integers(-5, 6, size=n).astype(np.float32))
               for k, n in zip(dims[:-1], dims[1:])] for _ in range(E)]
    if len(dims) > 2:   # keep the hidden layer's SiLU out of the way: only check its pre-activation path
        for m in range(E):
            layers[m][1] = (np.zeros_like(layers[m][1][0]), layers[m][1][1])
    _set_layers(net, layers)
    x = rng.integers(-3, 4, size=(batch, dims[0])).astype(np.float32)
    out = net.forward(_bf16_tensor(x)).cpu().numpy()
    torch.cuda.synchronize()
    net.check_status()
    for m in range(E):
        _, _, exp = MO.forward(layers[m], x)
        assert np.array_equal(out[m], exp), m


@pytest.mark.gpu
@pytest.mark.parametrize("dims,batch", [([16, 32], 1), ([256, 160], 16), ([64, 48, 32], 5), ([16, 256, 256, 160], 3)])
def test_fused_forward_exact_on_small_integers(built_lib, dims, batch):
    """The one-launch fused forward on integer weights, biases and inputs: exact sums, so the outputs
    equal the oracle bit for bit (weight slices of every cluster rank, activation exchange between
    the CTAs, ragged query counts)."""
    import torch
    rng = np.random.default_rng(len(dims) * 100 + batch)
    E = 3
    net = _ensemble(dims, E)
    layers = [[(rng.integers(-3, 4, size=(n, k)).astype(np.float32), rng.integers(-5, 6, size=n).astype(np.float32))
               for k, n in zip(dims[:-1], dims[1:])] for _ in range(E)]
    for m in range(E):   # the SiLU's rounding is not an integer: a zero layer after it keeps sums exact
        for ll in range(1, len(layers[m])):
            layers[m][ll] = (np.zeros_like(layers[m][ll][0]), layers[m][ll][1])
    _set_layers(net, layers)
    x = rng.integers(-3, 4, size=(batch, dims[0])).astype(np.float32)
    out = net.forward_fused(_bf16_tensor(x)).cpu().numpy()
    torch.cuda.synchronize()
    net.check_status()
    for m in range(E):
        _, _, exp = MO.forward(layers[m], x)
        assert np.array_equal(out[m], exp), m


@pytest.mark.gpu
@pytest.mark.parametrize("batch", [1, 7, 16])
def test_fused_forward_matches_tensor_core_forward(built_lib, batch):
    """The emulator's network shape with random weights: the fused forward agrees with the tensor-core
    layers within the bf16 activation rounding (their fp32 sums run in different orders)."""
    import torch
    rng = np.random.default_rng(batch)
    dims = [16, 256, 256, 256, 256, 160]
    E = 4
    net = _ensemble(dims, E)
    _set_layers(net, [_rand_layers(rng, dims) for _ in range(E)])
    x = _bf16_tensor(rng.uniform(-1, 1, size=(batch, 16)))
    ref = net.forward(x).cpu().numpy()
    got = net.forward_fused(x).cpu().numpy()
    net.check_status()
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() <= 1e-2 * np.abs(ref).max(), np.abs(got - ref).max() / np.abs(ref).max()


@pytest.mark.gpu
@pytest.mark.parametrize("k,batch", [(16, 256), (256, 128)])
def test_weight_gradient_exact_on_small_integers(built_lib, k, batch):
    """One linear layer, targets chosen so that d loss / d out is a small integer: the weight and bias
    gradients (split over batch partials and summed) equal the integer sums exactly."""
    import torch
    n = 64
    rng = np.random.default_rng(k + batch)
    net = _ensemble([k, n], 2)
    layers = [[(rng.integers(-2, 3, size=(n, k)).astype(np.float32), rng.integers(-2, 3, size=n).astype(np.float32))]
              for _ in range(2)]
    _set_layers(net, layers)
    x = rng.integers(-3, 4, size=(batch, k)).astype(np.float32)
    q = rng.integers(-3, 4, size=(batch, n)).astype(np.float32)
    out0 = MO.forward(layers[0], x)[2]
    scale = batch * n / 2.0                        # 2 / (B N) is a power of two here
    target = (out0 - scale * q).astype(np.float32)  # d loss / d out = q exactly (member 0)
    loss = net.gradients(_bf16_tensor(x), torch.as_tensor(target, device="cuda")).cpu().numpy()
    grad = net.grad.cpu().numpy()
    net.check_status()
    gw = grad[0, :n * k].reshape(n, k)
    gb = grad[0, n * k:n * k + n]
    assert np.array_equal(gw, q.T @ x)
    assert np.array_equal(gb, q.sum(axis=0))
    assert np.isclose(loss[0], np.mean((scale * q) ** 2), rtol=1e-5)


@pytest.mark.gpu
def test_backward_matches_oracle(built_lib):
    """Three SiLU layers, ragged batch (3 row tiles, 3 gradient partials), two members: loss and every
    gradient against the oracle (fp32 summation order differs; bf16 roundings follow)."""
    import torch
    rng = np.random.default_rng(5)
    dims = [16, 64, 48, 32]
    E, batch = 2, 300
    net = _ensemble(dims, E)
    layers = [_rand_layers(rng, dims) for _ in range(E)]
    for m in range(E):   # weights as the kernels see them (bf16), so the oracle's master = device master
        layers[m] = [(MO.bf16(w), b) for w, b in layers[m]]
    _set_layers(net, layers)
    x = MO.bf16(rng.uniform(-1, 1, size=(batch, 16)).astype(np.float32))
    t = rng.normal(size=(batch, 32)).astype(np.float32)
    loss = net.gradients(_bf16_tensor(x), torch.as_tensor(t, device="cuda")).cpu().numpy()
    grad = net.grad.cpu().numpy()
    out = net._buffers[(batch, True, None)]["out"].cpu().numpy()
    net.check_status()
    for m in range(E):
        exp_loss, grads = MO.backward(layers[m], x, t)
        _, _, exp_out = MO.forward(layers[m], x)
        assert np.abs(out[m] - exp_out).max() <= 2e-3 * np.abs(exp_out).max()
        assert abs(loss[m] - exp_loss) <= 1e-5 * exp_loss
        off = 0
        for (gw, gb), k, n in zip(grads, dims[:-1], dims[1:]):
            got_w = grad[m, off:off + n * k].reshape(n, k)
            got_b = grad[m, off + n * k:off + n * k + n]
            off += n * k + n
            for got, exp in ((got_w, gw), (got_b, gb)):
                assert np.linalg.norm(got - exp) <= 2e-3 * np.linalg.norm(exp) + 1e-12, (m, k, n)


@pytest.mark.gpu
def test_adamw_step_matches_oracle_and_training_converges(built_lib):
    import torch
    rng = np.random.default_rng(9)
    dims = [16, 64, 64, 16]
    net = _ensemble(dims, 3, seed=4)
    p0 = net.params.cpu().numpy().copy()
    x = rng.uniform(-1, 1, size=(256, 16)).astype(np.float32)
    x[:, 6:] = 0.0
    y = np.stack([np.sin(2 * x[:, i % 6]) * np.cos(x[:, (i + 1) % 6]) for i in range(16)], axis=1).astype(np.float32)
    xt, yt = _bf16_tensor(x), torch.as_tensor(y, device="cuda")
    net.train_step(xt, yt, lr=1e-3, weight_decay=0.1)
    g = net.grad.cpu().numpy()
    p1 = net.params.cpu().numpy()
    decay = np.zeros(net.n_params, dtype=bool)
    off = 0
    for k, n in zip(dims[:-1], dims[1:]):
        decay[off:off + n * k] = True
        off += n * k + n
    for m in range(3):
        p = p0[m].copy()
        MO.adamw(p, g[m], np.zeros_like(p), np.zeros_like(p), 1, 1e-3, 0.9, 0.999, 1e-8, 0.1, decay)
        assert np.allclose(p1[m], p, rtol=1e-6, atol=1e-7)
    # bf16 weight copies follow the master weights
    w = net.weights.float().cpu().numpy()
    assert np.array_equal(w[0, :dims[1] * 16], MO.bf16(p1[0, :dims[1] * 16]))
    first = None
    for step in range(400):
        loss = net.train_step(xt, yt, lr=3e-3)
        if first is None:
            first = loss.cpu().numpy()
    last = loss.cpu().numpy()
    net.check_status()
    assert np.all(last < 0.05 * first), (first, last)


@pytest.mark.gpu
def test_emulator_learns_a_library_and_beats_the_baselines(built_lib):
    """A small library of the classic parameter space: the trained ensemble predicts held-out samples
    better than the two answers available without it (the nearest library sample, the library mean),
    its CUDA-graph path agrees with the eager path and answers far faster than the plain SAM, and
    queries outside the box are re-solved by the SAM."""
    import time
    import torch
    from holodeck_gb300 import emulator as EM
    from holodeck_gb300.librarian import PS_Classic_Phenom_Uniform, batch
    nf, nr, shape = 6, 200, (22, 20, 18)
    train = PS_Classic_Phenom_Uniform(nsamples=384, seed=0)
    test = PS_Classic_Phenom_Uniform(nsamples=64, seed=1)
    kw = dict(shapes=shape, nreals=nr, nfreqs=nf, nloudest=1, seed=3, workers=4, waves=2)
    y_tr = EM.library_statistics(batch.run_library(train, **kw))
    y_te = EM.library_statistics(batch.run_library(test, **kw))
    assert np.all(np.isfinite(y_tr)) and np.all(np.isfinite(y_te))
    emu = EM.Emulator(train, nfreqs=nf, members=4, width=128, depth=4, seed=0)
    hist = emu.fit(train.param_samples, y_tr, epochs=250, batch=128, lr=3e-3)
    assert hist[-1] < 0.2 * hist[0]
    mean, spread, inside = emu.predict(test.param_samples)
    assert np.all(inside) and mean.shape == (64, nf, 4)
    err = np.abs(mean - y_te)[..., 1]                      # median log10 hc
    u_tr, u_te = emu.unit(train.param_samples), emu.unit(test.param_samples)
    nn = np.argmin(((u_te[:, None, :] - u_tr[None, :, :]) ** 2).sum(-1), axis=1)
    err_nn = np.abs(y_tr[nn] - y_te)[..., 1]
    err_mean = np.abs(y_tr.mean(axis=0)[None] - y_te)[..., 1]
    assert np.median(err) < 0.5 * np.median(err_nn), (np.median(err), np.median(err_nn))
    assert np.median(err) < 0.25 * np.median(err_mean), (np.median(err), np.median(err_mean))
    g = emu.graphed(64)
    assert np.allclose(g(test.param_samples), mean, rtol=0, atol=1e-9)
    g1 = emu.graphed(1)                                    # the fused one-kernel graph (pinned I/O)
    n1 = emu.native(1)                                     # the same kernel behind one native call
    n4 = emu.native(4)
    for row in test.param_samples[:5]:
        assert np.allclose(g1(row[None]), emu.predict(row[None])[0], rtol=0, atol=1e-2)
        assert np.allclose(n1(row), g1(row[None]), rtol=0, atol=1e-9)
    assert np.allclose(n4(test.param_samples[:3]), emu.graphed(4)(test.param_samples[:3]), rtol=0, atol=1e-9)
    t_emu = EM.timed(g, test.param_samples, repeat=20) / 64
    solve = EM.sam_fallback(train, sam_shape=shape, nreals=nr, nfreqs=nf, seed=3)
    t_sam = EM.timed(solve, test.param_samples[0], repeat=3)
    assert t_sam > 50 * t_emu, (t_sam, t_emu)
    q = test.param_samples[:3].copy()
    q[1, 4] = 20.0                                         # hard_time outside the training box
    stats, by_sam = emu.query(q, fallback=solve, max_spread=np.inf)
    assert list(by_sam) == [False, True, False]
    assert np.array_equal(stats[1], solve(q[1])) and np.array_equal(stats[0], mean[0])
    _, spread_q, _ = emu.predict(q)
    cut = float(np.median(spread_q))
    _, by_spread = emu.query(q, fallback=None, max_spread=cut)
    assert list(by_spread) == list((spread_q > cut) | np.array([False, True, False]))


def test_boundary_space_points_lie_on_faces():
    """Every point of the boundary library has exactly one coordinate at a bound of the box, and all
    coordinates inside it."""
    from holodeck_gb300 import emulator as EM
    from holodeck_gb300.librarian import PS_Classic_Phenom_Uniform
    sp = EM.boundary_space(PS_Classic_Phenom_Uniform, 200, seed=3)
    lo, hi = sp.extrema[:, 0], sp.extrema[:, 1]
    p = sp.param_samples
    assert p.shape == (200, len(sp.param_names))
    assert np.all(p >= lo - 1e-12) and np.all(p <= hi + 1e-12)
    on_face = np.isclose(p, lo, rtol=0, atol=1e-12) | np.isclose(p, hi, rtol=0, atol=1e-12)
    assert np.all(on_face.sum(axis=1) == 1)
    assert sp.param_dict(0)[sp.param_names[0]] == p[0, 0]


def test_residual_scaled_spread_on_the_host():
    """The residual-scaled spread divides each output's member standard deviation by
    max(max_spread, its training-residual scatter): a noisy output no longer flags the query."""
    from holodeck_gb300.emulator import Emulator
    emu = Emulator.__new__(Emulator)
    emu.nfreqs = 1
    emu.lo, emu.hi = np.zeros(2), np.ones(2)
    # members: output 0 (first statistic) spread 0.08 dex, the others 0.01
    base = np.zeros((4, 1, 1, 4))
    base[:, 0, 0, 0] = np.array([0.0, 0.16, 0.0, 0.16]) - 0.08   # std 0.08
    base[:, 0, 0, 1:] = np.array([0.0, 0.02, 0.0, 0.02])[:, None] - 0.01
    emu.predict_members = lambda params: base
    q = np.array([[0.5, 0.5]])
    _, spread, inside = emu.predict(q)
    assert inside.all() and np.isclose(spread[0], 0.08)
    emu.residual_scatter = np.array([0.1, 0.0, 0.0, 0.0])          # output 0 is that noisy anyway
    _, spread_rs, _ = emu.predict(q, residual_scaled=True, max_spread=0.05)
    assert np.isclose(spread_rs[0], 0.05 * 0.08 / 0.1)               # below the threshold: accepted
    emu.residual_scatter = np.zeros(4)
    _, spread_rs, _ = emu.predict(q, residual_scaled=True, max_spread=0.05)
    assert np.isclose(spread_rs[0], 0.08)                            # the plain criterion again
    emu.residual_scatter = None
    with pytest.raises(ValueError):
        emu.predict(q, residual_scaled=True)
