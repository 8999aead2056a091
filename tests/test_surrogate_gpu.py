"""GPU tests of the learned gradient surrogate (surrogate.cu, mlp_gemm.cuh)
and of surrogate-driven HMC.

Oracles: float64 numpy matmul for the tensor-core GEMM (BF16 operands are
exact in float64; FP32 accumulation, so 1e-5 relative), PyTorch-CPU FP64
autograd for the training loss and parameter gradients (the forward repeats
the kernel's BF16 rounding points; the backward's BF16 copies of dZ allow 2e-2
relative Frobenius error), and the numpy leapfrog restatement driven by the
surrogate through the host API for a whole trajectory."""
import numpy as np
import pytest

import oracle
from massivemds_gb300 import Engine, flags as F
from massivemds_gb300.hmc import hmc
from massivemds_gb300.surrogate import Surrogate, gemm_bf16
from oracle import hmc_oracle

pytestmark = pytest.mark.gpu


def _bf16_bits(x):
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return ((b + 0x7FFF + ((b >> 16) & 1)) >> 16).astype(np.uint16)


def _bf16_value(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.mark.parametrize("a_t,b_t", [(0, 0), (0, 1), (1, 1)])
def test_gemm_layouts_match_float64(a_t, b_t):
    m, n, k = 128, 192, 96
    rng = np.random.default_rng(10 * a_t + b_t)
    a = _bf16_bits(rng.standard_normal((k, m) if a_t else (m, k)))
    b = _bf16_bits(rng.standard_normal((k, n) if b_t else (n, k)))
    av, bv = _bf16_value(a), _bf16_value(b)
    ref = (av.T if a_t else av) @ (bv if b_t else bv.T)
    c = gemm_bf16(a, b, a_t, b_t, m, n, k)
    assert np.abs(c - ref).max() <= 1e-5 * np.abs(ref).max()


def _clustered(n, p, seed, dim=10, clusters=5):
    rng = np.random.default_rng(seed)
    centres = 3.0 * rng.standard_normal((clusters, dim))
    y = centres[np.arange(n) % clusters] + rng.standard_normal((n, dim))
    delta = np.sqrt(((y[:, None] - y[None]) ** 2).sum(-1))
    x0 = 0.5 * rng.standard_normal((n, p))
    return delta, x0


def _engine(delta, p, tau=1.0):
    e = Engine(p, delta.shape[0], F.FLOAT | F.LEFT_TRUNCATION)
    e.setPairwiseData(delta.astype(np.float32))
    e.setParameters([tau])
    return e


def _exact_gradient(e, x):
    e.updateLocations(-1, x)
    return np.asarray(e.getLogLikelihoodGradient()).reshape(x.shape)


def _harvest(e, s, delta, states, rows, seed):
    rng = np.random.default_rng(seed)
    n, p = delta.shape[0], e.embeddingDimension
    for t in range(states):
        x = rng.standard_normal((n, p))
        s.add_state(x, _exact_gradient(e, x), rows, seed=seed + t)


def test_training_gradients_match_torch_fp64_autograd():
    torch = pytest.importorskip("torch")
    n, p = 300, 2
    delta, _ = _clustered(n, p, 1)
    e = _engine(delta, p)
    s = Surrogate(e, landmarks=64, width=128, layers=2, max_training_rows=2000, seed=3)
    _harvest(e, s, delta, states=4, rows=100, seed=5)
    s.train(20, batch=128, learning_rate=1e-3, seed=1)  # move away from the initial weights
    rows = np.random.default_rng(7).integers(0, 400, 128).astype(np.int32)
    loss = s.batch_gradient(rows)
    info = s.info()
    layers = info["layers"]
    feat, dirs, tgt = s.training_rows(0, 400)
    params = [s.parameters(l) for l in range(layers + 1)]
    grads = [s.parameter_gradients(l) for l in range(layers + 1)]
    s.close()
    e.close()

    def bf16(t):
        return t.to(torch.bfloat16).to(torch.float64)

    X = torch.tensor(feat[rows], dtype=torch.float64)
    D = torch.tensor(dirs[rows], dtype=torch.float64)
    T = torch.tensor(tgt[rows], dtype=torch.float64)
    W = [torch.tensor(w, dtype=torch.float64, requires_grad=True) for w, _ in params]
    B = [torch.tensor(b, dtype=torch.float64, requires_grad=True) for _, b in params]
    h = X
    for l in range(layers):
        wr = W[l] + (bf16(W[l]) - W[l]).detach()
        a = torch.nn.functional.silu(h @ wr.T + B[l])
        h = a + (bf16(a) - a).detach()
    wr = W[layers] + (bf16(W[layers]) - W[layers]).detach()
    alpha = h @ wr.T + B[layers]
    pred = info["scale"] * torch.einsum("rk,rkp->rp", alpha, D)
    ref_loss = ((pred - T / info["target_scale"]) ** 2).sum() / len(rows)
    ref_loss.backward()
    assert abs(loss - ref_loss.item()) <= 1e-3 * ref_loss.item()
    for l in range(layers + 1):
        for got, want in ((grads[l][0], W[l].grad.numpy()), (grads[l][1], B[l].grad.numpy())):
            err = np.linalg.norm(got - want) / np.linalg.norm(want)
            assert err < 2e-2, (l, err)


def _bf16_round(x):
    return _bf16_value(_bf16_bits(np.asarray(x, dtype=np.float32)))


def _network_gradient(s, delta, x):
    """The surrogate gradient evaluated in float64 from the FP32 master
    weights, with the step kernel's BF16 rounding points."""
    info = s.info()
    k, layers = info["landmarks"], info["layers"]
    lm = s.landmarks()
    xf = x.astype(np.float32).astype(np.float64)
    d = np.sqrt(((xf[:, None, :] - xf[None, lm, :]) ** 2).sum(-1))
    dl = delta.astype(np.float32)[:, lm].astype(np.float64)
    feat_d = _bf16_round((d - dl) * info["inv_sigma_r"])
    feat_delta = _bf16_round((dl - info["mu"]) * info["inv_sigma"])
    h = np.concatenate([feat_d, feat_delta], axis=1)
    for l in range(layers):
        w, b = s.parameters(l)
        z = h @ _bf16_round(w).T + b
        h = _bf16_round(z / (1.0 + np.exp(-z)))
    w, b = s.parameters(layers)
    alpha = h @ _bf16_round(w).T + b
    dirs = xf[:, None, :] - xf[None, lm, :]
    return info["scale"] * info["target_scale"] * np.einsum("ik,ikp->ip", alpha, dirs)


@pytest.mark.parametrize("n,p,k,width,layers", [(300, 2, 64, 128, 2), (257, 3, 128, 64, 1), (200, 6, 64, 192, 3)])
def test_fused_step_gradient_matches_network(n, p, k, width, layers):
    delta, _ = _clustered(n, p, 11)
    e = _engine(delta, p)
    s = Surrogate(e, landmarks=k, width=width, layers=layers, max_training_rows=1000, seed=4)
    _harvest(e, s, delta, states=2, rows=200, seed=3)
    s.train(30, batch=128, learning_rate=2e-3, seed=2)
    x = np.random.default_rng(9).standard_normal((n, p))
    got = s.gradient(x)
    want = _network_gradient(s, delta, x)
    s.close()
    e.close()
    assert np.abs(got - want).max() <= 5e-3 * np.abs(want).max()


def _trained_surrogate(e, delta, landmarks=64, width=64, states=6, steps=300, seed=2):
    s = Surrogate(e, landmarks=landmarks, width=width, layers=2, max_training_rows=4000, seed=seed)
    _harvest(e, s, delta, states=states, rows=min(200, delta.shape[0]), seed=seed + 10)
    s.train(steps, batch=128, learning_rate=2e-3, seed=seed)
    return s


def test_surrogate_trajectory_matches_restatement():
    # FP64 engine: the accept uses the exact FP64 potential, so the Hamiltonian
    # difference is compared as tightly as for exact-gradient trajectories.
    n, p, tau, eps, steps, seed = 200, 2, 1.0, 0.003, 10, 13
    delta, x0 = _clustered(n, p, 4)
    e = Engine(p, n, F.LEFT_TRUNCATION)
    e.setPairwiseData(delta)
    e.setParameters([tau])
    s = _trained_surrogate(e, delta)
    res = hmc(e, x0, iterations=1, leapfrog_steps=steps, step_size=eps, seed=seed, surrogate=s,
              harvest_iterations=0, train_steps=0)
    assert res.column("surrogate")[0] == 1.0
    assert res.surrogate_evaluations == steps and res.gradient_evaluations == 2
    x_ref, dh_ref = hmc_oracle.trajectory(delta, x0, tau, eps, steps, seed, iteration=0,
                                          likelihood_gradient=s.gradient)
    s.close()
    e.close()
    assert abs(res.column("delta_h")[0] - dh_ref) < 1e-6
    expected = x_ref if res.column("accepted")[0] == 1.0 else x0
    assert np.abs(res.final_locations - expected).max() <= 1e-8 * max(1.0, np.abs(expected).max())


def test_fallback_to_exact_gradients_when_acceptance_drops():
    n, p = 300, 2
    delta, x0 = _clustered(n, p, 5)
    e = _engine(delta, p)
    s = Surrogate(e, landmarks=64, width=64, layers=2, max_training_rows=1000, seed=1)
    _harvest(e, s, delta, states=1, rows=100, seed=1)
    s.train(1, batch=64, learning_rate=1e-3)
    w, b = s.parameters(2)
    s.set_parameters(2, 1000.0 * w, b)  # a surrogate far from the gradient
    iters, window, steps = 40, 10, 5
    res = hmc(e, x0, iterations=iters, leapfrog_steps=steps, step_size=0.002, seed=4, surrogate=s,
              harvest_iterations=0, train_steps=0, fallback_accept=0.6, fallback_window=window)
    s.close()
    fb = res.fallback_iteration
    assert window - 1 <= fb < iters
    used = res.column("surrogate")
    assert np.all(used[:fb + 1] == 1.0) and np.all(used[fb + 1:] == 0.0)
    assert res.surrogate_evaluations == (fb + 1) * steps
    assert res.gradient_evaluations == 1 + (fb + 1) + (iters - fb - 1) * steps
    # the chain's state is exact whatever drove the trajectories
    ll = oracle.log_likelihood(oracle.sum_of_increments(delta.astype(np.float32), res.final_locations, 1.0), n, 1.0)
    assert abs(res.column("log_likelihood")[-1] - ll) < 1e-5 * abs(ll)
    e.close()


def test_harvest_train_then_surrogate_chain():
    # Mechanics of the surrogate phase: harvest window, training, surrogate
    # trajectories until the end or the fallback, and the evaluation counts.
    n, p = 512, 2
    delta, x0 = _clustered(n, p, 6)
    e = _engine(delta, p)
    s = Surrogate(e, landmarks=128, width=128, layers=2, max_training_rows=20_000, seed=7)
    iters, harvest, steps = 200, 100, 10
    res = hmc(e, x0, iterations=iters, burn_in=harvest, leapfrog_steps=steps, step_size=0.01, adapt_step_size=True,
              seed=8, surrogate=s, harvest_iterations=harvest, harvest_rows=100, train_steps=800, train_batch=256,
              train_learning_rate=2e-3, fallback_window=20)
    info = s.info()
    g_exact = _exact_gradient(e, res.final_locations)
    g_sur = s.gradient(res.final_locations)
    s.close()
    e.close()
    assert info["rows"] == (harvest - harvest // 2) * 100 and info["adam_steps"] == 800
    assert np.isfinite(res.train_loss) and res.train_loss < 2.0  # 2.0 = predicting zero (P = 2)
    used = res.column("surrogate")
    n_surr = int(used.sum())
    assert np.all(used[:harvest] == 0.0)
    fb = res.fallback_iteration
    if fb >= 0:
        assert harvest + 19 <= fb < iters and n_surr == fb - harvest + 1
        assert np.all(used[harvest:fb + 1] == 1.0) and np.all(used[fb + 1:] == 0.0)
    else:
        assert n_surr == iters - harvest
    assert res.surrogate_evaluations == n_surr * steps
    assert res.gradient_evaluations == 1 + (iters - n_surr) * steps + n_surr
    rel = np.linalg.norm(g_sur - g_exact) / np.linalg.norm(g_exact)
    assert rel < 0.9, rel
