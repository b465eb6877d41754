"""Learned warm start: the network kernels against the CPU oracle
(oracle/pcn_ref.py), training, and what the trained network gains.

CPU: the oracle's backward pass against finite differences of its forward
pass (FP64, no BF16 rounding), and its BF16 rounding rule.
GPU: features (1e-6), forward and backward against the oracle with the same
BF16 rounding points (tolerances set by BF16 resolution, 2^-8: an
accumulation-order difference can move a stored activation by one BF16 step),
loss (1e-9), a short training run that lowers the loss, and the committed
trained weights against the cold start on held-out geometries.
"""
import os

import numpy as np
import pytest
import torch

from oracle import pcn_ref as R

WEIGHTS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "electrodrive_gb300", "data",
                       "pcn_weights.npz")


def _problem(n, seed):
    rng = np.random.default_rng(seed)
    c = rng.normal(size=(n, 3))
    nr = rng.normal(size=(n, 3))
    nr /= np.linalg.norm(nr, axis=1, keepdims=True)
    a = rng.uniform(0.5, 1.5, n) / n
    b = rng.normal(size=n)
    s = rng.uniform(0.5, 2.0, n) * np.sign(b)
    sigma = s * (1 + 0.3 * rng.normal(size=n))
    return c, nr, a, b, s, sigma


def test_bf16_rounding_rule():
    x = np.array([1.0, 1.00390625, 1.0078125, 3.14159265, -2.5e-3, 0.0], np.float32)
    y = R.bf16(x)
    assert y[0] == 1.0 and y[1] == 1.0 and y[2] == 1.0078125  # ties to even
    assert abs(y[3] - 3.140625) < 1e-7 and abs(y[4] / -2.5e-3 - 1) < 2 ** -8


def test_oracle_gradients_match_finite_differences():
    c, nr, a, b, s, sigma = _problem(40, 0)
    f = R.features(c, nr, a, b).astype(np.float64)
    theta = R.init(1).astype(np.float64)
    theta[R.NPARAMS - 129:R.NPARAMS - 1] = np.random.default_rng(2).normal(0, 0.1, 128)  # a live output layer

    def L(t):
        y, _ = R.forward(t, f, emulate_bf16=False)
        return R.loss(y, s, sigma, a)[0]

    y, cache = R.forward(theta, f, emulate_bf16=False)
    _, dy = R.loss(y, s, sigma, a)
    g = R.backward(theta, cache, dy, emulate_bf16=False)
    rng = np.random.default_rng(3)
    idx = rng.choice(R.NPARAMS, 60, replace=False)
    idx = np.concatenate([idx, [R.NPARAMS - 1, 0, 5]])
    for i in idx:
        h = 1e-6
        tp, tm = theta.copy(), theta.copy()
        tp[i] += h
        tm[i] -= h
        fd = (L(tp) - L(tm)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, g[i])


@pytest.mark.gpu
def test_features_forward_backward_match_oracle(cuda_lib):
    from electrodrive_gb300.core.warm_start import PointCloudNet

    n = 3000
    c, nr, a, b, s, sigma = _problem(n, 5)
    theta = R.init(7)
    theta[R.NPARAMS - 129:R.NPARAMS - 1] = np.random.default_rng(8).normal(0, 0.05, 128).astype(np.float32)
    net = PointCloudNet(theta)
    T = lambda x: torch.as_tensor(x, device="cuda")
    f = net.features(T(c), T(nr), T(a), T(b))
    fr = R.features(c, nr, a, b)
    assert np.abs(f.cpu().numpy() - fr).max() < 1e-5
    y = net.forward(f)
    yr, cache = R.forward(theta, fr)
    yg = y.cpu().numpy()
    assert np.linalg.norm(yg - yr) <= 1e-2 * np.linalg.norm(yr)
    l, dy = net.loss(y, T(s), T(sigma), T(a))
    lr_, dyr = R.loss(yg.astype(np.float64), s, sigma, a)
    assert abs(float(l) - lr_) <= 1e-9 * lr_
    assert np.abs(dy.cpu().numpy() - dyr).max() <= 1e-6 * np.abs(dyr).max()
    g = net.backward(dy).cpu().numpy()
    gr = R.backward(theta, cache, dyr)
    for name, (lo, hi) in _blocks().items():
        err = np.linalg.norm(g[lo:hi] - gr[lo:hi]) / max(np.linalg.norm(gr[lo:hi]), 1e-30)
        assert err < 3e-2, (name, err)


def _blocks():
    out, o = {}, 0
    for name, shape in R._SHAPES:
        k = int(np.prod(shape))
        out[name] = (o, o + k)
        o += k
    return out


@pytest.mark.gpu
def test_training_lowers_the_loss(cuda_lib):
    from electrodrive_gb300.core.warm_start import KINDS, PointCloudNet, make_sample, random_case, train

    rng = np.random.default_rng(0)
    samples = [make_sample(*random_case(rng, KINDS[i % 4], 1500)) for i in range(8)]
    net = PointCloudNet(seed=0)
    hist = train(net, samples, epochs=40, lr=2e-3)
    assert hist[-1] < 0.5 * hist[0], hist[::8]


@pytest.mark.gpu
@pytest.mark.skipif(not os.path.exists(WEIGHTS), reason="no trained weights committed")
def test_trained_network_against_the_cold_start(cuda_lib):
    """Held-out geometries (seeds the training never used) of 10k-20k panels
    on the FMM operator.  What the network gains: a start far closer to the
    converged density than the cold start (b / I_self) and than the base
    guess it corrects (b / A(1)), and from it fewer FP64 refinement steps of
    the mixed FP32/FP64 solver (the cold start needs two on every geometry,
    the learned start one: 2.0 against 1.01 on the 100 held-out geometries of
    the training report).  Plain Jacobi GMRES iterations barely move on these
    systems (the first iterations remove the smooth error the network
    predicts, the rest go to the rest of the spectrum), so they are only
    checked to converge.  Every start reaches the same true residual."""
    from electrodrive_gb300.core.warm_start import KINDS, PointCloudNet, compare_starts, make_sample, random_case

    net = PointCloudNet.load(WEIGHTS)
    rng = np.random.default_rng(987654)
    res = []
    for i in range(8):
        mesh, spec = random_case(rng, KINDS[i % 4], int(rng.integers(10000, 20000)))
        res.append(compare_starts(net, make_sample(mesh, spec, operator="fmm")))
    for r in res:
        for k in ("cold", "base", "learned"):
            assert r[k]["code"] == 0 and r[k]["rel_resid"] <= 1e-6 * (1 + 1e-9)
            m = r[k]["mixed"]
            assert m["code"] == 0 and m["rel_resid"] <= 1e-6 * (1 + 1e-9), (k, m)
    err = {k: np.mean([r[k]["start_error"] for r in res]) for k in ("cold", "base", "learned")}
    outer = {k: np.mean([r[k]["mixed"]["outer"] for r in res]) for k in ("cold", "base", "learned")}
    fp64 = {k: np.mean([r[k]["mixed"]["fp64_matvecs"] for r in res]) for k in ("cold", "base", "learned")}
    assert err["learned"] < 0.5 * err["base"] and err["learned"] < 0.01 * err["cold"], err
    assert outer["learned"] <= outer["cold"] - 0.75 and outer["learned"] <= outer["base"], outer
    assert fp64["learned"] <= fp64["cold"] - 0.75 and fp64["learned"] <= fp64["base"], fp64


@pytest.mark.gpu
@pytest.mark.skipif(not os.path.exists(WEIGHTS), reason="no trained weights committed")
def test_bem_solve_with_the_learned_start(cuda_lib):
    """bem_solve(mixed=True, warm_start=net): the same density as the cold
    mixed solve (both stop at a 1e-6 relative FP64 residual) in fewer
    refinement steps."""
    from electrodrive_gb300.core.bem import bem_solve
    from electrodrive_gb300.core.warm_start import PointCloudNet, random_case
    from electrodrive_gb300.utils.config import BEMConfig

    net = PointCloudNet.load(WEIGHTS)
    mesh, spec = random_case(np.random.default_rng(4242), "torus", 12000)
    kw = dict(mesh=mesh, operator="fmm", self_integral="quadrature", mixed=True, mixed_rtol=1e-6)
    cold = bem_solve(spec, BEMConfig(), **kw)
    learned = bem_solve(spec, BEMConfig(), warm_start=net, **kw)
    for r in (cold, learned):
        assert "error" not in r and r["gmres_stats"]["precision"] == "mixed", r.get("error")
    a, c = np.asarray(mesh.areas), np.asarray(cold["surface_charge_density"])
    d = np.asarray(learned["surface_charge_density"]) - c
    assert np.sqrt((a * d * d).sum() / (a * c * c).sum()) < 1e-4
    assert learned["gmres_stats"]["outer"] < cold["gmres_stats"]["outer"], (learned["gmres_stats"]["outer"],
                                                                            cold["gmres_stats"]["outer"])
