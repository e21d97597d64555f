"""Learned momentum closure on the GPU: the tensor-core network kernels
against the FP64 oracle (forward, gradients, Adam), the feature gather
against the oracle's neighbour ordering, and the closure in a solver."""
import ctypes

import numpy as np
import pytest
import torch

import pysph_gb300
from oracle import mlp as M
from pysph_gb300 import learned as L
from pysph_gb300 import native
from pysph_gb300 import workloads as W

pytestmark = pytest.mark.gpu
API = pysph_gb300.api()


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _model(seed, bias=0.1):
    rng = np.random.default_rng(seed)
    p = M.init_params(seed)
    p[M.OFF_B1:M.OFF_W2] = rng.normal(0, bias, M.NH)
    p[M.OFF_B2:M.OFF_W3] = rng.normal(0, bias, M.NH)
    p[M.OFF_B3:] = rng.normal(0, bias, M.NOUT)
    model = L.MomentumMLP(device="cuda")
    model.set_params(p)
    return model, model.params.cpu().numpy().astype(np.float64)


def _x(n, seed):
    rng = np.random.default_rng(seed)
    x = torch.tensor(rng.normal(0, 1, (n, M.NIN)), dtype=torch.float32).to(torch.bfloat16)
    return x.cuda().contiguous(), x.to(torch.float64).numpy()


@pytest.mark.parametrize("n", [1, 128, 300, 5000])
def test_forward_matches_oracle(n):
    _need_gpu()
    model, p = _model(1)
    xg, xh = _x(n, 2)
    y, cache = model.forward(xg, save=True)
    torch.cuda.synchronize()
    model.check()
    yr, c = M.forward(p, xh)
    assert _rel(y.cpu().numpy(), yr) < 1e-3
    assert _rel(cache["z1"].cpu().numpy(), c["z1"]) < 1e-5
    assert _rel(cache["z2"].cpu().numpy(), c["z2"]) < 1e-3
    assert _rel(cache["h1"].float().cpu().numpy(), c["h1"]) < 1e-3
    # inference without the saved values gives the same outputs
    y2 = model.forward(xg)
    assert torch.equal(y, y2)


@pytest.mark.parametrize("n", [200, 4096, 20000])
def test_gradient_matches_oracle(n):
    """The GPU gradient (tensor-core products, FP32 accumulation) against
    the FP64 oracle with the same BF16 rounding points."""
    _need_gpu()
    model, p = _model(3)
    xg, xh = _x(n, 4)
    rng = np.random.default_rng(5)
    t = rng.normal(0, 1, (n, M.NOUT))
    tg = torch.tensor(t, dtype=torch.float32, device="cuda")
    y, cache = model.forward(xg, save=True)
    g, loss = model.backward(xg, cache, y, tg)
    torch.cuda.synchronize()
    model.check()
    lr, gr = M.backward(p, xh, t.astype(np.float32).astype(np.float64))
    g = g.cpu().numpy()
    for name, a, b in (("W1", M.OFF_W1, M.OFF_B1), ("b1", M.OFF_B1, M.OFF_W2),
                       ("W2", M.OFF_W2, M.OFF_B2), ("b2", M.OFF_B2, M.OFF_W3),
                       ("W3", M.OFF_W3, M.OFF_B3), ("b3", M.OFF_B3, M.NPARAM)):
        assert _rel(g[a:b], gr[a:b]) < 5e-3, (name, _rel(g[a:b], gr[a:b]))
    assert abs(float(loss.item()) - lr) / lr < 1e-4


def test_gradient_deterministic():
    _need_gpu()
    model, _ = _model(6)
    xg, _ = _x(3000, 7)
    tg = torch.randn(3000, 2, device="cuda")
    y, cache = model.forward(xg, save=True)
    g1 = model.backward(xg, cache, y, tg)[0].clone()
    g2 = model.backward(xg, cache, y, tg)[0].clone()
    assert torch.equal(g1, g2)


def test_adam_matches_oracle():
    _need_gpu()
    model, p = _model(8)
    xg, xh = _x(512, 9)
    tg = torch.randn(512, 2, device="cuda")
    m = np.zeros(M.NPARAM)
    v = np.zeros(M.NPARAM)
    for step in range(1, 4):
        y, cache = model.forward(xg, save=True)
        g, _ = model.backward(xg, cache, y, tg)
        gh = g.cpu().numpy().astype(np.float64)
        model.adam(1e-3)
        p, m, v = M.adam(p, gh, m, v, step, 1e-3)
    got = model.params.cpu().numpy()
    assert np.max(np.abs(got - p)) < 1e-6
    # the BF16 copies follow the FP32 parameters
    w1 = model.w1.float().cpu().numpy()
    assert np.array_equal(w1, M.bf16(got[M.OFF_W1:M.OFF_B1]).astype(np.float32))
    w2t = model.w2t.float().cpu().numpy().reshape(M.NH, M.NH)
    assert np.array_equal(w2t.T.ravel(), model.w2.float().cpu().numpy())


def test_training_fits_a_teacher_network():
    """Train against targets of a fixed random network: the loss falls by
    well over an order of magnitude."""
    _need_gpu()
    teacher, _ = _model(10, bias=0.3)
    xg, _ = _x(65536, 11)
    t = teacher.forward(xg)
    t = (t - t.mean(0)) / t.std(0)
    model = L.MomentumMLP(seed=12)
    losses = L.train(model, xg, t.contiguous(), epochs=20, batch=2048, lr=2e-3)
    assert losses[-1] < 0.1 * losses[0], losses


def _jittered_drop(seed=0, dx=0.05):
    props = W.elliptical_drop(dx=dx, c0=100.0, radius=0.6)
    rng = np.random.default_rng(seed)
    n = len(props["x"])
    props["x"] = props["x"] + rng.uniform(-0.1, 0.1, n) * dx
    props["y"] = props["y"] + rng.uniform(-0.1, 0.1, n) * dx
    props["u"] = props["u"] + rng.normal(0, 1, n)
    return props


def test_features_match_oracle():
    _need_gpu()
    props = _jittered_drop()
    s, particles = W.setup_drop(API, props, c0=100.0)
    integ = s.integrator
    integ.integrate(1e-5)            # a step, so rho and p are the device's
    cm = particles.cell_manager
    pa = particles.arrays[0]
    norm = L.Normalisation(100.0)
    # a density pass at the current positions refreshes the sorted state
    stage = integ.stages[0]
    integ.cstep = 1
    stage.run(integ, "k1")
    raw = L.features(cm, pa, norm, raw=True).cpu().numpy()
    host = {k: pa.get(k) for k in ("x", "y", "u", "v", "h", "rho", "p")}
    want = M.features(host, 100.0, np.zeros(6), np.ones(6))
    assert raw.shape == want.shape
    np.testing.assert_allclose(raw, want, rtol=1e-5, atol=2e-5)
    # standardised BF16 rows are the rounded standardised values
    fm = np.array([0.1, -0.2, 0.01, 0.02, 1.0, 5.0])
    fs = np.array([0.9, 0.8, 0.3, 0.4, 0.01, 20.0])
    bf = L.features(cm, pa, L.Normalisation(100.0, fm, fs)).float().cpu().numpy()
    want_s = M.features(host, 100.0, fm, 1.0 / fs)
    np.testing.assert_allclose(bf, M.bf16(want_s), rtol=1e-2, atol=1e-3)


def _feature_state():
    props = _jittered_drop()
    s, particles = W.setup_drop(API, props, c0=100.0)
    integ = s.integrator
    integ.integrate(1e-5)
    integ.cstep = 1
    integ.stages[0].run(integ, "k1")
    return particles.cell_manager, particles.arrays[0]


def test_closure_apply_matches_formula():
    """sph_mlp_apply: a_c = (y_c scale_c + mean_c) c0^2 / h on LocalReal
    particles (FP32 arithmetic, FP64 store), added to or replacing acc."""
    _need_gpu()
    cm, pa = _feature_state()
    n = pa.get_number_of_particles()
    rng = np.random.default_rng(3)
    y = torch.tensor(rng.normal(0, 1, (n, 2)), dtype=torch.float32, device="cuda")
    c0, scale, mean = 100.0, (0.7, 1.3), (-0.05, 0.2)
    h = pa.get("h").astype(np.float64)
    real = pa.get("tag") == 0
    want = [np.where(real, (y.cpu().numpy()[:, c].astype(np.float64) * scale[c] + mean[c])
                     * c0 * c0 / h, 0.0) for c in range(2)]
    base = [torch.tensor(rng.normal(0, 1, n), dtype=torch.float64, device="cuda")
            for _ in range(3)]
    for accumulate in (0, 1):
        acc = [b.clone() for b in base]
        ptrs = (ctypes.c_void_p * 3)(*[a.data_ptr() for a in acc])
        native.check(native.lib().sph_mlp_apply(
            cm.context(), cm.slot(pa), ctypes.c_void_p(y.data_ptr()), c0,
            (ctypes.c_double * 2)(*scale), (ctypes.c_double * 2)(*mean), ptrs, accumulate),
            "sph_mlp_apply")
        torch.cuda.synchronize()
        for c in range(2):
            exp = want[c] + (base[c].cpu().numpy() if accumulate else 0.0)
            got = acc[c].cpu().numpy()
            assert np.max(np.abs(got - exp)) <= 1e-6 * np.max(np.abs(exp)), (accumulate, c)
        if accumulate:
            assert torch.equal(acc[2], base[2])
        else:
            assert torch.count_nonzero(acc[2]) == 0


def test_feature_kernels_agree(monkeypatch):
    """The warp-per-destination feature kernel (a bitonic sort of each chunk
    of 32 listed neighbours) and the thread-per-destination one give the
    same rows, bit for bit, raw and standardised."""
    _need_gpu()
    cm, pa = _feature_state()
    norm = L.Normalisation(100.0, np.array([0.1, -0.2, 0.01, 0.02, 1.0, 5.0]),
                           np.array([0.9, 0.8, 0.3, 0.4, 0.01, 20.0]))
    out = {}
    for thread in ("1", "0"):
        monkeypatch.setenv("SPH_FEATURES_THREAD", thread)
        out[thread] = (L.features(cm, pa, norm, raw=True).clone(),
                       L.features(cm, pa, norm).clone())
    assert torch.equal(out["1"][0], out["0"][0])
    assert torch.equal(out["1"][1], out["0"][1])
    assert float((out["0"][0] != 0).any(dim=1).float().mean()) > 0.5


_FEAT_OVERFULL = r"""
import sys
sys.path.insert(0, ".")
sys.path.insert(0, "tests")
import os, torch
import test_gpu_mlp as T
from pysph_gb300 import learned as L
cm, pa = T._feature_state()
rows = {}
for thread in ("1", "0"):
    os.environ["SPH_FEATURES_THREAD"] = thread
    rows[thread] = L.features(cm, pa, L.Normalisation(100.0), raw=True).clone()
assert torch.equal(rows["1"], rows["0"])
print("ok")
"""


def test_feature_kernels_agree_on_overfull_lists():
    """Lists shorter than the neighbour counts (completed by the traversal,
    each neighbour inserted into the warp's sorted set): same rows as the
    thread-per-destination kernel, in a fresh process."""
    _need_gpu()
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, SPH_LIST_CAP="9")
    r = subprocess.run([sys.executable, "-c", _FEAT_OVERFULL], cwd=root, env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr[-3000:]


def _small_dam(dx=0.04):
    fluid, wall = W.dam_break(dx=dx)
    c0 = W.dam_break_c0()
    s, particles = W.setup_dam_break(API, fluid, wall, dx, c0)
    return s, particles, c0


def test_closure_records_trains_and_steps():
    _need_gpu()
    s, particles, c0 = _small_dam()
    fluid = particles.arrays[0]
    n = fluid.get_number_of_particles()
    rec = L.SampleRecorder(s.integrator, fluid, c0, capacity=40 * n, every=1)
    for _ in range(20):
        s.integrator.integrate(1e-4)
    rec.detach()
    x, t, norm = rec.finish()
    assert rec.count == 40 * n
    assert torch.isfinite(t).all() and torch.isfinite(x.float()).all()
    model = L.MomentumMLP(seed=0)
    losses = L.train(model, x, t, epochs=6, batch=2048, lr=2e-3)
    assert losses[-1] < losses[0]
    closure = L.LearnedClosure(s.integrator, fluid, model, norm)
    runner = L.GuardedRunner(s, particles, closure, k=5, tol=1.0)
    runner.window(1e-4)
    runner.window(1e-4)
    assert runner.checks == 2 and runner.fallbacks == 0
    assert np.isfinite(fluid.get("u")).all() and np.isfinite(fluid.get("rho")).all()
    assert np.isfinite(runner.max_err)


def test_guarded_runner_restores_exactly():
    """Re-running a window with the plain pair loop from its saved start
    reproduces it bit for bit (the density difference of a window whose
    closure is inactive is exactly zero)."""
    _need_gpu()
    import types
    s, particles, c0 = _small_dam()
    fluid = particles.arrays[0]
    for _ in range(5):
        s.integrator.integrate(1e-4)
    dummy = types.SimpleNamespace(active=False, dest=fluid)
    runner = L.GuardedRunner(s, particles, dummy, k=4, tol=0.0)
    runner.window(1e-4)
    runner.window(1e-4)
    assert runner.checks == 2 and runner.max_err == 0.0 and runner.fallbacks == 0
    assert runner.kept == 2 and runner.stats()["fallback_rate"] == 0.0


def test_trained_network_beats_no_network():
    """What the trained network gains: over 10 steps of the small dam
    break, the closure's density error against the plain pair loop is well
    below that of the same solver with the fluid-on-itself pressure
    gradient + viscosity left out (a zero network)."""
    _need_gpu()
    s, particles, c0 = _small_dam()
    fluid = particles.arrays[0]
    n = fluid.get_number_of_particles()
    rec = L.SampleRecorder(s.integrator, fluid, c0, capacity=200 * n, every=1)
    for _ in range(100):
        s.integrator.integrate(1e-4)
    rec.detach()
    x, t, norm = rec.finish()
    model = L.MomentumMLP(seed=0)
    L.train(model, x, t, epochs=10, batch=4096, lr=2e-3)
    zero = L.MomentumMLP(seed=0)
    zero.set_params(np.zeros(M.NPARAM))
    start = [{p: pa.get_device(p).clone() for p in L.STATE_PROPS if pa.has_array(p)}
             for pa in particles.arrays]

    def run(net):
        for pa, st in zip(particles.arrays, start):
            pa.set(**st)
        particles.cell_manager.skip_jump_once = True
        particles.update()
        closure = None
        if net is not None:
            closure = L.LearnedClosure(s.integrator, fluid, net, norm)
        for _ in range(10):
            s.integrator.integrate(1e-4)
        if closure is not None:
            closure.detach()
        return fluid.get_device("rho").clone()

    plain = run(None)
    err_net = float(((run(model) - plain).abs() / plain).max())
    err_zero = float(((run(zero) - plain).abs() / plain).max())
    print("density error: trained %.3g, without the term %.3g" % (err_net, err_zero))
    assert err_net < 0.5 * err_zero
