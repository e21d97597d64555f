"""Long runs against the FP64 oracle: mass stays exact, and total momentum
and kinetic energy of the FP32-pair-sum run are reported against the FP64
run of the same steps (printed; bounded here)."""
import numpy as np
import pytest
import torch

import oracle
import pysph_gb300
from pysph_gb300 import workloads as W

pytestmark = pytest.mark.gpu
API = pysph_gb300.api()


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")


def _host_invariants(a):
    m = a["m"]
    u, v = a["u"], a["v"]
    w = a.get("w", np.zeros_like(u))
    return {"mass": float(np.sum(m)),
            "momentum": np.array([np.sum(m * u), np.sum(m * v), np.sum(m * w)]),
            "kinetic_energy": float(np.sum(0.5 * m * (u * u + v * v + w * w)))}


def _report(name, rows):
    print("\n%s: step, |dP| / sum m|v|, dKE / KE (GPU FP32 pairs vs FP64 oracle)" % name)
    for r in rows:
        print("  %5d  %.3e  %.3e" % r)


def _compare(gpu_inv, ref_arrays, scale):
    ref = _host_invariants(ref_arrays)
    dp = float(np.linalg.norm(gpu_inv["momentum"] - ref["momentum"])) / scale
    dk = abs(gpu_inv["kinetic_energy"] - ref["kinetic_energy"]) / ref["kinetic_energy"]
    return dp, dk


def test_drop_long_run_invariants():
    """Elliptical drop (c0 = 100), 200 Euler steps."""
    _need_gpu()
    props = W.elliptical_drop(dx=0.025, c0=100.0)
    s, particles = W.setup_drop(API, props, c0=100.0)
    prob = oracle.Problem({"fluid": props}, oracle.drop_ops(c0=100.0), dim=2)
    m0 = particles.invariants()["mass"]
    scale = float(np.sum(props["m"] * np.hypot(props["u"], props["v"])))
    rows = []
    for k in range(1, 201):
        s.integrator.integrate(1e-5)
        prob.integrate_euler(1e-5)
        if k % 50 == 0:
            inv = particles.invariants()
            assert inv["mass"] == m0                      # bit for bit
            rows.append((k,) + _compare(inv, prob.arrays["fluid"], scale))
    _report("drop", rows)
    for _, dp, dk in rows:
        assert dp < 1e-5 and dk < 1e-4


def test_dam_break_long_run_invariants():
    """Dam break (dx = 0.04), 300 RK2 steps with gravity and walls."""
    _need_gpu()
    dx = 0.04
    fluid, wall = W.dam_break(dx=dx)
    c0 = W.dam_break_c0()
    s, particles = W.setup_dam_break(API, fluid, wall, dx, c0)
    prob = oracle.Problem({"fluid": fluid, "boundary": wall}, oracle.dam_ops(dx, c0), dim=2)
    fl = particles.arrays[0]
    m0 = particles.invariants(fl)["mass"]
    rows = []
    for k in range(1, 301):
        s.integrator.integrate(1e-4)
        prob.integrate_rk2(1e-4)
        if k % 100 == 0:
            inv = particles.invariants(fl)
            assert inv["mass"] == m0
            a = prob.arrays["fluid"]
            scale = float(np.sum(a["m"] * np.hypot(a["u"], a["v"])))
            rows.append((k,) + _compare(inv, a, scale))
    _report("dam break", rows)
    for _, dp, dk in rows:
        assert dp < 1e-3 and dk < 1e-3
