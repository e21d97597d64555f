"""The bench's workload at its full size: the 3D jittered lattice of
1 000 000 particles (100^3, h = 1.2 dx), SPHRho + Tait + PGrad + AV +
stepping, RK2.  Exact neighbour lists, one step against the FP64 oracle, and
size-independent properties over many steps."""
import numpy as np
import pytest
import torch

import oracle
import pysph_gb300
from golden_util import normwise
from pysph_gb300 import workloads as W

pytestmark = pytest.mark.gpu
API = pysph_gb300.api()
N = 1_000_000
DT = 1e-4
TOL = 1e-5


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")


def test_bench_workload_lists_and_rk2_step_match_oracle():
    _need_gpu()
    props = W.cube_lattice(N, seed=0)
    s, particles = W.setup_cube(API, props)
    pa = particles.arrays[0]
    # every neighbour list, index for index (ascending, self last)
    off, idx = oracle.neighbors(props, props, 2.0 * props["h"].max(), same=True)
    loc = particles.nnps_manager.get_neighbor_particle_locator(pa, pa, 2.0)
    goff, gidx = loc.neighbour_csr()
    assert np.array_equal(goff, off)
    assert np.array_equal(gidx, idx)
    del goff, gidx, off, idx
    s.integrator.integrate(DT)
    prob = oracle.Problem({"fluid": props}, oracle.cube_ops(), dim=3)
    prob.integrate_rk2(DT)
    ref = prob.arrays["fluid"]
    for p in ("rho", "p", "cs"):
        assert normwise(pa.get(p), ref[p]) < TOL, p
    for p in ("x", "y", "z", "u", "v", "w"):
        assert normwise(pa.get(p) - props[p], ref[p] - props[p]) < TOL, p


def test_bench_workload_conserves_mass_and_momentum():
    """20 RK2 steps (light refreshes and full builds): the total mass does
    not change in any bit; the pressure gradient and the artificial
    viscosity are antisymmetric in each pair, so the total momentum stays
    at its initial value up to the FP32 rounding of the pair sums."""
    _need_gpu()
    props = W.cube_lattice(N, seed=0, vel_std=0.05)
    s, particles = W.setup_cube(API, props)
    inv0 = particles.invariants()
    scale = float(np.sum(props["m"] * np.sqrt(props["u"] ** 2 + props["v"] ** 2 +
                                              props["w"] ** 2)))
    for _ in range(20):
        s.integrator.integrate(DT)
    inv = particles.invariants()
    assert inv["mass"] == inv0["mass"]
    dp = float(np.linalg.norm(np.asarray(inv["momentum"]) - np.asarray(inv0["momentum"])))
    assert dp / scale < 1e-6, dp / scale
    full, light = particles.cell_manager.build_stats()
    assert light > 0


def test_dam_break_full_size_matches_oracle():
    """The dam break at its full size (20 000 fluid particles at dx = 0.01,
    three layers of walls, gravity, boundary force), five RK2 steps at the
    stable dt of this configuration (2.5e-5) against the FP64 oracle."""
    _need_gpu()
    dx = 0.01
    fluid, wall = W.dam_break(dx=dx)
    assert len(fluid["x"]) == 20000
    c0 = W.dam_break_c0()
    s, particles = W.setup_dam_break(API, fluid, wall, dx, c0)
    prob = oracle.Problem({"fluid": fluid, "boundary": wall}, oracle.dam_ops(dx, c0), dim=2)
    for _ in range(5):
        s.integrator.integrate(2.5e-5)
        prob.integrate_rk2(2.5e-5)
    pa = particles.arrays[0]
    ref = prob.arrays["fluid"]
    for p in ("rho", "p"):
        assert normwise(pa.get(p), ref[p]) < TOL, p
    n = len(fluid["x"])
    for p in ("x", "y", "u", "v"):
        init = fluid.get(p, np.zeros(n))      # the column starts at rest
        assert normwise(pa.get(p) - init, ref[p] - init) < 1e-4, p
