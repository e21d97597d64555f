"""Edge cases of the neighbour search and the pair passes: a single
particle, isolated particles, coincident particles, an empty source array,
and an extent too large for the grid."""
import numpy as np
import pytest
import torch

import oracle
import pysph_gb300
from golden_util import csr_sets, normwise

pytestmark = pytest.mark.gpu
API = pysph_gb300.api()
base, sph, solver = API.base, API.sph, API.solver
Fluid = base.ParticleType.Fluid


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")


def _props(x, y, h=0.1, m=1.0, u=None, v=None):
    n = len(x)
    return {"x": np.asarray(x, float), "y": np.asarray(y, float), "h": np.full(n, h),
            "m": np.full(n, m), "rho": np.ones(n), "p": np.zeros(n), "cs": np.zeros(n),
            "u": np.zeros(n) if u is None else np.asarray(u, float),
            "v": np.zeros(n) if v is None else np.asarray(v, float)}


def _rho_and_pgrad(props, sources=None):
    """SPHRho and SPHPressureGradient of ``fluid`` through SPHCalc (and the
    oracle's values over its own lists)."""
    n = len(props["x"])
    extra = {"ax": np.zeros(n), "ay": np.zeros(n)}
    pa = base.get_particle_array(name="fluid", type=Fluid, **props, **extra)
    arrays = [pa] + list(sources or [])
    particles = base.Particles(arrays=arrays)
    kern = base.CubicSplineKernel(dim=2)
    srcs = [pa] + list(sources or [])
    calc = sph.SPHCalc(particles, srcs, pa, kern,
                       [sph.SPHRho.get_func(s, pa) for s in srcs], ["rho"])
    calc.sph("rho")
    pa.set(p=np.linspace(1.0, 2.0, n))
    calc = sph.SPHCalc(particles, srcs, pa, kern,
                       [sph.SPHPressureGradient.withargs(dim=2).get_func(s, pa) for s in srcs],
                       ["ax", "ay"])
    calc.sph("ax", "ay")
    return pa


def _oracle(props):
    st = dict(props)
    st["p"] = np.linspace(1.0, 2.0, len(props["x"]))
    off, idx = oracle.neighbors(st, st, 2.0 * st["h"].max(), same=True)
    rho = oracle.pair_sum("rho", props, props, off, idx, 2, nout=1)[0]
    st["rho"] = rho
    ax, ay = oracle.pair_sum("pgrad", st, st, off, idx, 2, nout=2)
    return off, idx, rho, ax, ay


def test_single_particle_sees_itself_only():
    _need_gpu()
    props = _props([0.3], [0.7])
    pa = _rho_and_pgrad(props)
    off, idx, rho, ax, ay = _oracle(props)
    assert idx.tolist() == [0]
    assert normwise(pa.get("rho"), rho) < 1e-6
    assert not pa.get("ax").any() and not pa.get("ay").any()   # no self force


def test_isolated_and_coincident_particles():
    """Three isolated particles (far beyond 2h of each other) and a pair at
    one position: W(0) from the partner, no force between coincident
    particles (r = 0), exactly as the oracle."""
    _need_gpu()
    x = [0.0, 1.0, 2.0, 3.0, 3.0]
    y = [0.0, 0.0, 0.0, 0.5, 0.5]
    props = _props(x, y)
    pa = _rho_and_pgrad(props)
    off, idx, rho, ax, ay = _oracle(props)
    particles_sets = csr_sets(off, idx)
    assert particles_sets[:3] == [{0}, {1}, {2}] and particles_sets[3] == {3, 4}
    assert normwise(pa.get("rho"), rho) < 1e-6
    np.testing.assert_allclose(pa.get("rho")[3], 2 * pa.get("rho")[0], rtol=1e-6)
    assert not pa.get("ax").any() and not pa.get("ay").any()


def test_empty_source_array_adds_nothing():
    """A second, empty array among the sources (a boundary with no particles
    yet): the sums are those over the fluid alone."""
    _need_gpu()
    rng = np.random.default_rng(3)
    n = 400
    props = _props(rng.uniform(0, 1, n), rng.uniform(0, 1, n), h=0.06, m=0.0025)
    empty = base.get_particle_array(name="wall", type=base.ParticleType.Solid,
                                    **_props([], []))
    pa = _rho_and_pgrad(props, sources=[empty])
    off, idx, rho, ax, ay = _oracle(props)
    assert normwise(pa.get("rho"), rho) < 1e-5
    assert normwise(pa.get("ax"), ax) < 1e-5 and normwise(pa.get("ay"), ay) < 1e-5


def test_extent_beyond_the_grid_limit_raises():
    """Two particles 10^6 smoothing lengths apart in 3D would need more than
    2^27 dense cells: the build fails with a RuntimeError, nothing faults."""
    _need_gpu()
    props = _props([0.0, 1e5], [0.0, 1e5])
    props["z"] = np.array([0.0, 1e5])
    pa = base.get_particle_array(name="fluid", type=Fluid, **props)
    with pytest.raises(RuntimeError, match="grid cells"):
        base.Particles(arrays=[pa])
