"""Deferred check of light neighbour refreshes: the integrators' updates
return before the device has checked the refresh, the next pair pass is
launched gated and repeated after a full build when the lists were stale.
Results must be those of the synchronous update, bit for bit."""
import numpy as np
import pytest
import torch

import oracle
import pysph_gb300
from golden_util import csr_sets
from pysph_gb300 import workloads as W

pytestmark = pytest.mark.gpu
API = pysph_gb300.api()
PROPS = ("x", "y", "z", "u", "v", "w", "rho", "p", "cs")


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")


def _drop(deferred, steps, integrator, monkeypatch):
    monkeypatch.setenv("PYSPH_GB300_SKIN", "0.05")
    # the deferred check belongs to steps run call by call (a recorded step
    # replayed as a graph gates its launches on the refresh's verdict itself)
    monkeypatch.setenv("PYSPH_GB300_GRAPHS", "0")
    props = W.elliptical_drop(dx=0.025, c0=100.0)
    s, particles = W.setup_drop(API, props, c0=100.0, integrator=integrator)
    cm = particles.cell_manager
    assert cm.deferred_check      # set up by the integrator
    cm.set_deferred_check(deferred)
    for _ in range(steps):
        s.integrator.integrate(1e-5)
    pa = particles.arrays[0]
    out = {k: pa.get(k) for k in PROPS}
    return out, cm.build_stats(), cm.deferred_stats()


@pytest.mark.parametrize("integrator", ["euler", "rk2"])
def test_deferred_matches_synchronous(integrator, monkeypatch):
    """The fast drop moves past half the skin every few steps: deferred
    refreshes found stale are replaced at their first pass by the build the
    synchronous update makes, so every array matches exactly."""
    _need_gpu()
    a, st_a, df_a = _drop(True, 40, integrator, monkeypatch)
    b, st_b, df_b = _drop(False, 40, integrator, monkeypatch)
    assert df_b == (0, 0), df_b
    assert df_a[0] > 0 and df_a[1] > 0, df_a      # deferred refreshes, some stale
    assert st_a == st_b, (st_a, st_b)              # same full builds and light refreshes
    for p in PROPS:
        assert np.array_equal(a[p], b[p]), p


def test_deferred_jump_reported_by_next_pass():
    """A particle moved by more than one cell: the deferred update returns,
    the density pass reports the jump and writes nothing."""
    _need_gpu()
    props = W.elliptical_drop(dx=0.05, c0=100.0)
    s, particles = W.setup_drop(API, props, c0=100.0)
    s.integrator.integrate(1e-6)
    pa = particles.arrays[0]
    cm = particles.cell_manager
    rho0 = pa.get("rho")
    x = pa.get("x")
    x[5] += 2.5 * cm.cell_size
    pa.set(x=x)
    with pytest.raises(RuntimeError, match="more than one cell"):
        s.integrator.integrate(1e-6)
    assert np.array_equal(pa.get("rho"), rho0)


def test_pending_refresh_resolved_by_neighbour_export():
    """A deferred update found stale, followed directly by the neighbour
    export: the export reads the verdict first and sees the full build."""
    _need_gpu()
    props = W.cube_lattice(32768, seed=3, vel_std=0.5)
    s, particles = W.setup_cube(API, props)
    s.integrator.integrate(1e-4)
    pa = particles.arrays[0]
    cm = particles.cell_manager
    full0, _ = cm.build_stats()
    # every particle by 0.3 of the search radius: far past half the skin,
    # within one cell
    x = pa.get("x")
    x += 0.6 * pa.get("h")
    pa.set(x=x)
    cm.update()
    loc = particles.nnps_manager.get_neighbor_particle_locator(pa, pa, 2.0)
    off, idx = loc.neighbour_csr()
    n_def, n_stale = cm.deferred_stats()
    assert n_stale >= 1 and n_def >= n_stale
    assert cm.build_stats()[0] == full0 + 1
    host = {k: pa.get(k) for k in ("x", "y", "z", "h")}
    ro, ri = oracle.neighbors(host, host, 2.0 * host["h"].max(), 2.0, same=True)
    assert csr_sets(off, idx) == csr_sets(ro, ri)
