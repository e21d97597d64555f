"""Batched independent simulations against the same simulations run one by
one through the solver API, and against the oracle."""
import numpy as np
import pytest
import torch

import oracle
import pysph_gb300
from golden_util import normwise
from pysph_gb300 import workloads as W
from pysph_gb300.batch import SimulationBatch

pytestmark = pytest.mark.gpu
TOL = 1e-5
API = pysph_gb300.api()


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")


def _drops(count, seed=0):
    return W.drop_batch(count, seed=seed, max_particles=3000, c0=100.0)


@pytest.mark.parametrize("graph", [True, False])
def test_batch_matches_single_runs(graph):
    _need_gpu()
    drops = _drops(6, seed=1)
    steps = 5
    batch = SimulationBatch(drops, dim=2, dt=1e-5, co=100.0, use_graph=graph)
    batch.step(steps)
    for k, props in enumerate(drops):
        s, particles = W.setup_drop(API, props, c0=100.0)
        for _ in range(steps):
            s.integrator.integrate(1e-5)
        pa = particles.arrays[0]
        for p in ("x", "y", "u", "v"):
            got = batch.get(k, p) - props[p]
            ref = pa.get(p) - props[p]
            assert normwise(got, ref) < TOL, (k, p, normwise(got, ref))
        for p in ("rho", "p"):
            assert normwise(batch.get(k, p), pa.get(p)) < TOL, (k, p)


def test_batch_instances_vs_oracle():
    _need_gpu()
    drops = _drops(3, seed=2)
    batch = SimulationBatch(drops, dim=2, dt=1e-5, co=100.0)
    batch.step(3)
    for k, props in enumerate(drops):
        prob = oracle.Problem({"fluid": props}, oracle.drop_ops(c0=100.0), dim=2)
        for _ in range(3):
            prob.integrate_euler(1e-5)
        ref = prob.arrays["fluid"]
        for p in ("x", "v"):
            assert normwise(batch.get(k, p) - props[p], ref[p] - props[p]) < TOL, (k, p)
        assert normwise(batch.get(k, "rho"), ref["rho"]) < TOL


def test_batch_rk2_from_solvers():
    _need_gpu()
    drops = _drops(4, seed=3)
    solvers = [W.setup_drop(API, p, c0=100.0, integrator="rk2") for p in drops]
    batch = SimulationBatch.from_solvers(solvers, dt=1e-5)
    assert batch.recipe.scheme == 1
    batch.step(2)
    for k, (s, particles) in enumerate(solvers):
        for _ in range(2):
            s.integrator.integrate(1e-5)
        pa = particles.arrays[0]
        for p in ("x", "u"):
            assert normwise(batch.get(k, p) - drops[k][p], pa.get(p) - drops[k][p]) < TOL


def test_batch_reports_particles_leaving_their_grid():
    _need_gpu()
    drops = _drops(2, seed=4)
    batch = SimulationBatch(drops, dim=2, dt=1e-5, co=100.0, margin=0.0)
    # push instance 1 far outside its region through the device arrays
    a, b = int(batch.offsets[1]), int(batch.offsets[2])
    batch.arrays["u"][a:b] = 1e5
    with pytest.raises(RuntimeError):
        batch.step(3)


def test_batch_staged_transfers_match_set_and_get():
    """SimulationBatch.upload / set_staged / download: the same state and
    results as set / step / get_all, with the copies on copy streams."""
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from pysph_gb300 import workloads as W
    from pysph_gb300.batch import SimulationBatch
    drops = [W.elliptical_drop(dx=0.05, radius=r, c0=100.0) for r in (0.6, 1.0, 1.3)]
    batch = SimulationBatch(drops, dim=2, dt=1e-5, co=100.0)
    batch.step(2)
    fin = ("x", "y", "u", "v")
    fout = ("x", "y", "u", "v", "rho", "p")
    host = {f: torch.from_numpy(batch.get_all(f)).pin_memory() for f in fin}
    serial = []
    for _ in range(3):
        batch.set(**host)
        batch.step(1)
        serial.append(batch.get_all(*fout))
    staged = []
    up = batch.upload(**host)
    pending = None
    for k in range(3):
        batch.set_staged(up)
        if k < 2:
            up = batch.upload(**host)
        batch.step(1)
        dl = batch.download(*fout)
        if pending is not None:
            staged.append(pending.result())
        pending = dl
    staged.append(pending.result())
    for a, b in zip(serial, staged):
        for p, x, y in zip(fout, a, b):
            assert np.array_equal(x, y), p
    with pytest.raises(ValueError):
        batch.upload(q=np.zeros(batch.n))


@pytest.mark.parametrize("integrator", ["euler", "rk2"])
def test_batch_regions_follow_the_instances(integrator):
    """Regions re-derived as the drops deform (a small margin: several
    re-derivations, each after a step stopped on the device and repeated)
    give the same trajectories, bit for bit, as regions that never change
    (cell boundaries, and so the sorted order and the neighbour order, do
    not depend on the region)."""
    _need_gpu()
    drops = _drops(4, seed=5)
    kw = dict(dim=2, dt=1e-5, co=100.0, integrator=integrator)
    moving = SimulationBatch(drops, margin=0.01, **kw)
    fixed = SimulationBatch(drops, margin=2.0, **kw)
    # the edges move by up to ~1e-3 per step: past the four cells of
    # padding within a few hundred steps
    for _ in range(8):
        moving.step(75)
        fixed.step(75)
    st = moving.stats()
    assert st["regrids"] >= 1 and st["steps"] == 600, st
    assert fixed.stats()["regrids"] == 0
    assert st["cells"] < fixed.stats()["cells"]
    for p in ("x", "y", "u", "v", "rho", "p"):
        np.testing.assert_array_equal(moving.get_all(p), fixed.get_all(p), err_msg=p)


def test_batch_per_instance_subdivisions():
    """Instances with cell subdivisions 1, 2 and 3 in one batch (one pair
    launch per group) against the same drops run one by one."""
    _need_gpu()
    drops = _drops(6, seed=6)
    subdiv = [3, 1, 2, 1, 3, 2]
    batch = SimulationBatch(drops, dim=2, dt=1e-5, co=100.0, subdiv=subdiv)
    assert batch.stats()["groups"] == 3
    batch.step(4)
    for k, props in enumerate(drops):
        s, particles = W.setup_drop(API, props, c0=100.0)
        for _ in range(4):
            s.integrator.integrate(1e-5)
        pa = particles.arrays[0]
        for p in ("x", "y", "u", "v"):
            assert normwise(batch.get(k, p) - props[p], pa.get(p) - props[p]) < TOL, (k, p)
        for p in ("rho", "p"):
            assert normwise(batch.get(k, p), pa.get(p)) < TOL, (k, p)
    with pytest.raises(ValueError):
        SimulationBatch(drops, dim=2, dt=1e-5, co=100.0, subdiv=[1, 2])


def test_autotune_chooses_per_instance():
    _need_gpu()
    from pysph_gb300 import tuning
    drops = _drops(12, seed=7)
    choice, report = tuning.autotune_batch(drops, steps=2, dim=2, dt=1e-5, co=100.0)
    assert len(choice) == 12 and set(choice) <= {1, 2, 3}
    assert report["bins"] and "per_instance" in report["whole_batch_ms_per_step"]
    batch = SimulationBatch(drops, dim=2, dt=1e-5, co=100.0, subdiv=choice)
    batch.step(2)
    batch.check()
