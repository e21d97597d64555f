"""Staged host transfers (ParticleArray.upload / set_staged / download): the
same values as set / get, with the link overlapped with stepping."""
import numpy as np
import pytest
import torch

import pysph_gb300
from pysph_gb300 import workloads as W

pytestmark = pytest.mark.gpu
API = pysph_gb300.api()
IN = ("x", "y", "z", "u", "v", "w")
OUT = ("x", "y", "z", "u", "v", "w", "rho", "p")


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")


def test_upload_and_download_round_trip():
    _need_gpu()
    props = W.cube_lattice(4096, seed=1, vel_std=0.3)
    pa = API.base.get_particle_array(name="fluid", **props)
    rng = np.random.default_rng(7)
    vals = {p: rng.standard_normal(4096) for p in ("u", "v")}
    pinned = {"u": torch.from_numpy(vals["u"]).pin_memory(), "v": vals["v"]}   # one pageable
    up = pa.upload(**pinned)
    pa.set_staged(up)
    dl = pa.download("u", "v", "x")
    u, v, x = dl.result()
    assert np.array_equal(u, vals["u"]) and np.array_equal(v, vals["v"])
    assert np.array_equal(x, props["x"])
    # the download is a snapshot: later writes do not reach it
    dl = pa.download("u")
    pa.set(u=np.zeros(4096))
    assert np.array_equal(dl.result(), vals["u"])
    assert np.array_equal(pa.get("u"), np.zeros(4096))


def test_upload_errors():
    _need_gpu()
    pa = API.base.get_particle_array(name="fluid", x=np.zeros(8), y=np.zeros(8))
    with pytest.raises(ValueError):
        pa.upload(x=np.zeros(7))
    with pytest.raises(ValueError):
        pa.upload(tag=np.zeros(8, np.int64))
    up = pa.upload(x=np.ones(8))
    pa.set_staged(up)
    with pytest.raises(ValueError):
        pa.set_staged(up)
    other = API.base.get_particle_array(name="other", x=np.zeros(8))
    with pytest.raises(ValueError):
        other.set_staged(pa.upload(x=np.ones(8)))


def test_staged_loop_matches_serial_loop():
    """The bench's end-to-end loop, staged and serial: every step uploads the
    same state, integrates one RK2 step and reads the results back; both
    loops return the same arrays bit for bit."""
    _need_gpu()
    props = W.cube_lattice(32768, seed=3, vel_std=0.5)
    s, particles = W.setup_cube(API, props)
    integ = s.integrator
    pa = particles.arrays[0]
    integ.integrate(1e-4)
    host = {f: torch.from_numpy(pa.get(f)).pin_memory() for f in IN}
    steps = 6
    serial = []
    for _ in range(steps):
        pa.set(**host)
        integ.integrate(1e-4)
        serial.append(pa.get(*OUT))
    staged = []
    up = pa.upload(**host)
    pending = None
    for k in range(steps):
        pa.set_staged(up)
        if k + 1 < steps:
            up = pa.upload(**host)
        integ.integrate(1e-4)
        dl = pa.download(*OUT)
        if pending is not None:
            staged.append(pending.result())
        pending = dl
    staged.append(pending.result())
    for a, b in zip(serial, staged):
        for p, x, y in zip(OUT, a, b):
            assert np.array_equal(x, y), p
