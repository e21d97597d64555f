"""Parity at the largest sizes of the 3D throughput configuration: the
jittered lattice at 161^3 = 4,173,281 and 256^3 = 16,777,216 particles
(h = 1.2 dx, SPHRho + Tait + PGrad + AV + stepping, RK2), where absolute
FP32 coordinates would lose the 1e-5 accuracy and the list-streaming kernels
switch to base-5 cell-offset codes (subdivision 2 above 2^23 particles).

Neighbour sets: every destination's count and an order-independent digest
of its source indices (wrap-around sum of a 64-bit mix of each index,
``oracle.neighbor_digest``), so host memory stays linear in the particle
count.  The reference's relation is the FP64 strict test of
base/nnps.pyx:337-353.  One RK2 step (solver/integrator.py:597-645) against
the FP64 oracle, with both kernel families (brick-staged and
list-streaming), at 1e-5 normwise; per-particle relative errors above a
1e-3 max|ref| floor are printed and bounded for the density.
"""
import ctypes

import numpy as np
import pytest
import torch

import oracle
import pysph_gb300
from golden_util import normwise, rel_percentiles
from pysph_gb300 import native
from pysph_gb300 import workloads as W

pytestmark = pytest.mark.gpu
API = pysph_gb300.api()
DT = 1e-4
TOL = 1e-5
CHUNK = 1 << 21          # destinations digested per host copy


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")


def _gpu_digest(particles):
    """Counts and digests of the device's exported lists (sph_nnps_count /
    sph_nnps_fill into device memory, digested on the host in chunks)."""
    cm = particles.cell_manager
    cm.ensure_current()
    L = native.lib()
    ctx = cm.context()
    n = particles.arrays[0].get_number_of_particles()
    dev = torch.device("cuda")
    counts = torch.zeros(n, dtype=torch.int64, device=dev)
    native.check(L.sph_nnps_count(ctx, 0, 0, 2.0, ctypes.c_void_p(counts.data_ptr())), "count")
    off = torch.zeros(n + 1, dtype=torch.int64, device=dev)
    torch.cumsum(counts, 0, out=off[1:])
    index = torch.empty(int(off[-1].item()), dtype=torch.int64, device=dev)
    native.check(L.sph_nnps_fill(ctx, 0, 0, 2.0, ctypes.c_void_p(off.data_ptr()),
                                 ctypes.c_void_p(index.data_ptr())), "fill")
    offh = off.cpu().numpy()
    dig = np.empty(n, np.uint64)
    for a in range(0, n, CHUNK):
        b = min(n, a + CHUNK)
        seg = index[offh[a]:offh[b]].cpu().numpy()
        dig[a:b] = np.add.reduceat(oracle.mix64(seg), offh[a:b] - offh[a])
    del index
    return counts.cpu().numpy(), dig


def _report(name, got, ref):
    p50, p99, mx, cnt = rel_percentiles(got, ref)
    print("%-4s normwise %.2e  per-particle p50 %.2e p99 %.2e max %.2e (%d above floor)"
          % (name, normwise(got, ref), p50, p99, mx, cnt))
    return mx


@pytest.mark.parametrize("n1", [161, 256])
def test_large_lattice_sets_and_rk2_step(n1, monkeypatch):
    _need_gpu()
    n = n1 ** 3
    props = W.cube_lattice(n, seed=0)
    prob = oracle.Problem({"fluid": props}, oracle.cube_ops(), dim=3)
    ccount, cdig = oracle.neighbor_digest(props, props, 2.0 * props["h"].max())
    prob.integrate_rk2(DT)
    ref = prob.arrays["fluid"]
    for bricks in ("1", "0"):
        monkeypatch.setenv("PYSPH_GB300_BRICKS", bricks)
        s, particles = W.setup_cube(API, props)
        gcount, gdig = _gpu_digest(particles)
        assert np.array_equal(gcount, ccount), (bricks, int(np.sum(gcount != ccount)))
        assert np.array_equal(gdig, cdig), (bricks, int(np.sum(gdig != cdig)))
        s.integrator.integrate(DT)
        assert (particles.cell_manager.brick_pass_count() > 0) == (bricks == "1")
        pa = particles.arrays[0]
        print("N = %d, bricks %s, subdivision %d, mean neighbours %.2f"
              % (n, bricks, particles.cell_manager._subdivision(), ccount.mean()))
        for p in ("rho", "p", "cs"):
            got = pa.get(p)
            assert normwise(got, ref[p]) < TOL, (bricks, p, normwise(got, ref[p]))
            mx = _report(p, got, ref[p])
            if p == "rho":
                assert mx < TOL, (bricks, mx)
        for p in ("x", "y", "z", "u", "v", "w"):
            d_got, d_ref = pa.get(p) - props[p], ref[p] - props[p]
            assert normwise(d_got, d_ref) < TOL, (bricks, p, normwise(d_got, d_ref))
            _report("d" + p, d_got, d_ref)
        del s, particles, pa
        torch.cuda.empty_cache()
