"""The allocation-free invariant sums against the context-based ones.

``sph_invariants_noalloc`` serves callers that cannot allocate device
memory: real-time loops that forbid allocation after start-up, and hosts
whose own allocator reserves all device memory.  It keeps its scratch in a
fixed device array inside the library.  This file is collected last so that
a failure here comes after every other test has run; it also passes on its
own in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

RTOL = 1e-12   # FP64 sums in a different order than sph_invariants


def _setup(n, seed):
    import pysph_gb300
    from pysph_gb300 import workloads as W
    api = pysph_gb300.api()
    props = W.cube_lattice(n, seed=seed)
    pa = api.base.get_particle_array(name="fluid", **props)
    particles = api.base.Particles(arrays=[pa])
    return pa, particles


def _noalloc(pa):
    from pysph_gb300 import native
    from pysph_gb300.base.cell import array_view
    v = array_view(pa)
    out = (ctypes.c_double * 6)()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    native.check(native.lib().sph_invariants_noalloc(ctypes.byref(v), out, stream),
                 "sph_invariants_noalloc")
    return np.array(out[:])


def _context(particles):
    inv = particles.invariants()
    return np.array([inv["mass"], *inv["momentum"], inv["kinetic_energy"], inv["count"]])


def _close(a, b):
    scale = np.maximum(np.abs(b), 1e-300)
    return np.all(np.abs(a - b) <= RTOL * np.maximum(scale, np.abs(b).max()))


def test_noalloc_matches_context_version_on_consecutive_calls():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    big, pbig = _setup(64000, seed=11)
    small, psmall = _setup(8000, seed=12)
    ref_big, ref_small = _context(pbig), _context(psmall)
    # two calls in a row on the same array, then one on a smaller array that
    # reuses fewer scratch slots than the call before it
    first = _noalloc(big)
    second = _noalloc(big)
    third = _noalloc(small)
    assert _close(first, ref_big), (first, ref_big)
    assert _close(second, ref_big), (second, ref_big)
    np.testing.assert_array_equal(first, second)
    assert _close(third, ref_small), (third, ref_small)
    assert first[5] == 64000 and third[5] == 8000


def test_noalloc_rejects_arrays_beyond_its_scratch():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from pysph_gb300 import native
    v = native.ArrayView()
    v.n = (1 << 24) + 1
    out = (ctypes.c_double * 6)()
    rc = native.lib().sph_invariants_noalloc(ctypes.byref(v), out, None)
    assert rc == native.SPH_ERR_ARG
    assert "16777216" in native.last_error()


def test_noalloc_counts_only_local_real_particles():
    """Non-LocalReal particles (ghosts, remote copies) are left out of every
    sum, as in sph_invariants."""
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    pa, particles = _setup(8000, seed=13)
    tag = np.zeros(8000, dtype=np.int64)
    tag[::7] = 1
    tag[3::11] = 2
    pa.set(tag=tag)              # align_particles moves the non-real ones to the end
    real = pa.get("tag", only_real_particles=False) == 0
    assert real.size == 8000 and 0 < real.sum() < 8000
    m, u, v, w = (pa.get(k, only_real_particles=False) for k in ("m", "u", "v", "w"))
    want = np.array([m[real].sum(), (m * u)[real].sum(), (m * v)[real].sum(),
                     (m * w)[real].sum(), (0.5 * m * (u * u + v * v + w * w))[real].sum(),
                     float(real.sum())])
    got = _noalloc(pa)
    ref = _context(particles)
    assert got[5] == real.sum() and ref[5] == real.sum()
    assert _close(got, ref), (got, ref)
    assert _close(got, want), (got, want)


def test_noalloc_empty_array_gives_zeros():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from pysph_gb300 import native
    v = native.ArrayView()
    v.n = 0
    out = (ctypes.c_double * 6)(*([7.0] * 6))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    native.check(native.lib().sph_invariants_noalloc(ctypes.byref(v), out, stream),
                 "sph_invariants_noalloc")
    assert list(out) == [0.0] * 6
