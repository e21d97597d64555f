"""The FP64 integrator update kernel against the NumPy expressions of the
reference's integrators (solver/integrator.py:472-912), bit for bit: given
the same rates, every scheme's state update rounds exactly like the
reference's (the rates themselves are the pair kernels' FP32 sums; their
parity is tested elsewhere)."""
import numpy as np
import pytest
import torch

from pysph_gb300.sph import gpu

pytestmark = pytest.mark.gpu


class _CM:
    """The minimum of a cell manager that gpu.axpy needs: a context."""

    def __init__(self):
        import ctypes
        from pysph_gb300 import native
        L = native.lib()
        self.h = ctypes.c_void_p()
        native.check(L.sph_ctx_create(3, ctypes.byref(self.h)), "ctx")
        native.check(L.sph_ctx_set_stream(self.h, ctypes.c_void_p(
            torch.cuda.current_stream().cuda_stream)), "stream")

    def context(self):
        return self.h

    def __del__(self):
        from pysph_gb300 import native
        native.lib().sph_ctx_destroy(self.h)


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")


def _arrays(n, k, seed):
    rng = np.random.default_rng(seed)
    # magnitudes spread over decades so rounding differences would show
    return [rng.normal(0, 1, n) * 10.0 ** rng.uniform(-6, 3, n) for _ in range(k)]


def test_every_update_line_is_bit_exact():
    _need_gpu()
    n = 100_003
    x0, x, k1, k2, k3, k4 = _arrays(n, 6, 0)
    dt = 1.2345e-4
    dev = [torch.from_numpy(a).cuda() for a in (x0, x, k1, k2, k3, k4)]
    X0, X, K1, K2, K3, K4 = dev
    cm = _CM()
    out = torch.empty_like(X)
    cases = [
        # (line, reference NumPy expression)
        ((out, None, X, K1, None, dt, 1), x + k1 * dt),                        # step (:509)
        ((out, None, X0, K1, None, dt, 1), x0 + k1 * dt),                      # Euler (:549)
        ((out, None, X0, K1, K2, 0.5 * dt, 0), x0 + 0.5 * dt * (k1 + k2)),     # RK2 (:614)
        ((out, None, X0, K1, None, 0.0, 2), x0.copy()),                        # set_initial
        ((out, None, X0, K1, K2, dt / 6.0, 5, K3, K4),
         x0 + (dt / 6.0) * (k1 + 2 * k2 + 2 * k3 + k4)),                       # RK4 (:686)
        ((out, None, X, X0, None, 0.0, 3), 2 * x - x0),                        # PC (:762)
        ((out, None, X, K1, K2, 0.5 * dt, 4), x + 0.5 * dt * (k2 - k1)),       # LeapFrog (:887)
        ((out, None, X, K1, None, 0.5 * dt * dt, 1), x + 0.5 * dt * dt * k1),  # LeapFrog (:867)
    ]
    for line, ref in cases:
        gpu.axpy(cm, n, [line])
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), ref)


def test_save_copies_the_result():
    _need_gpu()
    n = 4097
    x0, k1 = _arrays(n, 2, 1)
    X0, K1 = (torch.from_numpy(a).cuda() for a in (x0, k1))
    out = torch.empty_like(X0)
    save = torch.empty_like(X0)
    cm = _CM()
    gpu.axpy(cm, n, [(out, save, X0, K1, None, 1e-3, 1)])
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), x0 + k1 * 1e-3)
    np.testing.assert_array_equal(save.cpu().numpy(), out.cpu().numpy())


def test_lines_of_one_launch_chained_and_independent():
    """Several lines in one launch.  Independent lines (none reads what
    another writes) have their loads issued together; a line that reads an
    earlier line's output sees that output, as in one NumPy statement after
    the other."""
    _need_gpu()
    n = 65_537
    x0, y0, k1, k2, k3 = _arrays(n, 5, 2)
    X0, Y0, K1, K2, K3 = (torch.from_numpy(a).cuda() for a in (x0, y0, k1, k2, k3))
    dt = 3.3e-4
    cm = _CM()
    # independent: two RK2-style lines and a copy, each with its own output
    ox, oy, oc = (torch.empty_like(X0) for _ in range(3))
    gpu.axpy(cm, n, [(ox, None, X0, K1, K2, 0.5 * dt, 0),
                     (oy, None, Y0, K3, None, dt, 1),
                     (oc, None, X0, K1, None, 0.0, 2)])
    torch.cuda.synchronize()
    np.testing.assert_array_equal(ox.cpu().numpy(), x0 + 0.5 * dt * (k1 + k2))
    np.testing.assert_array_equal(oy.cpu().numpy(), y0 + k3 * dt)
    np.testing.assert_array_equal(oc.cpu().numpy(), x0)
    # chained: the second line reads the first's output, the third the
    # second's saved copy
    a, b, c, sb = (torch.empty_like(X0) for _ in range(4))
    gpu.axpy(cm, n, [(a, None, X0, K1, None, dt, 1),
                     (b, sb, a, K2, None, dt, 1),
                     (c, None, sb, a, None, 0.0, 3)])
    torch.cuda.synchronize()
    ra = x0 + k1 * dt
    rb = ra + k2 * dt
    np.testing.assert_array_equal(a.cpu().numpy(), ra)
    np.testing.assert_array_equal(b.cpu().numpy(), rb)
    np.testing.assert_array_equal(sb.cpu().numpy(), rb)
    np.testing.assert_array_equal(c.cpu().numpy(), 2 * rb - ra)
