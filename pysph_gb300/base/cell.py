"""CellManager: the GPU neighbour structure of one collection of arrays.

Reference: base/cell.pyx:757-1437.  The reference bins particles into a
dict of ``Cell`` objects with one index list per array and rebins the
escaped particles on every update.  Here an update is one native build
(``sph_nnps_build``): every array is binned on a dense grid, sorted by cell
and gathered into FP32 cell-local snapshots that the pair kernels read.

Kept from the reference: ``cell_size = max_radius_scale * max(h)`` computed
once at initialisation (:893-925), the jump-tolerance check that raises
``RuntimeError('Particle moved by more than one cell width')`` (:1422-1437),
``array_indices`` and ``arrays_to_bin``.  Periodic domains (:1277-1376,
:1568) are not part of this build.
"""
import ctypes

import torch

from .. import native

SNAPSHOT_PROPS = frozenset(("x", "y", "z", "u", "v", "w", "m", "h", "rho", "p", "cs",
                            "nx", "ny", "nz", "tx", "ty", "tz", "tag"))


def array_view(pa):
    """``sph_array_view`` of a ParticleArray's device tensors."""
    v = native.ArrayView()
    v.n = pa.get_number_of_particles()
    props = pa.properties
    for f in native.VIEW_FIELDS:
        t = props.get(f)
        if t is not None and t.dtype != torch.float64:
            t = None
        setattr(v, f, t.data_ptr() if t is not None and t.numel() > 0 else None)
    t = props.get("tag")
    v.tag = t.data_ptr() if t is not None and t.numel() > 0 else None
    return v


class PeriodicDomain:
    """base/cell.pyx:1568-1598: limits of a periodic box.  An axis whose
    limits span exactly 2000 (the default -1000 .. 1000) is not periodic
    (translate 0); the others translate by max - min."""

    def __init__(self, xmin=-1000.0, xmax=1000.0, ymin=-1000.0, ymax=1000.0, zmin=-1000.0,
                 zmax=1000.0):
        self.xmin, self.xmax = xmin, xmax
        self.ymin, self.ymax = ymin, ymax
        self.zmin, self.zmax = zmin, zmax
        self.xtranslate = 0.0 if (xmax - xmin) == 2000 else xmax - xmin
        self.ytranslate = 0.0 if (ymax - ymin) == 2000 else ymax - ymin
        self.ztranslate = 0.0 if (zmax - zmin) == 2000 else zmax - zmin


class CellManager:
    """Dense-grid cell structure over ``arrays_to_bin``."""

    def __init__(self, arrays_to_bin=None, min_cell_size=-1.0, max_cell_size=0,
                 periodic_domain=None, initialize=True, max_radius_scale=2.0):
        if periodic_domain is not None and (periodic_domain.ytranslate != 0.0
                                            or periodic_domain.ztranslate != 0.0):
            # the reference replicates ghost cells along x only
            # (cell.pyx:1308-1352); y and z periodicity have no reference
            raise NotImplementedError("periodic domains are periodic along x only "
                                      "(as the reference's ghost cells)")
        self.max_radius_scale = max_radius_scale
        self.min_cell_size = min_cell_size
        self.max_cell_size = max_cell_size
        self.arrays_to_bin = list(arrays_to_bin or [])
        self.num_arrays = len(self.arrays_to_bin)
        self.array_indices = {}
        self.coord_x, self.coord_y, self.coord_z = "x", "y", "z"
        self.jump_tolerance = 1
        # the next build starts afresh (no jump check): set after the
        # particle state was replaced rather than advanced
        self.skip_jump_once = False
        self.cell_size = 0.0
        self.periodic_domain = periodic_domain
        self.is_dirty = True
        self.initialized = False
        # internal grid cells per reference cell (1..3); see the autotuner
        self.cell_subdivision = None
        # variable h: the symmetric neighbour relation of
        # VarHNbrParticleLocator (set by NNPSManager(variable_h=True))
        self.symmetric = False
        # deferred check of light refreshes (set by the integrators): the
        # update returns without waiting for the device, the next pair pass
        # reads its verdict
        self.deferred_check = False
        self._ctx = None
        self._snap_versions = []
        self._build_count = 0
        if initialize:
            self.initialize()

    # -- setup ----------------------------------------------------------------
    def _rebuild_array_indices(self):
        self.array_indices = {pa.name: i for i, pa in enumerate(self.arrays_to_bin)}

    def initialize(self):
        if self.initialized:
            return
        self._rebuild_array_indices()
        self.compute_cell_size(self.min_cell_size, self.max_cell_size)
        self.initialized = True
        self.update()

    def _compute_minmax_h(self):
        lo, hi = float("inf"), 0.0
        for pa in self.arrays_to_bin:
            if pa.get_number_of_particles() == 0:
                continue
            h = pa.get_device("h")
            lo = min(lo, float(h.min()))
            hi = max(hi, float(h.max()))
        return lo, hi

    def compute_cell_size(self, min_size=0, max_size=0):
        """cell.pyx:893-925."""
        if min_size <= 0:
            min_h, max_h = self._compute_minmax_h()
            self.min_h, self.max_h = min_h, max_h
            self.cell_size = self.max_radius_scale * max_h
        else:
            self.cell_size = min_size
        if self.cell_size > max_size > 0:
            self.cell_size = max_size
        if self.cell_size == 0.0:
            self.cell_size = 1.0
        return self.cell_size

    def add_array_to_bin(self, parr):
        self.arrays_to_bin.append(parr)
        self.num_arrays = len(self.arrays_to_bin)
        self._rebuild_array_indices()
        self.is_dirty = True

    def set_jump_tolerance(self, jump_tolerance):
        if jump_tolerance != 1:
            raise NotImplementedError("only the reference's default jump tolerance of 1 is supported")
        self.jump_tolerance = jump_tolerance

    def get_number_of_particles(self):
        return sum(pa.get_number_of_particles() for pa in self.arrays_to_bin)

    # -- device structure -------------------------------------------------------
    def context(self):
        """The native context (created on first use; needs a GPU)."""
        L = native.lib()
        if self._ctx is None:
            dim = 3
            h = ctypes.c_void_p()
            native.check(L.sph_ctx_create(dim, ctypes.byref(h)), "sph_ctx_create")
            native.check(L.sph_ctx_set_skin(h, self.list_skin()), "sph_ctx_set_skin")
            native.check(L.sph_ctx_set_symmetric(h, 1 if self.symmetric else 0),
                         "sph_ctx_set_symmetric")
            dom = self.periodic_domain
            if dom is not None and dom.xtranslate != 0.0:
                native.check(L.sph_ctx_set_periodic(h, 1, float(dom.xmin), float(dom.xmax)),
                             "sph_ctx_set_periodic")
            if self.deferred_check:
                native.check(L.sph_ctx_set_deferred(h, 1), "sph_ctx_set_deferred")
            from ..tuning import brick_passes
            native.check(L.sph_ctx_set_bricks(h, 1 if brick_passes() else 0), "sph_ctx_set_bricks")
            self._ctx = h
        native.check(L.sph_ctx_set_stream(self._ctx, ctypes.c_void_p(
            torch.cuda.current_stream().cuda_stream)), "sph_ctx_set_stream")
        return self._ctx

    def set_symmetric(self, on):
        """Use the variable-h (symmetric) neighbour relation from the next build."""
        on = bool(on)
        if on != self.symmetric:
            self.symmetric = on
            self.is_dirty = True
            if self._ctx is not None:
                native.check(native.lib().sph_ctx_set_symmetric(self._ctx, 1 if on else 0),
                             "sph_ctx_set_symmetric")

    def set_skin(self, fraction):
        """Neighbour-list skin as a fraction of the search radius.  With a
        structure already built, a full build with the new skin follows at
        once (from the current positions), so every later call finds one."""
        self.skin = float(fraction)
        if self._ctx is not None:
            native.check(native.lib().sph_ctx_set_skin(self._ctx, self.skin), "sph_ctx_set_skin")
            if getattr(self, "_views", None) is not None:
                self.rebuild()

    def list_skin(self):
        """The neighbour-list skin in effect."""
        s = getattr(self, "skin", None)
        if s is None:
            from ..tuning import list_skin
            s = self.skin = list_skin()
        return s

    def set_deferred_check(self, on):
        """Let updates return before the device has checked a light refresh
        (a jump is then reported by the next pair pass instead of by the
        update; results are unchanged)."""
        on = bool(on)
        if on != self.deferred_check:
            self.deferred_check = on
            if self._ctx is not None:
                native.check(native.lib().sph_ctx_set_deferred(self._ctx, 1 if on else 0),
                             "sph_ctx_set_deferred")

    def _subdivision(self):
        if self.cell_subdivision is None:
            from ..tuning import choose_subdivision
            self.cell_subdivision = choose_subdivision(self)
        return self.cell_subdivision

    def update_status(self):
        for pa in self.arrays_to_bin:
            if pa.is_dirty:
                self.is_dirty = True
        return 0

    def update(self):
        """Rebuild the device structure if any array moved (cell.pyx:927-962)."""
        self.update_status()
        if not self.is_dirty:
            return 0
        if not torch.cuda.is_available():
            # no device: the structure is built on first use, where the
            # computation itself raises (there is no CPU path)
            return 0
        ctx = self.context()
        views = (native.ArrayView * len(self.arrays_to_bin))(
            *[array_view(pa) for pa in self.arrays_to_bin])
        # no jump check with a periodic domain (cell.pyx:404-407)
        check = 0 if (self.skip_jump_once or self.periodic_domain is not None) else 1
        rebuilt = ctypes.c_int(1)
        rc = native.lib().sph_nnps_update(ctx, views, len(self.arrays_to_bin), self.cell_size,
                                          self.max_radius_scale, self._subdivision(), check,
                                          ctypes.byref(rebuilt))
        self.skip_jump_once = False
        native.check(rc, "CellManager.update")
        self._views = views
        self._snap_versions = [pa.version for pa in self.arrays_to_bin]
        for pa in self.arrays_to_bin:
            pa.set_dirty(False)
        self.is_dirty = False
        self._build_count += 1
        return 0

    def rebuild(self, check_jump=True):
        """A full neighbour build now, sorting afresh (the lists then depend
        only on the current state, not on the update history)."""
        if not torch.cuda.is_available():
            return 0
        ctx = self.context()
        views = (native.ArrayView * len(self.arrays_to_bin))(
            *[array_view(pa) for pa in self.arrays_to_bin])
        rc = native.lib().sph_nnps_build(ctx, views, len(self.arrays_to_bin), self.cell_size,
                                         self.max_radius_scale, self._subdivision(),
                                         1 if (check_jump and self.periodic_domain is None) else 0)
        native.check(rc, "CellManager.rebuild")
        self._views = views
        self._snap_versions = [pa.version for pa in self.arrays_to_bin]
        for pa in self.arrays_to_bin:
            pa.set_dirty(False)
        self.is_dirty = False
        self.skip_jump_once = False
        self._build_count += 1
        return 0

    def ensure_current(self):
        """Make every snapshot reflect the arrays' current device data."""
        self.update_status()
        if self.is_dirty:
            self.update()
            return
        ctx = None
        for i, pa in enumerate(self.arrays_to_bin):
            if pa.version != self._snap_versions[i]:
                ctx = ctx or self.context()
                v = array_view(pa)
                native.check(native.lib().sph_refresh_state(ctx, i, ctypes.byref(v)),
                             "refresh snapshot")
                self._snap_versions[i] = pa.version

    def build_stats(self):
        """(full neighbour builds, light refreshes) of this cell manager."""
        if self._ctx is None:
            return (0, 0)
        out = (ctypes.c_int64 * 2)()
        native.check(native.lib().sph_nnps_stats(self._ctx, out), "sph_nnps_stats")
        return (int(out[0]), int(out[1]))

    def brick_pass_count(self):
        """Pair passes the brick-staged kernels have run for this cell manager."""
        if self._ctx is None:
            return 0
        out = (ctypes.c_int64 * 1)()
        native.check(native.lib().sph_pair_pass_stats(self._ctx, out), "sph_pair_pass_stats")
        return int(out[0])

    def deferred_stats(self):
        """(deferred light refreshes, those found stale at their first pass)."""
        if self._ctx is None:
            return (0, 0)
        out = (ctypes.c_int64 * 2)()
        native.check(native.lib().sph_nnps_deferred_stats(self._ctx, out),
                     "sph_nnps_deferred_stats")
        return (int(out[0]), int(out[1]))

    def mark_fresh(self, pa):
        """The snapshot of ``pa`` already matches its data (written together)."""
        self._snap_versions[self.array_indices[pa.name]] = pa.version

    def slot(self, pa):
        try:
            return self.array_indices[pa.name]
        except KeyError:
            raise ValueError("Source %s does not exist" % pa.name) from None

    def __del__(self):
        ctx = getattr(self, "_ctx", None)
        if ctx is not None:
            try:
                native.load_library(False).sph_ctx_destroy(ctx)
            except Exception:
                pass
