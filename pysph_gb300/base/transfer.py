"""Staged host transfers of particle properties, overlapped with stepping.

``ParticleArray.set`` / ``get`` (base/particle_array.pyx:1106-1168 in the
reference, where they copy into / out of the host arrays the Cython loops
read) each end with a synchronisation, so a loop of
``set -> integrate -> get`` runs the link and the device one after the
other.  The staged forms split each transfer in two:

* ``upload`` copies page-locked host values into the rows of a fresh device
  buffer (one per dtype) on a host-to-device copy stream and returns at
  once; ``set_staged`` later makes the compute stream wait for those copies
  and moves the rows into the properties (one multi-tensor copy kernel).
  The upload of step k+1 thus crosses the link while step k computes.
* ``download`` stacks the properties into a fresh device buffer on the
  compute stream (one kernel per dtype) and copies it to a fresh page-locked
  host buffer on a device-to-host copy stream (one copy); ``result()`` waits
  for that copy only.  The read-back of step k thus crosses the link while
  step k+1 computes.

Buffers come from torch's caching allocators and are marked as used by the
other stream, so none is reused before the copies that read it are done.
"""
import numpy as np
import torch

_STREAMS = {}


def copy_stream(kind):
    """The process-wide copy stream of one direction ("h2d" or "d2h") on the
    current device."""
    key = (kind, torch.cuda.current_device())
    s = _STREAMS.get(key)
    if s is None:
        s = torch.cuda.Stream()
        _STREAMS[key] = s
    return s


class StagedUpload:
    """Host values in flight to a particle array (``ParticleArray.upload``)
    or a batch of simulations (``SimulationBatch.upload``)."""

    def __init__(self, pa, groups, ready):
        self.pa = pa
        self.groups = groups      # [(property names, device [k, n] buffer)]
        self.ready = ready        # event on the copy stream after the copies
        self.applied = False


class StagedDownload:
    """Properties in flight to the host (``ParticleArray.download``)."""

    def __init__(self, names, rows, done):
        self.names = names
        self._rows = rows         # per name: (page-locked [k, n] buffer, row)
        self._done = done         # event on the copy stream after the copies
        self._out = None

    def ready(self):
        """True when the host copies have landed (no wait)."""
        return self._done.query()

    def result(self):
        """The downloaded values as NumPy arrays (owned by the caller), in the
        order asked for; waits for the device-to-host copies only."""
        if self._out is None:
            self._done.synchronize()
            out = [h.numpy()[r] for h, r in self._rows]
            self._out = out[0] if len(out) == 1 else tuple(out)
            self._rows = None
        return self._out


def _host_source(val, dtype):
    """A page-locked CPU tensor of ``dtype`` holding ``val``."""
    if isinstance(val, torch.Tensor):
        t = val.detach().reshape(-1)
        if t.is_cuda:
            raise ValueError("upload takes host values (use set for device tensors)")
        if t.dtype != dtype:
            t = t.to(dtype)
    else:
        t = torch.from_numpy(np.ascontiguousarray(val).reshape(-1)).to(dtype)
    if not t.is_pinned():
        t = t.pin_memory()
    return t


def _by_dtype(tensors, names):
    """Names grouped by the dtype of their tensors, in first-seen order."""
    groups = {}
    for a in names:
        groups.setdefault(tensors[a].dtype, []).append(a)
    return list(groups.values())


def _copy_all(dst, src):
    if hasattr(torch, "_foreach_copy_"):
        torch._foreach_copy_(dst, src)       # one multi-tensor kernel
    else:
        for d, s in zip(dst, src):
            d.copy_(s)


def upload_tensors(targets, props, n):
    """Start the host-to-device copies of ``props`` (name -> host values)
    for the device tensors ``targets`` (name -> tensor of ``n`` values) on
    the copy stream; returns a ``StagedUpload`` (its ``pa`` left unset)."""
    srcs = {}
    for p, val in props.items():
        src = _host_source(val, targets[p].dtype)
        if src.numel() != n:
            raise ValueError("size mismatch uploading %s: %d != %d" % (p, src.numel(), n))
        srcs[p] = src
    cs = copy_stream("h2d")
    groups = []
    with torch.cuda.stream(cs):
        for names in _by_dtype(targets, list(props)):
            # one device buffer per dtype, allocated for the copy stream
            buf = torch.empty((len(names), n), dtype=targets[names[0]].dtype,
                              device=targets[names[0]].device)
            for r, p in enumerate(names):
                buf[r].copy_(srcs[p], non_blocking=True)
            groups.append((names, buf))
        ready = torch.cuda.Event()
        ready.record(cs)
    return StagedUpload(None, groups, ready)


def apply_staged(targets, up, stream):
    """Make ``stream`` wait for the upload's copies and copy its rows into
    ``targets`` there (one multi-tensor copy per dtype)."""
    if up.applied:
        raise ValueError("set_staged: upload already applied")
    stream.wait_event(up.ready)
    with torch.cuda.stream(stream):
        for names, buf in up.groups:
            buf.record_stream(stream)
            _copy_all([targets[p] for p in names], list(buf.unbind(0)))
    up.applied = True
    names = [p for names, _ in up.groups for p in names]
    up.groups = None
    return names


def download_tensors(tensors, names, stream):
    """Stack ``tensors`` (name -> device tensor, same length) on ``stream``
    and copy the stack to page-locked host memory on the copy stream."""
    cs = copy_stream("d2h")
    snaps = []
    with torch.cuda.stream(stream):
        for group in _by_dtype(tensors, list(dict.fromkeys(names))):
            s = torch.stack([tensors[a] for a in group])
            s.record_stream(cs)                # read there by the copy
            snaps.append((group, s))
        snapped = torch.cuda.Event()
        snapped.record(stream)
    where = {}
    with torch.cuda.stream(cs):
        cs.wait_event(snapped)
        for group, s in snaps:
            h = torch.empty(s.shape, dtype=s.dtype, pin_memory=True)
            h.copy_(s, non_blocking=True)
            for r, a in enumerate(group):
                where[a] = (h, r)
        done = torch.cuda.Event()
        done.record(cs)
    return StagedDownload(tuple(names), [where[a] for a in names], done)


def upload(pa, props):
    if not props:
        raise ValueError("upload: no properties")
    for p in props:
        pa._check_property(p)
        if p == "tag" or p not in pa._props:
            raise ValueError("upload: %s is not a numeric property" % p)
        if not pa._props[p].is_cuda:
            raise RuntimeError("upload needs the arrays on a GPU")
    up = upload_tensors(pa._props, props, pa.get_number_of_particles())
    up.pa = pa
    return up


def set_staged(pa, up):
    if not isinstance(up, StagedUpload) or up.pa is not pa:
        raise ValueError("set_staged takes an upload of this particle array")
    if up.groups and up.groups[0][1].shape[1] != pa.get_number_of_particles():
        raise ValueError("set_staged: the particle count changed since the upload")
    names = apply_staged(pa._props, up, torch.cuda.current_stream())
    if any(p in ("x", "y", "z") for p in names):
        pa.set_dirty(True)
    pa.touch()


def download(pa, names, only_real_particles=True):
    if not names:
        raise ValueError("download: no properties")
    for a in names:
        pa._check_property(a)
        if a not in pa._props:
            raise ValueError("download: %s is not a property" % a)
        if not pa._props[a].is_cuda:
            raise RuntimeError("download needs the arrays on a GPU")
    m = pa.num_real_particles if only_real_particles else pa.get_number_of_particles()
    tensors = {a: pa._props[a][:m] for a in dict.fromkeys(names)}
    return download_tensors(tensors, names, torch.cuda.current_stream())
