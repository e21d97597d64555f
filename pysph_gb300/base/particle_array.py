"""Device-resident ParticleArray with the reference's interface.

Reference: base/particle_array.pyx:96-1283.  The reference keeps one
malloc'd C array per property; here every property is a 1-D torch tensor on
the GPU (float64 for ``double``, int64 for ``long``, int32 for ``int``), so
the pair kernels read them in place.  ``get`` returns host NumPy copies (the
reference returns views that alias the C array: write back with ``set``);
``get_device`` returns the device tensor itself.

Structural operations (add/remove/align particles) are host-side
bookkeeping done through NumPy copies, as they are in the reference.
"""
import itertools

import numpy as np
import torch

from . import transfer
from .carray import BaseArray, DoubleArray, IntArray, LongArray
from .particle_types import ParticleType

# particle tags, base/particle_array.pxd:20-26
LocalReal = 0
Dummy = 1
LocalDummy = 2
RemoteReal = 3
RemoteDummy = 4
GhostParticle = 5

_VERSIONS = itertools.count(1)

_DTYPES = {"double": torch.float64, "float": torch.float32, "long": torch.int64,
           "int": torch.int32}
_NP = {torch.float64: np.float64, torch.float32: np.float32, torch.int64: np.int64,
       torch.int32: np.int32}


def is_local_real(tag):
    return tag == LocalReal


def is_local_dummy(tag):
    return tag == LocalDummy


def is_remote_real(tag):
    return tag == RemoteReal


def is_remote_dummy(tag):
    return tag == RemoteDummy


def is_ghost_particle(tag):
    return tag == GhostParticle


def get_local_real_tag():
    return LocalReal


def get_dummy_tag():
    return Dummy


def get_local_dummy_tag():
    return LocalDummy


def get_remote_real_tag():
    return RemoteReal


def get_remote_dummy_tag():
    return RemoteDummy


def get_ghost_particle_tag():
    return GhostParticle


def storage_device():
    """The GPU if there is one.  Without one, arrays can still be built and
    inspected (host logic), but every computation raises."""
    return torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")


class DeviceArray:
    """What ``get_carray`` returns: a handle on one device property with the
    carray accessors the reference API exposes."""

    def __init__(self, pa, name):
        self._pa = pa
        self.name = name

    @property
    def tensor(self):
        return self._pa._props[self.name]

    @property
    def length(self):
        return self.tensor.numel()

    def __len__(self):
        return self.length

    def get_npy_array(self):
        return self.tensor.detach().cpu().numpy()

    def set_data(self, data):
        self._pa.set(**{self.name: data})

    def __getitem__(self, i):
        return self.get_npy_array()[i]


class ParticleArray:
    """A named collection of per-particle properties on the GPU."""

    def __init__(self, name="", default_particle_tag=LocalReal, particle_type=ParticleType.Fluid,
                 cl_precision="double", constants=None, **props):
        d = self.__dict__
        d["_props"] = {"tag": torch.zeros(0, dtype=torch.int64, device=storage_device()),
                       "group": torch.zeros(0, dtype=torch.int64, device=storage_device()),
                       "local": torch.zeros(0, dtype=torch.int32, device=storage_device())}
        d["default_values"] = {"tag": default_particle_tag, "group": 0, "local": 1}
        d["temporary_arrays"] = {}
        d["constants"] = dict(constants or {})
        d["name"] = name
        d["is_dirty"] = True
        d["indices_invalid"] = True
        d["particle_type"] = particle_type
        d["cl_precision"] = cl_precision
        d["num_real_particles"] = 0
        d["_version"] = next(_VERSIONS)
        if props:
            self.initialize(**props)

    # -- attribute access (particle_array.pyx:175-198) -----------------------
    @property
    def properties(self):
        return self._props

    def __getattr__(self, name):
        props = self.__dict__.get("_props", {})
        if name in props:
            return self._get_real(name)
        consts = self.__dict__.get("constants", {})
        if name in consts:
            return consts[name]
        raise AttributeError("property %s not found" % name)

    def __setattr__(self, name, value):
        if name in self.__dict__ or name in type(self).__dict__:
            object.__setattr__(self, name, value)
        elif name in self._props:
            self.set(**{name: value})
        elif name in self.constants:
            self.constants[name] = value
        else:
            raise AttributeError("property %s not found" % name)

    def __reduce__(self):
        props = {}
        for k, t in self._props.items():
            props[k] = {"data": t.cpu().numpy(), "type": self._type_of(k),
                        "default": self.default_values.get(k, 0)}
        return (_rebuild, (self.name, self.particle_type, self.cl_precision,
                           dict(self.constants), props))

    # -- flags ------------------------------------------------------------------
    def set_dirty(self, value):
        self.__dict__["is_dirty"] = bool(value)

    def set_indices_invalid(self, value):
        self.__dict__["indices_invalid"] = bool(value)

    def has_array(self, arr_name):
        return arr_name in self._props

    def set_name(self, name):
        self.__dict__["name"] = name

    def set_particle_type(self, particle_type):
        self.__dict__["particle_type"] = particle_type

    def touch(self):
        """Mark device data as changed (after writing a ``get_device`` tensor)."""
        self.__dict__["_version"] = next(_VERSIONS)

    @property
    def version(self):
        return self._version

    def clear(self):
        tagdef = self.default_values["tag"]
        self.__init__(name=self.name, default_particle_tag=tagdef,
                      particle_type=self.particle_type, cl_precision=self.cl_precision,
                      constants=self.constants)

    # -- construction -----------------------------------------------------------
    def initialize(self, **props):
        self.clear()
        for prop, info in props.items():
            info = dict(info)
            info["name"] = prop
            self.add_property(info)
        self.align_particles()

    def get_number_of_particles(self):
        for t in self._props.values():
            return int(t.numel())
        return 0

    def _type_of(self, name):
        t = self._props[name].dtype
        return {torch.float64: "double", torch.float32: "float", torch.int64: "long",
                torch.int32: "int"}[t]

    def _new(self, dtype_name, n, default):
        dt = _DTYPES.get(dtype_name or "double")
        if dt is None:
            raise ValueError("Trying to create carray of unknown datatype: %s" % dtype_name)
        return torch.full((int(n),), default if default is not None else 0, dtype=dt,
                          device=storage_device())

    def add_property(self, prop_info):
        """particle_array.pyx:729-888."""
        name = prop_info.get("name")
        if name is None:
            raise ValueError("Cannot add property with no name")
        dtype_name = prop_info.get("type")
        data = prop_info.get("data")
        default = prop_info.get("default")
        n = self.get_number_of_particles()
        if data is not None and n != 0 and len(data) != 0 and len(data) != n:
            raise ValueError("Array sizes incompatible")
        if default is None:
            default = self.default_values.get(name, 0)
        self.default_values[name] = default
        if n == 0:
            if data is None or len(data) == 0:
                if name not in self._props:
                    self._props[name] = self._new(dtype_name, 0, default)
            else:
                m = len(data)
                for k in list(self._props):
                    self._props[k] = self._new(self._type_of(k), m, self.default_values.get(k, 0))
                if name in self._props:
                    t = self._props[name]
                    self._props[name] = torch.as_tensor(np.asarray(data, dtype=_NP[t.dtype]),
                                                        device=t.device).clone()
                else:
                    dt = dtype_name or "double"
                    arr = np.asarray(data, dtype=_NP[_DTYPES[dt]])
                    self._props[name] = torch.as_tensor(arr, device=storage_device()).clone()
        else:
            if data is None or len(data) == 0:
                if name not in self._props:
                    self._props[name] = self._new(dtype_name, n, default)
            else:
                if name in self._props:
                    t = self._props[name]
                    t.copy_(torch.as_tensor(np.asarray(data, dtype=_NP[t.dtype]), device=t.device))
                else:
                    dt = dtype_name or "double"
                    arr = np.asarray(data, dtype=_NP[_DTYPES[dt]])
                    self._props[name] = torch.as_tensor(arr, device=storage_device()).clone()
        self.touch()

    def remove_property(self, prop_name):
        self._props.pop(prop_name, None)
        self.default_values.pop(prop_name, None)
        self.touch()

    # -- get / set (particle_array.pyx:617-718) -----------------------------------
    def _check_property(self, prop):
        if prop in self._props or prop in self.temporary_arrays or prop in self.constants:
            return
        raise AttributeError("property %s not present" % prop)

    def _get_real(self, name):
        return self._props[name][: self.num_real_particles].detach().cpu().numpy()

    def get(self, *args, only_real_particles=True):
        """Host copies of properties (numpy arrays the caller owns).  Device
        properties are copied into page-locked host buffers on the current
        stream, all of them before one synchronisation."""
        if len(args) == 0:
            return None
        out = []
        pending = False
        for a in args:
            self._check_property(a)
            if a in self._props:
                t = self._props[a]
                if only_real_particles:
                    t = t[: self.num_real_particles]
                t = t.detach()
                if t.is_cuda:
                    h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
                    h.copy_(t, non_blocking=True)
                    pending = True
                    out.append(h)
                else:
                    out.append(t)
            else:
                out.append(self.constants[a])
        if pending:
            torch.cuda.current_stream().synchronize()
        out = [o.numpy() if isinstance(o, torch.Tensor) else o for o in out]
        return out[0] if len(out) == 1 else tuple(out)

    def get_device(self, name):
        """The device tensor of a property (no copy)."""
        self._check_property(name)
        return self._props[name]

    def set(self, **props):
        """Copy values into properties.  Host sources in page-locked memory
        are copied asynchronously on the current stream, all of them before
        one synchronisation (the caller may reuse its buffers on return)."""
        for p in props:
            self._check_property(p)
        pending = False
        for p, val in props.items():
            if p in self._props:
                t = self._props[p]
                src = val if isinstance(val, torch.Tensor) else torch.as_tensor(
                    np.asarray(val, dtype=_NP[t.dtype]))
                src = src.reshape(-1)
                if src.numel() != t.numel():
                    raise ValueError("size mismatch setting %s: %d != %d" %
                                     (p, src.numel(), t.numel()))
                if src.device == t.device:
                    t.copy_(src)
                elif (not src.is_cuda) and t.is_cuda and src.is_pinned() and src.dtype == t.dtype:
                    t.copy_(src, non_blocking=True)
                    pending = True
                else:
                    t.copy_(src.to(dtype=t.dtype))
            if p == "tag":
                self.align_particles()
            if p in ("x", "y", "z"):
                self.set_dirty(True)
        if pending:
            torch.cuda.current_stream().synchronize()
        self.touch()

    # -- staged host transfers (overlap the link with stepping) ----------------
    def upload(self, **props):
        """Start copying host values (page-locked tensors or arrays; others
        are staged through a page-locked copy) to device buffers on a copy
        stream and return a ``StagedUpload`` at once.  Page-locked sources
        must stay unchanged until ``set_staged`` has been called with it."""
        return transfer.upload(self, props)

    def set_staged(self, up):
        """``set`` with the values of an earlier ``upload``: the current
        stream waits for its copies, then copies them into the properties on
        the device (no host synchronisation)."""
        transfer.set_staged(self, up)

    def download(self, *names, only_real_particles=True):
        """Start reading properties back: a device snapshot on the current
        stream, copied to page-locked host buffers on a copy stream.  Returns
        a ``StagedDownload``; its ``result()`` waits for those copies and
        returns NumPy arrays as ``get`` does."""
        return transfer.download(self, names, only_real_particles)

    def get_carray(self, prop):
        if prop in self._props:
            return DeviceArray(self, prop)
        return None

    # -- structural ops -----------------------------------------------------------
    def _host_all(self):
        return {k: t.detach().cpu().numpy().copy() for k, t in self._props.items()}

    def _replace_all(self, host):
        dev = storage_device()
        for k, a in host.items():
            self._props[k] = torch.as_tensor(np.ascontiguousarray(a), device=dev).clone()
        self.touch()

    def align_particles(self):
        """Move LocalReal particles to the front (particle_array.pyx:954-1040)."""
        n = self.get_number_of_particles()
        if n == 0:
            self.__dict__["num_real_particles"] = 0
            return 0
        tag = self._props["tag"].cpu().numpy()
        index = np.arange(n)
        nxt = 0
        nreal = 0
        moves = 0
        for i in range(n):
            if tag[i] == LocalReal:
                nreal += 1
                if i != nxt:
                    index[nxt], index[i] = i, index[nxt]
                    moves += 1
                nxt += 1
        self.__dict__["num_real_particles"] = nreal
        if moves:
            host = self._host_all()
            for k, a in host.items():
                # the reference's _align_array swaps element i with index[i]
                for i in range(n):
                    if index[i] != i:
                        a[i], a[index[i]] = a[index[i]], a[i]
            self._replace_all(host)
            self.set_dirty(True)
            self.set_indices_invalid(True)
        return 0

    def remove_particles(self, index_list):
        """particle_array.pyx:363-418 (swap-with-last removal)."""
        idx = index_list.get_npy_array() if isinstance(index_list, BaseArray) else np.asarray(index_list)
        if idx.size > self.get_number_of_particles():
            raise ValueError("Number of particles to be removed is greater than"
                             "number of particles in array")
        if idx.size == 0:
            return
        srt = np.sort(idx.astype(np.int64))
        host = self._host_all()
        for k, a in host.items():
            length = a.size
            for r in srt[::-1]:
                a[r] = a[length - 1]
                length -= 1
            host[k] = a[:length].copy()
        self._replace_all(host)
        self.align_particles()
        self.set_dirty(True)
        self.set_indices_invalid(True)

    def remove_tagged_particles(self, tag):
        t = self._props["tag"].cpu().numpy()
        self.remove_particles(np.nonzero(t == tag)[0])

    def add_particles(self, **particle_props):
        """particle_array.pyx:461-521."""
        if not particle_props:
            return
        n_new = len(next(iter(particle_props.values())))
        host = self._host_all()
        for k, a in host.items():
            if k in particle_props:
                ext = np.asarray(particle_props[k], dtype=a.dtype)
            else:
                ext = np.full(n_new, self.default_values.get(k, 0), dtype=a.dtype)
            host[k] = np.concatenate([a, ext])
        self._replace_all(host)
        self.align_particles()
        self.set_dirty(True)

    def append_parray(self, parray):
        props = {k: parray.get(k, only_real_particles=False) for k in parray.properties
                 if k in self._props}
        self.add_particles(**props)
        return 0

    def extend(self, num_particles):
        host = self._host_all()
        for k, a in host.items():
            host[k] = np.concatenate([a, np.full(num_particles, self.default_values.get(k, 0),
                                                 dtype=a.dtype)])
        self._replace_all(host)
        self.align_particles()

    def extract_particles(self, index_array, props=None):
        idx = index_array.get_npy_array() if isinstance(index_array, BaseArray) else np.asarray(index_array)
        names = list(self._props) if props is None else props
        out = ParticleArray(name=self.name, particle_type=self.particle_type)
        for k in names:
            out.add_property({"name": k, "type": self._type_of(k),
                              "data": self._props[k].cpu().numpy()[idx],
                              "default": self.default_values.get(k, 0)})
        out.align_particles()
        return out

    def copy_properties(self, source, start_index=-1, end_index=-1):
        for k in source.properties:
            if k in self._props:
                s = source.get_device(k)
                a, b = (0, s.numel()) if start_index < 0 else (start_index, end_index)
                self._props[k][a:b].copy_(s[: b - a])
        self.touch()

    def set_tag(self, tag_value, indices):
        idx = indices.get_npy_array() if isinstance(indices, BaseArray) else np.asarray(indices)
        t = self._props["tag"]
        t[torch.as_tensor(idx, device=t.device, dtype=torch.int64)] = int(tag_value)
        self.align_particles()
        self.touch()

    def __repr__(self):
        return "ParticleArray(name=%r, n=%d, props=%s)" % (
            self.name, self.get_number_of_particles(), sorted(self._props))


def _rebuild(name, particle_type, cl_precision, constants, props):
    return ParticleArray(name=name, particle_type=particle_type, cl_precision=cl_precision,
                         constants=constants, **props)


__all__ = ["ParticleArray", "DeviceArray", "LocalReal", "Dummy", "LocalDummy", "RemoteReal",
           "RemoteDummy", "GhostParticle", "DoubleArray", "LongArray", "IntArray"]
