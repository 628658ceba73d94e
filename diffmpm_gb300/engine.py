"""GPU-resident simulation: the Python face of one C handle.

``Simulation`` owns one ``MpmHandle`` (include/diffmpm_gb300.h).  Arrays passed
in or out may be NumPy arrays (host memory; the library copies) or CUDA torch
tensors (device memory on the handle's GPU; used in place, ordered on torch's
current stream).  All arithmetic runs in the CUDA library.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import weakref
from pathlib import Path
from typing import Sequence

import numpy as np

from . import _lib
from .functions import Linear, Unit

_FIELD_NCOMP = {"loc": "ndim", "velocity": "ndim", "momentum": "ndim", "stress": 6, "strain": 6}
_INT_FIELDS = ("material_id", "element_ids")


def _is_cuda_tensor(a) -> bool:
    return type(a).__module__.startswith("torch") and getattr(a, "is_cuda", False)


def _stream_for(a):
    if _is_cuda_tensor(a):
        import torch
        return C.c_void_p(torch.cuda.current_stream(a.device).cuda_stream)
    return None


def _in_arg(a, dtype, count):
    """(pointer, on_device, keepalive) for an input of ``count`` elements."""
    if _is_cuda_tensor(a):
        import torch
        want = torch.float32 if dtype == np.float32 else torch.int32
        if a.dtype != want or not a.is_contiguous() or a.numel() != count:
            raise ValueError(f"expected a contiguous {want} tensor of {count} elements")
        return C.c_void_p(a.data_ptr()), 1, a
    arr = np.ascontiguousarray(np.asarray(a, dtype=dtype).reshape(-1))
    if arr.size != count:
        raise ValueError(f"expected {count} values, found {arr.size}")
    return _lib.ptr(arr), 0, arr


def _out_arg(out, dtype, count):
    """(pointer, on_device) for a caller-provided destination of ``count``
    elements: a C-contiguous, writeable NumPy array or a contiguous CUDA
    tensor of exactly that dtype and size (the library writes
    ``count * 4`` bytes there, so anything else is refused)."""
    if _is_cuda_tensor(out):
        import torch
        want = torch.float32 if dtype == np.float32 else torch.int32
        if out.dtype != want or not out.is_contiguous() or out.numel() != count:
            raise ValueError(f"out must be a contiguous {want} tensor of {count} elements, "
                             f"found {out.dtype} with {out.numel()} elements")
        return C.c_void_p(out.data_ptr()), 1
    if not isinstance(out, np.ndarray):
        raise ValueError("out must be a NumPy array or a CUDA tensor")
    if out.dtype != np.dtype(dtype) or not out.flags.c_contiguous or not out.flags.writeable \
            or out.size != count:
        raise ValueError(f"out must be a writeable C-contiguous {np.dtype(dtype).name} array of "
                         f"{count} elements, found {out.dtype.name} with {out.size} elements")
    return _lib.ptr(out), 0


_TUNING_KEYS = ("block_steps", "resort_every", "nk_ctas", "g2p_ctas", "forces_lpc", "ms_per_step")
# The candidates mpm_batch_autotune tries; part of the cache key, so that a
# result chosen among other candidates is not read back.
_TUNING_SPACE = "nk_ctas 2,3; g2p_ctas 2,3; forces_lpc 0,1,2; block_steps 10,25,50,100,200; resort_every 1,2,4"


def device_name(device=None) -> str:
    """The CUDA device's name, compute capability and SM count (the current
    device by default)."""
    lib = _lib.load()
    if device is None:
        try:
            import torch
            device = torch.cuda.current_device() if torch.cuda.is_available() else 0
        except ImportError:
            device = 0
    buf = C.create_string_buffer(256)
    _lib.check(lib.mpm_device_name(int(device), buf, len(buf)))
    return buf.value.decode()


def tuning_cache_path() -> Path:
    """The tuning cache: $DIFFMPM_GB300_TUNING_CACHE, else
    ~/.cache/diffmpm_gb300/tuning.json."""
    env = os.environ.get("DIFFMPM_GB300_TUNING_CACHE")
    return Path(env) if env else Path.home() / ".cache" / "diffmpm_gb300" / "tuning.json"


def _read_tuning_cache(path: Path) -> dict:
    try:
        return json.loads(Path(path).read_text())
    except (OSError, ValueError):
        return {}


def _write_tuning_cache(path: Path, key: str, value: dict):
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    data = _read_tuning_cache(path)
    data[key] = value
    tmp = path.with_name(path.name + f".{os.getpid()}.tmp")
    tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
    os.replace(tmp, path)


class PinnedBuffer:
    """Page-locked host memory from the library (mpm_host_alloc), the
    destination of :meth:`Simulation.output_enqueue`."""

    def __init__(self, nbytes: int):
        self._lib = _lib.load()
        p = C.c_void_p()
        _lib.check(self._lib.mpm_host_alloc(int(nbytes), C.byref(p)))
        self.ptr, self.nbytes = p, int(nbytes)
        self.view = (C.c_char * max(self.nbytes, 1)).from_address(p.value) if p.value else bytearray(1)

    def close(self):
        if self.ptr is not None and self.ptr.value:
            self.view = None
            self._lib.mpm_host_free(self.ptr)
        self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Simulation:
    """One explicit-MPM simulation on the current CUDA device.

    Parameters mirror Quadrilateral4Node (nelements, el_len, constraints,
    concentrated_nodal_forces) and MPMExplicit (dt, scheme, velocity_update);
    ``reinit_each_step`` selects solve_jit semantics (True) or solve semantics.
    ``functions`` lists the Linear time functions that forces and tractions
    may refer to.
    """

    def __init__(self, nelements, el_len, dt, *, scheme="usf", velocity_update=False,
                 reinit_each_step=True, gravity=(0.0, 0.0), constraints=(), functions=(),
                 nodal_forces=(), materials=(), ndim=2):
        self._lib = _lib.load()
        self._h = C.c_void_p()
        self._batches = weakref.WeakSet()   # batches holding this handle
        if scheme not in ("usf", "usl"):
            raise ValueError(f"Please select scheme from ('usf', 'usl'). Found {scheme}")
        nel = np.asarray(nelements, dtype=np.int64).reshape(-1)
        el = np.broadcast_to(np.asarray(el_len, dtype=np.float64).reshape(-1), (2,))
        self.ndim = ndim
        self.nelements = (int(nel[0]), int(nel[1]) if nel.size > 1 else 1)
        self.nnodes = (self.nelements[0] + 1) * ((self.nelements[1] + 1) if ndim == 2 else 1)
        self.functions = [f for f in functions if isinstance(f, Linear)]
        self._fn_index = {id(f): k for k, f in enumerate(self.functions)}
        g = np.broadcast_to(np.asarray(gravity, dtype=np.float64).reshape(-1), (2,))

        d = _lib.MpmDesc()
        d.ndim = ndim
        d.nelements[0], d.nelements[1] = self.nelements
        d.el_len[0], d.el_len[1] = float(el[0]), float(el[1])
        d.scheme = _lib.USF if scheme == "usf" else _lib.USL
        d.velocity_update = int(bool(velocity_update))
        d.reinit_each_step = int(bool(reinit_each_step))
        d.dt = float(dt)
        d.gravity[0], d.gravity[1] = float(g[0]), float(g[1])
        keep = []

        def arr(values, dtype, ctype):
            a = np.ascontiguousarray(np.asarray(values, dtype=dtype).reshape(-1))
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(ctype))

        cn, cd, cv = [], [], []
        for ids, con in constraints:
            ids = np.asarray(ids, dtype=np.int64).reshape(-1)
            cn.extend(ids.tolist())
            cd.extend([con.dir] * ids.size)
            cv.extend([float(con.velocity)] * ids.size)
        d.n_constraints = len(cn)
        d.constraint_node = arr(cn, np.int32, C.c_int32)
        d.constraint_dir = arr(cd, np.int32, C.c_int32)
        d.constraint_velocity = arr(cv, np.float64, C.c_double)

        d.n_functions = len(self.functions)
        d.function_npoints = arr([f.xvalues.size for f in self.functions], np.int32, C.c_int32)
        d.function_x = arr(np.concatenate([f.xvalues for f in self.functions]) if self.functions else [],
                           np.float64, C.c_double)
        d.function_y = arr(np.concatenate([f.fxvalues for f in self.functions]) if self.functions else [],
                           np.float64, C.c_double)

        fnode, fdir, fval, ffn = [], [], [], []
        for f in nodal_forces:
            ids = np.asarray(f.node_ids, dtype=np.int64).reshape(-1)
            fnode.extend(ids.tolist())
            fdir.extend([int(f.dir)] * ids.size)
            fval.extend([float(f.force)] * ids.size)
            ffn.extend([self.function_code(f.function)] * ids.size)
        d.n_nodal_forces = len(fnode)
        d.nodal_force_node = arr(fnode, np.int32, C.c_int32)
        d.nodal_force_dir = arr(fdir, np.int32, C.c_int32)
        d.nodal_force_value = arr(fval, np.float64, C.c_double)
        d.nodal_force_function = arr(ffn, np.int32, C.c_int32)

        mats = (_lib.MpmMaterial * max(1, len(materials)))()
        for i, m in enumerate(materials):
            mats[i] = m.to_c()
        d.n_materials = len(materials)
        d.materials = mats
        self.materials = list(materials)
        rc = self._lib.mpm_create(C.byref(d), C.byref(self._h))
        if rc != _lib.MPM_OK:
            self._h = C.c_void_p()
            _lib.check(rc, None)
        self.n = -1
        self._config = {"ndim": ndim, "nelements": list(self.nelements),
                        "el_len": [float(el[0]), float(el[1])], "dt": float(dt), "scheme": scheme,
                        "velocity_update": bool(velocity_update),
                        "reinit_each_step": bool(reinit_each_step), "materials": len(materials),
                        "constraints": len(cn), "nodal_forces": len(fnode)}

    def config(self) -> dict:
        """The configuration that decides this simulation's step cost (mesh,
        time step, scheme, particle count), for tuning-cache keys."""
        return dict(self._config, particles=int(self.n))

    def set_empty_split(self, min_empty):
        """Launch the empty tiles apart when there are at least ``min_empty``
        of them (mpm_set_empty_split): the same results either way."""
        self._ok(self._lib.mpm_set_empty_split(self._h, int(min_empty)))

    def set_kernel_variant(self, nk_ctas=3, g2p_ctas=2, forces_lpc=0):
        """Kernel builds of the step (mpm_set_kernel_variant): the same results,
        built for 2 or 3 resident CTAs per SM, and any of the three forces
        paths (0 row slots, 1 lane per cell, 2 staged row)."""
        self._ok(self._lib.mpm_set_kernel_variant(self._h, int(nk_ctas), int(g2p_ctas),
                                                  int(forces_lpc)))

    # ------------------------------------------------------------------
    def function_code(self, fn) -> int:
        if fn is None or isinstance(fn, Unit):
            return -1
        if id(fn) not in self._fn_index:
            raise ValueError("time function was not registered with the simulation")
        return self._fn_index[id(fn)]

    def _ok(self, rc):
        _lib.check(rc, self._h)

    def close(self):
        # a batch refers to its members' handles: it goes first
        for b in list(getattr(self, "_batches", ())):
            b.close()
        if self._h:
            self._lib.mpm_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def ncomp(self, field) -> int:
        n = _FIELD_NCOMP.get(field, 1)
        return self.ndim if n == "ndim" else n

    # ------------------------------------------------------------------
    def set_particles(self, loc, material_id=None):
        """Set the population at ``loc`` (n, ndim); every other field takes the
        reference's initial value (diffmpm/particle.py:53-71)."""
        n = int(np.prod(np.shape(loc))) // self.ndim if not _is_cuda_tensor(loc) else loc.numel() // self.ndim
        p, dev, keep = _in_arg(loc, np.float32, n * self.ndim)
        mp, mdev, mkeep = (None, dev, None) if material_id is None else _in_arg(material_id, np.int32, n)
        if material_id is not None and mdev != dev:
            raise ValueError("loc and material_id must both be host arrays or both CUDA tensors")
        self._ok(self._lib.mpm_set_particles(self._h, n, p, mp, dev, _stream_for(loc)))
        self.n = n

    def write(self, field, values):
        dtype = np.int32 if field in _INT_FIELDS else np.float32
        p, dev, keep = _in_arg(values, dtype, self.n * self.ncomp(field))
        self._ok(self._lib.mpm_write_field(self._h, _lib.FIELD[field], p, dev, _stream_for(values)))

    def read(self, field, out=None):
        """Field in original particle order, shape (n, ncomp) (or (n,))."""
        nc = self.ncomp(field)
        dtype = np.int32 if field in _INT_FIELDS else np.float32
        if out is None:
            out = np.empty((self.n, nc) if nc > 1 else (self.n,), dtype=dtype)
        p, dev = _out_arg(out, dtype, self.n * nc)
        self._ok(self._lib.mpm_read_field(self._h, _lib.FIELD[field], p, dev, _stream_for(out)))
        return out

    def output_enqueue(self, fields, buffer: "PinnedBuffer", stream=None) -> int:
        """Enqueue the copy of ``fields`` (names, original order, laid out one
        after the other as :meth:`read` returns them) into ``buffer`` and
        return a ticket for :meth:`output_wait`; does not wait."""
        codes = (C.c_int * len(fields))(*[_lib.FIELD[f] for f in fields])
        need = sum(4 * self.n * self.ncomp(f) for f in fields)
        if buffer.nbytes < need:
            raise ValueError(f"buffer holds {buffer.nbytes} bytes, the fields need {need}")
        t = C.c_int64()
        self._ok(self._lib.mpm_output_enqueue(self._h, len(fields), codes, buffer.ptr,
                                              int(buffer.nbytes), stream, C.byref(t)))
        return t.value

    def output_wait(self, ticket: int):
        """Block until the copy of ``ticket`` is in host memory (callable from
        another thread while this one steps)."""
        self._ok(self._lib.mpm_output_wait(self._h, int(ticket)))

    def output_views(self, fields, buffer: "PinnedBuffer"):
        """NumPy views of ``fields`` inside ``buffer`` (layout of
        :meth:`output_enqueue`)."""
        out, off = {}, 0
        for f in fields:
            nc = self.ncomp(f)
            dt = np.int32 if f in _INT_FIELDS else np.float32
            a = np.frombuffer(buffer.view, dtype=dt, count=self.n * nc, offset=off)
            out[f] = a.reshape((self.n, nc) if nc > 1 else (self.n,))
            off += 4 * self.n * nc
        return out

    def set_tractions(self, pids, dirs, values, functions):
        """Particle tractions: entry k adds f_k(t) * values[k] * V / size in
        direction dirs[k] of particle pids[k] (diffmpm/particle.py:329-343)."""
        pids = np.ascontiguousarray(np.asarray(pids, dtype=np.int64).reshape(-1))
        dirs = np.ascontiguousarray(np.asarray(dirs, dtype=np.int32).reshape(-1))
        vals = np.ascontiguousarray(np.asarray(values, dtype=np.float64).reshape(-1))
        fns = np.ascontiguousarray(np.asarray([self.function_code(f) for f in functions],
                                              dtype=np.int32).reshape(-1))
        self._ok(self._lib.mpm_set_tractions(self._h, int(pids.size), _lib.ptr(pids), _lib.ptr(dirs),
                                             _lib.ptr(vals), _lib.ptr(fns), None))

    def set_particle_velocity_constraints(self, pids, dirs, values):
        """After every particle velocity update, the velocity of particle
        pids[k] in direction dirs[k] is set to values[k] (later entries win);
        an empty list clears them."""
        pids = np.ascontiguousarray(np.asarray(pids, dtype=np.int64).reshape(-1))
        dirs = np.ascontiguousarray(np.asarray(dirs, dtype=np.int32).reshape(-1))
        vals = np.ascontiguousarray(np.asarray(values, dtype=np.float64).reshape(-1))
        if not (pids.size == dirs.size == vals.size):
            raise ValueError("pids, dirs and values must have the same length")
        self._ok(self._lib.mpm_set_particle_velocity_constraints(
            self._h, int(pids.size), _lib.ptr(pids), _lib.ptr(dirs), _lib.ptr(vals), None))

    def read_nodal(self, field, out=None):
        nc = 1 if field == "mass" else self.ndim
        if out is None:
            out = np.empty((self.nnodes, nc) if nc > 1 else (self.nnodes,), dtype=np.float32)
        p, dev = _out_arg(out, np.float32, self.nnodes * nc)
        self._ok(self._lib.mpm_read_nodal_field(self._h, _lib.NODAL_FIELD[field], p, dev, _stream_for(out)))
        return out

    def write_nodal(self, field, values):
        nc = 1 if field == "mass" else self.ndim
        p, dev, keep = _in_arg(values, np.float32, self.nnodes * nc)
        self._ok(self._lib.mpm_write_nodal_field(self._h, _lib.NODAL_FIELD[field], p, dev, _stream_for(values)))

    def initialize(self, stream=None):
        self._ok(self._lib.mpm_initialize(self._h, stream))

    def step(self, nsteps=1, stream=None):
        self._ok(self._lib.mpm_step(self._h, int(nsteps), stream))

    def run_phase(self, phase, stream=None):
        self._ok(self._lib.mpm_run_phase(self._h, _lib.PHASE[phase], stream))

    @property
    def step_index(self) -> int:
        v = C.c_int64()
        self._ok(self._lib.mpm_get_step(self._h, C.byref(v)))
        return v.value

    @step_index.setter
    def step_index(self, value):
        self._ok(self._lib.mpm_set_step(self._h, int(value)))

    def time_phases(self, nsteps, stream=None):
        """Advance ``nsteps`` steps and return the device milliseconds spent in
        each phase kernel, {"nodal_kinematics", "forces", "particle_kinematics"}."""
        ms = (C.c_float * 3)()
        self._ok(self._lib.mpm_time_phases(self._h, int(nsteps), ms, stream))
        return dict(zip(_lib.PHASE, list(ms)))

    def set_block_steps(self, n):
        self._ok(self._lib.mpm_set_block_steps(self._h, int(n)))

    def set_gravity(self, gravity):
        g = np.broadcast_to(np.asarray(gravity, dtype=np.float64).reshape(-1), (2,))
        self._ok(self._lib.mpm_set_gravity(self._h, float(g[0]), float(g[1])))

    def counters(self):
        a, b = C.c_int64(), C.c_int64()
        self._ok(self._lib.mpm_get_counters(self._h, C.byref(a), C.byref(b)))
        return {"resorts": a.value, "rollbacks": b.value}

    # ------------------------------------------------------------------
    def record(self, nsteps, checkpoint_steps=100, stream=None):
        """Advance ``nsteps`` steps keeping a checkpoint every
        ``checkpoint_steps`` steps for :meth:`adjoint`."""
        self._ok(self._lib.mpm_record(self._h, int(nsteps), int(checkpoint_steps), stream))

    def adjoint(self, dl_dloc, dl_dvel=None, *, want=("youngs_modulus", "loc", "velocity")):
        """Reverse of the last :meth:`record` for seeds dL/dx_end (n, ndim) and
        dL/dv_end (n, ndim, optional), original particle order.  Returns a dict
        with the requested gradients at the recorded start: "youngs_modulus"
        (n,), "loc" (n, ndim), "velocity" (n, ndim).  Seeds and outputs are
        NumPy arrays, or CUDA tensors (then the outputs are CUDA tensors too)."""
        n, d = self.n, self.ndim
        p, dev, keep = _in_arg(dl_dloc, np.float32, n * d)
        pv, keepv = None, None
        if dl_dvel is not None:
            pv, vdev, keepv = _in_arg(dl_dvel, np.float32, n * d)
            if vdev != dev:
                raise ValueError("seeds must both be host arrays or both CUDA tensors")
        shapes = {"youngs_modulus": (n,), "loc": (n, d), "velocity": (n, d)}
        out = {}
        for k in want:
            if dev:
                import torch
                out[k] = torch.empty(shapes[k], dtype=torch.float32, device=dl_dloc.device)
            else:
                out[k] = np.empty(shapes[k], dtype=np.float32)

        def optr(k):
            if k not in out:
                return None
            return C.c_void_p(out[k].data_ptr()) if dev else _lib.ptr(out[k])

        self._ok(self._lib.mpm_adjoint(self._h, p, pv, optr("youngs_modulus"), optr("loc"),
                                       optr("velocity"), dev, _stream_for(dl_dloc)))
        return out


class Batch:
    """Simulations advanced together, one kernel launch per phase per step for
    all of them (include/diffmpm_gb300.h, mpm_batch_*).  The members stay
    ordinary ``Simulation`` objects: set them up and read them as usual."""

    def __init__(self, sims: Sequence[Simulation]):
        self._lib = _lib.load()
        self.sims = list(sims)
        handles = (C.c_void_p * len(self.sims))(*[s._h.value for s in self.sims])
        self._b = C.c_void_p()
        rc = self._lib.mpm_batch_create(handles, len(self.sims), C.byref(self._b))
        if rc != _lib.MPM_OK:
            self._b = C.c_void_p()
            _lib.check_batch(rc, None)
        for s in self.sims:
            s._batches.add(self)

    def _ok(self, rc):
        _lib.check_batch(rc, self._b)

    def close(self):
        if self._b:
            self._lib.mpm_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def size(self):
        """(number of simulations, tiles per phase launch)."""
        n, t = C.c_int(), C.c_int()
        self._ok(self._lib.mpm_batch_size(self._b, C.byref(n), C.byref(t)))
        return n.value, t.value

    def step(self, nsteps=1, stream=None):
        self._ok(self._lib.mpm_batch_step(self._b, int(nsteps), stream))

    # ------------------------------------------------------------------
    # whole-batch state transfers (one host copy for all members)
    def _counts(self, field):
        return [s.n * s.ncomp(field) for s in self.sims]

    def write(self, field, values):
        """Write ``field`` of every member: one array holding the members'
        fields one after the other (member order, original particle order),
        or a sequence of per-member arrays; host memory or a CUDA tensor."""
        total = sum(self._counts(field))
        if isinstance(values, (list, tuple)):
            values = np.concatenate([np.asarray(v, np.float32).reshape(-1) for v in values])
        p, dev, keep = _in_arg(values, np.float32, total)
        self._ok(self._lib.mpm_batch_write_field(self._b, _lib.FIELD[field], p, dev,
                                                 _stream_for(values)))

    def read(self, field, out=None):
        """``field`` of every member as one array (member order); ``out`` may
        be a preallocated host array or CUDA tensor of that size.  Returns it
        with per-member views in ``split(...)`` order."""
        counts = self._counts(field)
        dtype = np.int32 if field in _INT_FIELDS else np.float32
        if out is None:
            out = np.empty(sum(counts), dtype=dtype)
        p, dev = _out_arg(out, dtype, sum(counts))
        self._ok(self._lib.mpm_batch_read_field(self._b, _lib.FIELD[field], p, dev, _stream_for(out)))
        return out

    def split(self, field, flat):
        """Per-member arrays (n_i, ncomp) or (n_i,) of a whole-batch ``flat``."""
        out, off = [], 0
        for s, c in zip(self.sims, self._counts(field)):
            nc = s.ncomp(field)
            v = flat[off:off + c]
            out.append(v.reshape((s.n, nc) if nc > 1 else (s.n,)))
            off += c
        return out

    def write_nodal(self, field, values):
        """Nodal ``field`` ("mass", "velocity", "acceleration") of every member,
        one array in member order or a sequence of per-member arrays."""
        nc = 1 if field == "mass" else 2
        total = sum(s.nnodes * nc for s in self.sims)
        if isinstance(values, (list, tuple)):
            values = np.concatenate([np.asarray(v, np.float32).reshape(-1) for v in values])
        p, dev, keep = _in_arg(values, np.float32, total)
        self._ok(self._lib.mpm_batch_write_nodal_field(self._b, _lib.NODAL_FIELD[field], p, dev,
                                                       _stream_for(values)))

    def restart(self, stream=None):
        """Step counters to 0 and every member re-initialised (re-sort, volume
        set-up) from the state written since; one wait for all members."""
        self._ok(self._lib.mpm_batch_restart(self._b, stream))

    def set_block_steps(self, n):
        self._ok(self._lib.mpm_batch_set_block_steps(self._b, int(n)))

    def tuning(self) -> dict:
        """The batch's current tuning (see :meth:`autotune`)."""
        t = _lib.MpmTuning()
        self._ok(self._lib.mpm_batch_get_tuning(self._b, C.byref(t)))
        return {k: getattr(t, k) for k in _TUNING_KEYS}

    def set_tuning(self, block_steps, resort_every=1, nk_ctas=3, g2p_ctas=2, forces_lpc=0):
        t = _lib.MpmTuning(int(block_steps), int(resort_every), int(nk_ctas), int(g2p_ctas),
                           int(forces_lpc), 0.0)
        self._ok(self._lib.mpm_batch_set_tuning(self._b, C.byref(t)))

    def config_key(self, trial_steps) -> str:
        """Key of this batch's configuration in the tuning cache: the GPU's
        name and a hash of every member's mesh, time step, scheme and
        particle count, of the trial length and of the candidate set."""
        import hashlib
        import json
        desc = [s.config() for s in self.sims]
        h = hashlib.sha256(json.dumps({"members": desc, "trial_steps": int(trial_steps),
                                       "candidates": _TUNING_SPACE},
                                      sort_keys=True).encode()).hexdigest()[:20]
        return f"{device_name()}|{h}"

    def autotune(self, trial_steps=100, cache=True, stream=None) -> dict:
        """Choose the batch's tuning by timing ``trial_steps`` steps per
        candidate from the current state (mpm_batch_autotune: kernel builds,
        step-block length, re-sort cadence) and leave the state unchanged.
        With ``cache`` (True: ``tuning_cache_path()``, or a path) the choice
        is stored in a JSON file under :meth:`config_key` and read back,
        without timing, by the next autotune of the same configuration on the
        same kind of GPU.  Returns the tuning with "from_cache" and "key"."""
        path = tuning_cache_path() if cache is True else (Path(cache) if cache else None)
        key = self.config_key(trial_steps)
        if path is not None:
            hit = _read_tuning_cache(path).get(key)
            if hit is not None and all(k in hit for k in _TUNING_KEYS):
                self.set_tuning(**{k: hit[k] for k in _TUNING_KEYS if k != "ms_per_step"})
                return dict(hit, from_cache=True, key=key)
        t = _lib.MpmTuning()
        self._ok(self._lib.mpm_batch_autotune(self._b, int(trial_steps), C.byref(t), stream))
        out = {k: getattr(t, k) for k in _TUNING_KEYS}
        if path is not None:
            _write_tuning_cache(path, key, out)
        return dict(out, from_cache=False, key=key)

    def record(self, nsteps, checkpoint_steps=100, stream=None):
        """``Simulation.record`` for every member at once."""
        self._ok(self._lib.mpm_batch_record(self._b, int(nsteps), int(checkpoint_steps), stream))

    def adjoint(self, dl_dloc, dl_dvel=None, *, want=("youngs_modulus", "loc", "velocity")):
        """``Simulation.adjoint`` for every member at once: ``dl_dloc`` (and the
        optional ``dl_dvel``) are sequences with one (n_i, 2) array per member
        (all NumPy, or all CUDA tensors); returns one dict per member."""
        k = len(self.sims)
        if len(dl_dloc) != k or (dl_dvel is not None and len(dl_dvel) != k):
            raise ValueError("one seed array per simulation")
        keep, dev = [], None
        P = C.c_void_p * k

        def table(arrs, count_of):
            nonlocal dev
            t = P()
            for i, a in enumerate(arrs):
                p, d, kp = _in_arg(a, np.float32, count_of(i))
                if dev is None:
                    dev = d
                elif d != dev:
                    raise ValueError("seeds must all be host arrays or all CUDA tensors")
                keep.append(kp)
                t[i] = p.value if isinstance(p, C.c_void_p) else p
            return t

        tl = table(dl_dloc, lambda i: 2 * self.sims[i].n)
        tv = table(dl_dvel, lambda i: 2 * self.sims[i].n) if dl_dvel is not None else None
        shapes = {"youngs_modulus": lambda n: (n,), "loc": lambda n: (n, 2), "velocity": lambda n: (n, 2)}
        outs = [{} for _ in range(k)]
        tabs = {}
        for key in ("youngs_modulus", "loc", "velocity"):
            if key not in want:
                tabs[key] = None
                continue
            t = P()
            for i, sim in enumerate(self.sims):
                if dev:
                    import torch
                    o = torch.empty(shapes[key](sim.n), dtype=torch.float32, device=dl_dloc[i].device)
                    t[i] = o.data_ptr()
                else:
                    o = np.empty(shapes[key](sim.n), dtype=np.float32)
                    t[i] = o.ctypes.data
                outs[i][key] = o
            tabs[key] = t
        stream = _stream_for(dl_dloc[0])
        self._ok(self._lib.mpm_batch_adjoint(self._b, tl, tv, tabs["youngs_modulus"], tabs["loc"],
                                             tabs["velocity"], dev or 0, stream))
        return outs
