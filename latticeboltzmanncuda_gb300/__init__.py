"""GB300-native lattice Boltzmann collide-stream step.

The compute path is liblbm_gb300.so (hand-written sm_103a CUDA kernels behind the C ABI of
include/lbm_capi.h).  This package is the Python host side over that ABI: ``Lattice`` owns one
library context; the generators produce seeded flag masks.  A C++ layer with the reference's own
class names (Lattice, RunCudaFunctions, ... of simulation/include) sits on the same ABI in
``simulation/``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi
from .capi import (BF16S, D2Q9, D3Q27_REF, F16S, F32, F64, FLUID, FORCE_MOMENTUM_EXCHANGE,
                   FORCE_REFERENCE, INTERNAL, LATTICE_POINT, MOVING_WALL, OP_COLLIDE, OP_FLOW,
                   OP_REFLECT, OP_STREAM, ORDER_CLI, ORDER_STREAM_COLLIDE, REFLECTED,
                   REFLECTION_VALUES, SOURCE, WALL, LBMError, check, ptr)

__all__ = ["Lattice", "Batch", "Mesh", "serve", "gen_channel", "gen_cavity", "gen_disks_fraction", "rotate_vector",
           "distribute_vector", "LBMError", "capi"]


def _mode(mode):
    return capi.MODES[mode] if isinstance(mode, str) else int(mode)


def _dtype(dtype):
    return capi.DTYPES[dtype] if isinstance(dtype, str) else int(dtype)


class Lattice:
    """One library context: a D2Q9 domain or a D3Q27_REF lattice resident on one GPU."""

    def __init__(self, nx, ny, nz=1, *, mode="d2q9", dtype="f32", tau=1.0, periodic=0,
                 body_force=(0.0, 0.0, 0.0), wall_velocity=(0.0, 0.0, 0.0), order=ORDER_STREAM_COLLIDE,
                 force_mode=FORCE_REFERENCE, device=0, stream=None):
        L = capi.lib()
        d = capi.Desc()
        L.lbm_desc_init(ctypes.byref(d))
        d.mode, d.dtype = _mode(mode), _dtype(dtype)
        d.nx, d.ny, d.nz = int(nx), int(ny), int(nz)
        d.periodic = int(periodic)
        d.tau = float(tau)
        for k in range(3):
            d.body_force[k] = float(body_force[k]) if k < len(body_force) else 0.0
            d.wall_velocity[k] = float(wall_velocity[k]) if k < len(wall_velocity) else 0.0
        d.order, d.force_mode, d.device = int(order), int(force_mode), int(device)
        d.stream = stream
        self.desc = d
        self._ctx = ctypes.c_void_p()
        check(L.lbm_create(ctypes.byref(d), ctypes.byref(self._ctx)))
        self.mode = d.mode
        self.shape = (int(nx), int(ny), int(nz))
        self.cells = int(nx) * int(ny) * int(nz)
        self.q = 9 if d.mode == D2Q9 else 27

    # ------------------------------------------------------------------ life cycle
    def close(self):
        if getattr(self, "_ctx", None) and self._ctx.value:
            capi.lib().lbm_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _call(self, name, *args):
        check(getattr(capi.lib(), name)(self._ctx, *args), self._ctx)

    @property
    def handle(self):
        return self._ctx

    def info(self) -> dict:
        i = capi.Info()
        self._call("lbm_get_info", ctypes.byref(i))
        return {k: getattr(i, k) for k, _ in capi.Info._fields_}

    @property
    def stream(self) -> int:
        s = ctypes.c_void_p()
        self._call("lbm_get_stream", ctypes.byref(s))
        return s.value or 0

    def synchronize(self):
        self._call("lbm_synchronize")

    def set_params(self, tau, body_force=None, wall_velocity=None):
        bf = None if body_force is None else np.array(list(body_force) + [0.0] * (3 - len(body_force)), np.float32)
        wv = None if wall_velocity is None else np.array(list(wall_velocity) + [0.0] * (3 - len(wall_velocity)), np.float32)
        self._call("lbm_set_params", float(tau), ptr(bf), ptr(wv))

    # ------------------------------------------------------------------ geometry and state
    def _host_shape(self):
        nx, ny, nz = self.shape
        return (ny, nx) if self.mode == D2Q9 else (self.cells,)

    def set_flags(self, flags):
        a = np.ascontiguousarray(flags, dtype=np.uint8).reshape(-1)
        if a.size != self.cells:
            raise LBMError(capi.ERR_INVALID, f"flags need {self.cells} cells, got {a.size}")
        self._call("lbm_set_flags", ptr(a))

    def get_flags(self):
        a = np.empty(self.cells, np.uint8)
        self._call("lbm_get_flags", ptr(a))
        return a.reshape(self._host_shape())

    def init_equilibrium(self, rho=None, ux=None, uy=None):
        arrs = [None if v is None else np.ascontiguousarray(v, dtype=np.float32).reshape(-1) for v in (rho, ux, uy)]
        for v in arrs:
            if v is not None and v.size != self.cells:
                raise LBMError(capi.ERR_INVALID, "field size mismatch")
        self._call("lbm_init_equilibrium", *[ptr(v) for v in arrs])

    def _pop_shape(self):
        nx, ny, nz = self.shape
        return (9, ny, nx) if self.mode == D2Q9 else (self.cells, 27)

    def load_populations(self, f):
        f = np.asarray(f)
        dt = F64 if f.dtype == np.float64 else F32
        a = np.ascontiguousarray(f, dtype=np.float64 if dt == F64 else np.float32)
        if a.size != self.cells * self.q:
            raise LBMError(capi.ERR_INVALID, f"populations need {self.cells * self.q} values, got {a.size}")
        self._call("lbm_load_populations", ptr(a), dt)

    def retrieve_populations(self, dtype=np.float32, out=None):
        dtype = np.dtype(dtype)
        a = np.empty(self._pop_shape(), dtype) if out is None else out
        self._call("lbm_retrieve_populations", ptr(a), F64 if dtype == np.float64 else F32)
        return a

    def load_aos(self, points):
        a = np.ascontiguousarray(points, dtype=LATTICE_POINT)
        self._call("lbm_load_aos", ptr(a), int(a.size))

    def retrieve_aos(self):
        a = np.zeros(self.cells, LATTICE_POINT)
        self._call("lbm_retrieve_aos", ptr(a), int(a.size))
        return a

    def set_reflection_tables(self, cells, records):
        c = np.ascontiguousarray(cells, dtype=np.int32)
        r = np.ascontiguousarray(records, dtype=REFLECTION_VALUES)
        self._call("lbm_set_reflection_tables", int(c.size), ptr(c), ptr(r))

    def set_flow(self, mask=None, induced=None):
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8).reshape(-1)
        i = None if induced is None else np.ascontiguousarray(induced, dtype=np.float32)
        self._call("lbm_set_flow", ptr(m), ptr(i))

    def set_force(self, value=(0.0, 0.0, 0.0), enabled=True):
        v = np.ascontiguousarray(value, dtype=np.float32)
        self._call("lbm_set_force", ptr(v), int(bool(enabled)))

    def get_force(self):
        v = np.zeros(3, np.float32)
        self._call("lbm_get_force", ptr(v))
        return v

    # ------------------------------------------------------------------ stepping
    def step(self, n=1):
        self._call("lbm_step", int(n))

    def apply(self, op):
        self._call("lbm_apply", int(op))

    def set_equilibrium_evaluation(self, mode):
        """D3Q27_REF: "float_float" (or False; the default, float-float with FP64 fallback, bit for bit
        the reference's FP64 value), "fp64" (or True; FP64 throughout), "fp32" (FP32 throughout)."""
        modes = {"float_float": capi.EQ_FLOAT_FLOAT, "fp64": capi.EQ_FP64, "fp32": capi.EQ_FP32,
                 False: capi.EQ_FLOAT_FLOAT, True: capi.EQ_FP64}
        self._call("lbm_set_equilibrium_evaluation", modes[mode] if mode in modes else int(mode))

    def set_order(self, order):
        """D3Q27_REF: step order of later step() calls (ORDER_STREAM_COLLIDE or ORDER_CLI)."""
        self._call("lbm_set_order", int(order))

    def step_force_series(self, nsteps):
        """D3Q27_REF: step nsteps and return the accumulated force after every step, float32[nsteps, 3]."""
        out = np.zeros((int(nsteps), 3), np.float32)
        self._call("lbm_step_force_series", int(nsteps), ptr(out))
        return out

    def autotune(self, retune=False):
        """Run the launch-shape tuner; returns (cells_per_thread, block_threads, rows_per_block, l2_policy)."""
        self._call("lbm_autotune", int(bool(retune)))
        i = self.info()
        return i["cells_per_thread"], i["block_threads"], i["rows_per_block"], i["l2_policy"]

    def set_launch(self, cells_per_thread, block_threads, rows_per_block=1, l2_policy=0):
        self._call("lbm_set_launch", int(cells_per_thread), int(block_threads), int(rows_per_block), int(l2_policy))

    def set_sweep_alternation(self, enabled):
        self._call("lbm_set_sweep_alternation", int(bool(enabled)))

    def set_pipeline_wait(self, wait_ns=1_000_000_000, skip_task=-1):
        """Bulk-copy pipeline: the limit of its waits, and (diagnostic) a task whose copies it leaves
        out so that the wait for them gives up (the next synchronisation raises LBM_ERR_TIMEOUT)."""
        self._call("lbm_set_pipeline_wait", int(wait_ns), int(skip_task))

    # ------------------------------------------------------------------ checkpoint
    def save(self, path):
        """Write the context's state to `path` (lbm_save); load() resumes it bit for bit."""
        self._call("lbm_save", str(path).encode())

    def load(self, path):
        """Restore a checkpoint written by save() into this context (same mode, storage and size)."""
        self._call("lbm_load", str(path).encode())

    @classmethod
    def from_checkpoint(cls, path, device=0, stream=None):
        """A context created from a checkpoint's descriptor with its state loaded."""
        d = capi.Desc()
        check(capi.lib().lbm_checkpoint_desc(str(path).encode(), ctypes.byref(d)))
        names = {v: k for k, v in capi.MODES.items()}
        L = cls(d.nx, d.ny, d.nz, mode=names[d.mode], dtype=d.dtype, tau=d.tau, periodic=d.periodic,
                body_force=tuple(d.body_force), wall_velocity=tuple(d.wall_velocity), order=d.order,
                force_mode=d.force_mode, device=device, stream=stream)
        L.load(path)
        return L

    # ------------------------------------------------------------------ results
    def moments(self, out=None):
        """(rho, ux, uy) for D2Q9, (rho, ux, uy, uz) for D3Q27_REF; `out` may give float32 arrays
        (for example pinned host memory) to write into."""
        shp = self._host_shape()
        n = 4 if self.mode == D3Q27_REF else 3
        if out is None:
            out = [np.empty(shp, np.float32) for _ in range(n)]
        for o in out:
            if o is not None and (o.dtype != np.float32 or o.size != self.cells or not o.flags.c_contiguous):
                raise LBMError(capi.ERR_INVALID, "moment outputs must be contiguous float32 arrays of one value per cell")
        args = [ptr(o) for o in out] + [None] * (4 - len(out))
        self._call("lbm_moments", *args)
        return tuple(out)

    def conservation(self):
        out = np.zeros(4, np.float64)
        self._call("lbm_conservation", ptr(out))
        return out


def gen_channel(nx, ny, ndisks, rmin, rmax, seed):
    flags = np.empty((ny, nx), np.uint8)
    disks = np.empty((max(ndisks, 1), 3), np.float32)
    check(capi.lib().lbm_gen_channel(int(nx), int(ny), int(ndisks), float(rmin), float(rmax),
                                     ctypes.c_uint64(int(seed)), ptr(flags), ptr(disks)))
    return flags, disks[:ndisks]


def gen_cavity(nx, ny):
    flags = np.empty((ny, nx), np.uint8)
    check(capi.lib().lbm_gen_cavity(int(nx), int(ny), ptr(flags)))
    return flags


def gen_disks_fraction(flags, solid_fraction, rmin, rmax, seed):
    flags = np.ascontiguousarray(flags, dtype=np.uint8).copy()
    ny, nx = flags.shape
    ach = ctypes.c_float()
    check(capi.lib().lbm_gen_disks_fraction(int(nx), int(ny), float(solid_fraction), float(rmin), float(rmax),
                                            ctypes.c_uint64(int(seed)), ptr(flags), ctypes.byref(ach)))
    return flags, float(ach.value)


class Mesh:
    """A triangle mesh for the D3Q27_REF geometry front end (Model, Model.cpp:22-91; host only)."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def load_obj(cls, path):
        h = ctypes.c_void_p()
        check(capi.lib().lbm_mesh_load_obj(str(path).encode(), ctypes.byref(h)))
        return cls(h)

    @classmethod
    def from_arrays(cls, vertices, faces):
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        sizes = np.ascontiguousarray([len(f) for f in faces], dtype=np.int32)
        idx = np.ascontiguousarray([i for f in faces for i in f], dtype=np.int32)
        h = ctypes.c_void_p()
        check(capi.lib().lbm_mesh_create(ptr(v), int(len(v)), ptr(sizes), int(len(sizes)), ptr(idx), ctypes.byref(h)))
        return cls(h)

    def close(self):
        if self._h:
            capi.lib().lbm_mesh_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def info(self) -> dict:
        i = capi.MeshInfo()
        check(capi.lib().lbm_mesh_get_info(self._h, ctypes.byref(i)))
        return {"vertices": i.vertices, "faces": i.faces, "triangle_mesh": bool(i.triangle_mesh),
                "closed": bool(i.closed), "valid": bool(i.valid), "bbox_min": tuple(i.bbox_min),
                "bbox_max": tuple(i.bbox_max)}

    def point_inside(self, p) -> bool:
        pt = (ctypes.c_float * 3)(*[float(v) for v in p])
        out = ctypes.c_int32()
        check(capi.lib().lbm_mesh_point_inside(self._h, pt, ctypes.byref(out)))
        return bool(out.value)

    def reflection_vector(self, p1, p2):
        a = (ctypes.c_float * 3)(*[float(v) for v in p1])
        b = (ctypes.c_float * 3)(*[float(v) for v in p2])
        out = (ctypes.c_float * 3)()
        check(capi.lib().lbm_mesh_reflection_vector(self._h, a, b, out))
        return np.array(out[:], dtype=np.float32)

    def rasterize(self, dims, spacing, flags=None):
        """Lattice::insertModel: returns (flags[X*Y*Z] with LBM_INTERNAL set/cleared, applied)."""
        X, Y, Z = (int(d) for d in dims)
        fl = np.zeros(X * Y * Z, np.uint8) if flags is None else np.ascontiguousarray(flags, dtype=np.uint8).reshape(-1).copy()
        applied = ctypes.c_int32()
        check(capi.lib().lbm_mesh_rasterize(self._h, X, Y, Z, float(spacing), ptr(fl), ctypes.byref(applied)))
        return fl, bool(applied.value)

    def reflection_tables(self, dims, spacing, flags):
        """Lattice::preProcessModel: returns (cells, records, flags with LBM_REFLECTED added)."""
        X, Y, Z = (int(d) for d in dims)
        fl = np.ascontiguousarray(flags, dtype=np.uint8).reshape(-1).copy()
        n = ctypes.c_int64()
        L = capi.lib()
        check(L.lbm_mesh_reflection_tables(self._h, X, Y, Z, float(spacing), ptr(fl), 0, None, None, ctypes.byref(n)))
        cells = np.zeros(n.value, np.int32)
        recs = np.zeros(n.value, REFLECTION_VALUES)
        if n.value:
            check(L.lbm_mesh_reflection_tables(self._h, X, Y, Z, float(spacing), ptr(fl), n.value, ptr(cells), ptr(recs),
                                               ctypes.byref(n)))
        return cells, recs, fl


def rotate_vector(axis, v, angle):
    """rotateVectorAroundAxis (Geometry.cpp:22-42)."""
    a = (ctypes.c_float * 3)(*[float(x) for x in axis])
    b = (ctypes.c_float * 3)(*[float(x) for x in v])
    out = (ctypes.c_float * 3)()
    capi.lib().lbm_rotate_vector(a, b, ctypes.c_float(float(angle)), out)
    return np.array(out[:], dtype=np.float32)


def distribute_vector(v):
    """Lattice::distributeVector (Lattice.cpp:262-321): (scores[27], directions[27]), best first."""
    a = (ctypes.c_float * 3)(*[float(x) for x in v])
    score = np.zeros(27, np.float32)
    dirs = np.zeros(27, np.int32)
    capi.lib().lbm_distribute_vector(a, ptr(score), ptr(dirs))
    return score, dirs


def _desc_for(nx, ny, tau, periodic=0, body_force=(0.0, 0.0), wall_velocity=(0.0, 0.0)):
    d = capi.Desc()
    capi.lib().lbm_desc_init(ctypes.byref(d))
    d.mode = D2Q9
    d.nx, d.ny, d.nz = int(nx), int(ny), 1
    d.tau = float(tau)
    d.periodic = int(periodic)
    for k in range(2):
        d.body_force[k] = float(body_force[k])
        d.wall_velocity[k] = float(wall_velocity[k])
    return d


class Batch:
    """Many independent D2Q9 domains advanced together, one launch per time step (lbm_batch_*)."""

    def __init__(self, dtype="f32", device=0, stream=None):
        self._b = ctypes.c_void_p()
        check(capi.lib().lbm_batch_create(_dtype(dtype), int(device), stream, ctypes.byref(self._b)))
        self.shapes = {}

    def _chk(self, status):
        if status != capi.OK:
            raise LBMError(status, (capi.lib().lbm_batch_last_error(self._b) or b"").decode())

    def close(self):
        if getattr(self, "_b", None) and self._b.value:
            capi.lib().lbm_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @staticmethod
    def slot_bytes(dtype, nx, ny):
        return int(capi.lib().lbm_batch_slot_bytes(_dtype(dtype), int(nx), int(ny)))

    def add(self, nx, ny, tau, flags=None, periodic=0, body_force=(0.0, 0.0), wall_velocity=(0.0, 0.0)):
        d = _desc_for(nx, ny, tau, periodic, body_force, wall_velocity)
        fl = None if flags is None else np.ascontiguousarray(flags, dtype=np.uint8).reshape(-1)
        if fl is not None and fl.size != nx * ny:
            raise LBMError(capi.ERR_INVALID, "flags size mismatch")
        slot = ctypes.c_int32()
        self._chk(capi.lib().lbm_batch_add(self._b, ctypes.byref(d), ptr(fl), ctypes.byref(slot)))
        self.shapes[slot.value] = (int(nx), int(ny))
        return slot.value

    def remove(self, slot):
        self._chk(capi.lib().lbm_batch_remove(self._b, int(slot)))
        self.shapes.pop(slot, None)

    def step(self, n=1):
        self._chk(capi.lib().lbm_batch_step(self._b, int(n)))

    def autotune(self):
        self._chk(capi.lib().lbm_batch_autotune(self._b))
        return self.info()

    def set_launch(self, cells_per_thread, block_threads, rows_per_block):
        self._chk(capi.lib().lbm_batch_set_launch(self._b, int(cells_per_thread), int(block_threads), int(rows_per_block)))

    def synchronize(self):
        self._chk(capi.lib().lbm_batch_synchronize(self._b))

    def set_persistent(self, mode=1, wait_ns=1_000_000_000, skip_block=-1):
        """Step sequences as one persistent launch: mode 0 never (the batch's default), 1 batches of
        at most 2^19 live cells, 2 whenever the tile shape allows; skip_block >= 0 is a diagnostic
        that makes the launch's wait run out (synchronize then raises LBM_ERR_TIMEOUT)."""
        self._chk(capi.lib().lbm_batch_set_persistent(self._b, int(mode), int(wait_ns), int(skip_block)))

    @property
    def stream(self):
        s = ctypes.c_void_p()
        self._chk(capi.lib().lbm_batch_get_stream(self._b, ctypes.byref(s)))
        return s.value or 0

    def info(self):
        out = np.zeros(8, np.int64)
        self._chk(capi.lib().lbm_batch_info(self._b, ptr(out)))
        keys = ("slots", "cells", "fluid_cells", "device_bytes", "cells_per_thread", "block_threads",
                "rows_per_block", "tiles")
        return dict(zip(keys, (int(v) for v in out)))

    def set_slot_steps(self, slot, steps):
        """Step budget of a slot (-1: none): later steps advance it by at most `steps` in total."""
        self._chk(capi.lib().lbm_batch_set_slot_steps(self._b, int(slot), int(steps)))

    def steps_done(self, slot):
        v = ctypes.c_int64()
        self._chk(capi.lib().lbm_batch_slot_steps(self._b, int(slot), ctypes.byref(v)))
        return v.value

    def moments(self, slot):
        nx, ny = self.shapes[slot]
        out = [np.empty((ny, nx), np.float32) for _ in range(3)]
        self._chk(capi.lib().lbm_batch_moments(self._b, int(slot), *[ptr(o) for o in out]))
        return tuple(out)

    def moments_async(self, slot):
        """Queue the read-back of a slot's density and velocity; returns a ticket for collect()."""
        t = ctypes.c_int64(0)
        self._chk(capi.lib().lbm_batch_moments_async(self._b, int(slot), ctypes.byref(t)))
        return t.value, self.shapes[slot]

    def collect(self, ticket, wait=True):
        """(rho, ux, uy) of a ticket from moments_async(), or None while its copy is still running
        (wait=False)."""
        tid, (nx, ny) = ticket
        out = [np.empty((ny, nx), np.float32) for _ in range(3)]
        ready = ctypes.c_int32(0)
        self._chk(capi.lib().lbm_batch_collect(self._b, int(tid), int(bool(wait)), *[ptr(o) for o in out],
                                               ctypes.byref(ready)))
        return tuple(out) if ready.value else None

    def load_populations(self, slot, f):
        f = np.asarray(f)
        dt = F64 if f.dtype == np.float64 else F32
        a = np.ascontiguousarray(f, dtype=np.float64 if dt == F64 else np.float32)
        self._chk(capi.lib().lbm_batch_load_populations(self._b, int(slot), ptr(a), dt))

    def retrieve_populations(self, slot, dtype=np.float32):
        nx, ny = self.shapes[slot]
        dtype = np.dtype(dtype)
        a = np.empty((9, ny, nx), dtype)
        self._chk(capi.lib().lbm_batch_retrieve_populations(self._b, int(slot), ptr(a),
                                                            F64 if dtype == np.float64 else F32))
        return a


def serve(requests, dtype="f32", budget_bytes=150e9, max_slots=0, round_steps=200, time_limit=0.0,
          outputs=False, device=0, stream=None):
    """Play `requests` (objects with nx, ny, tau, flags, periodic, body_force, wall_velocity, steps
    and arrival in seconds) through the continuous-batching server (lbm_server_run).  Returns
    (results, stats, run_status): per request a dict with status, admitted, finished, latency and,
    with outputs=True (every request) or a collection of request indices (those requests),
    (rho, ux, uy)."""
    L = capi.lib()
    cfg = capi.ServerConfig()
    L.lbm_server_config_init(ctypes.byref(cfg))
    cfg.dtype, cfg.device = _dtype(dtype), int(device)
    cfg.budget_bytes, cfg.max_slots, cfg.round_steps = int(budget_bytes), int(max_slots), int(round_steps)
    cfg.time_limit, cfg.stream = float(time_limit), stream
    srv = ctypes.c_void_p()
    check(L.lbm_server_create(ctypes.byref(cfg), ctypes.byref(srv)))
    n = len(requests)
    arr = (capi.Request * max(n, 1))()
    keep, outs = [], []
    for i, r in enumerate(requests):
        q = arr[i]
        q.nx, q.ny, q.tau, q.periodic = int(r.nx), int(r.ny), float(r.tau), int(r.periodic)
        q.body_force[0], q.body_force[1] = float(r.body_force[0]), float(r.body_force[1])
        q.wall_velocity[0], q.wall_velocity[1] = float(r.wall_velocity[0]), float(r.wall_velocity[1])
        fl = None if r.flags is None else np.ascontiguousarray(r.flags, dtype=np.uint8)
        keep.append(fl)
        q.flags = None if fl is None else fl.ctypes.data
        q.steps, q.arrival = int(r.steps), float(r.arrival)
        if outputs is True or (outputs and i in outputs):
            o = [np.zeros((r.ny, r.nx), np.float32) for _ in range(3)]
            outs.append(o)
            q.out_rho, q.out_ux, q.out_uy = (a.ctypes.data for a in o)
        else:
            outs.append(None)
    res = (capi.RequestResult * max(n, 1))()
    st = capi.ServerStats()
    try:
        status = L.lbm_server_run(srv, arr, n, res, ctypes.byref(st))
    finally:
        L.lbm_server_destroy(srv)
    results = []
    for i in range(n):
        d = {"status": res[i].status, "admitted": res[i].admitted, "finished": res[i].finished,
             "latency": res[i].finished - float(requests[i].arrival)}
        if outs[i] is not None:
            d["moments"] = tuple(outs[i])
        results.append(d)
    stats = {k: getattr(st, k) for k, _ in capi.ServerStats._fields_}
    stats["tile_shape"] = list(stats["tile_shape"])
    return results, stats, status
