"""ctypes binding of liblbdem_gb300 (the C ABI in include/lbdem_gpu.h).

This is a thin host-side mirror of the reference's coupling surface for Python
callers and tests:

    reference (LBDEMcoupling, Palabos side)        here
    setSpheresOnLattice(lattice, wrapper, ...)     Lattice.set_particles(...)
    lattice.collideAndStream()                     Lattice.collide_and_stream()
    getForcesFromLattice(lattice, wrapper, ...)    Lattice.get_forces(n)

There is no CPU fallback: constructing a Lattice without the built library or
without a GB300 raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "liblbdem_gb300.so"

PREC_FP64 = 0
PREC_FP32_DEV = 1
FLAG_CELL_FORCE = 0x1
FLAG_PROBE_TIMEOUT = 0x2

FIELD_POPULATIONS = 0
FIELD_SOLID_FRACTION = 1
FIELD_PARTICLE_ID = 2
FIELD_PARTICLE_VELOCITY = 3
FIELD_HYDRO_FORCE = 4
FIELD_DENSITY = 5
FIELD_VELOCITY = 6
FIELD_SUBCELL_COUNT = 7

DEVERR_TILE_LIST = 0x1
DEVERR_TAG_RANGE = 0x4
DEVERR_UNMAPPED_TAG = 0x8
DEVERR_RADIUS = 0x10
DEVERR_TIMEOUT = 0x20

STATUS = {0: "LBDEM_OK", 1: "LBDEM_ERR_INVALID_ARG", 2: "LBDEM_ERR_CUDA", 3: "LBDEM_ERR_OUT_OF_MEMORY",
          4: "LBDEM_ERR_CAPACITY", 5: "LBDEM_ERR_DEVICE", 6: "LBDEM_ERR_NO_DEVICE"}

# Every function the C ABI exports, with (restype, argtypes).
_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I = C.c_int32


class Config(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("periodic", C.c_int32 * 3), ("omega", C.c_double), ("body_force", C.c_double * 3),
                ("precision", C.c_int32), ("device", C.c_int32), ("max_particles", C.c_int32),
                ("max_tag", C.c_int32), ("max_radius", C.c_double), ("flags", C.c_int32),
                ("reserved", C.c_int32)]


class PressureDrop(C.Structure):
    _fields_ = [("dimension", C.c_int32), ("inlet", C.c_int32 * 6), ("outlet", C.c_int32 * 6),
                ("in_direction", C.c_int32), ("out_direction", C.c_int32),
                ("rho_in", C.c_double), ("rho_out", C.c_double)]


class Domain(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("periodic", C.c_int32 * 3),
                ("omega", C.c_double), ("body_force", C.c_double * 3), ("max_particles", C.c_int32),
                ("has_pressure_drop", C.c_int32), ("drop", PressureDrop)]


class BatchConfig(C.Structure):
    _fields_ = [("precision", C.c_int32), ("device", C.c_int32), ("max_tag", C.c_int32),
                ("max_radius", C.c_double), ("use_graph", C.c_int32), ("autotune", C.c_int32),
                ("reserved", C.c_int32 * 2)]


PROFILE_PRESSURE_GRADIENT = 0
PROFILE_POISEUILLE = 1

SIGNATURES = {
    "lbdem_config_default": (None, [C.POINTER(Config)]),
    "lbdem_debug_fail_allocation": (None, [_I]),
    "lbdem_create": (C.c_int, [C.POINTER(Config), C.POINTER(_P)]),
    "lbdem_destroy": (C.c_int, [_P]),
    "lbdem_last_error": (C.c_char_p, [_P]),
    "lbdem_status_string": (C.c_char_p, [C.c_int]),
    "lbdem_set_stream": (C.c_int, [_P, _P]),
    "lbdem_set_omega": (C.c_int, [_P, C.c_double]),
    "lbdem_set_periodic": (C.c_int, [_P, C.POINTER(_I)]),
    "lbdem_synchronize": (C.c_int, [_P]),
    "lbdem_init_equilibrium": (C.c_int, [_P, C.c_double, _D]),
    "lbdem_set_populations": (C.c_int, [_P, _P]),
    "lbdem_get_populations": (C.c_int, [_P, _P]),
    "lbdem_set_particles": (C.c_int, [_P, _I, _D, _D, _D, _D, C.POINTER(_I), _I]),
    "lbdem_set_particles_device": (C.c_int, [_P, _I, _P, _I]),
    "lbdem_collide_and_stream": (C.c_int, [_P]),
    "lbdem_get_forces": (C.c_int, [_P, _I, _D, _D]),
    "lbdem_get_forces_device": (C.c_int, [_P, _I, _P]),
    "lbdem_cycle": (C.c_int, [_P, _I, _D, _D, _D, _D, C.POINTER(_I), _I, _D, _D]),
    "lbdem_get_field": (C.c_int, [_P, _I, _P]),
    "lbdem_mass": (C.c_int, [_P, _D]),
    "lbdem_get_device_errors": (C.c_int, [_P, C.POINTER(C.c_uint32)]),
    "lbdem_get_step": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "lbdem_device_bytes": (C.c_int, [_P, C.POINTER(C.c_size_t)]),
    "lbdem_get_launch_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "lbdem_voxelize_static": (C.c_int, [_I, _I, _I, _I, _I, _P, _P, _P, _P, _P]),
    "lbdem_average_density": (C.c_int, [_P, C.POINTER(_I), _D]),
    "lbdem_zhang_rescale": (C.c_int, [_P, C.POINTER(_I), _I, _I, C.c_double, C.c_double]),
    "lbdem_set_pressure_drop": (C.c_int, [_P, C.POINTER(PressureDrop)]),
    "lbdem_init_profile": (C.c_int, [_P, _I, C.c_double, C.c_double, C.c_double, C.POINTER(_I), _I]),
    "lbdem_save_state": (C.c_int, [_P, C.c_char_p]),
    "lbdem_load_state": (C.c_int, [_P, C.c_char_p]),
    "lbdem_adjoint_window": (C.c_int, [_P, _I, _I, _I, _D, _D, _D, _D, _D, _D, _P]),
    "lbdem_adjoint_timing": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "lbdem_batch_config_default": (None, [C.POINTER(BatchConfig)]),
    "lbdem_batch_create": (C.c_int, [C.POINTER(BatchConfig), _I, C.POINTER(Domain), C.POINTER(_P)]),
    "lbdem_batch_destroy": (C.c_int, [_P]),
    "lbdem_batch_last_error": (C.c_char_p, [_P]),
    "lbdem_batch_init_equilibrium": (C.c_int, [_P, C.c_double, _D]),
    "lbdem_batch_init_profile": (C.c_int, [_P, _I, _I, C.c_double, C.c_double, C.c_double, C.POINTER(_I), _I]),
    "lbdem_batch_set_particles": (C.c_int, [_P, C.POINTER(_I), _D, _I]),
    "lbdem_batch_step": (C.c_int, [_P]),
    "lbdem_batch_get_forces": (C.c_int, [_P, _D, _D]),
    "lbdem_batch_cycle": (C.c_int, [_P, C.POINTER(_I), _D, _I, _D, _D]),
    "lbdem_batch_get_field": (C.c_int, [_P, _I, _I, _P]),
    "lbdem_batch_synchronize": (C.c_int, [_P]),
    "lbdem_batch_get_step": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "lbdem_batch_get_launch_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "lbdem_batch_device_bytes": (C.c_int, [_P, C.POINTER(C.c_size_t)]),
    "lbdem_batch_cells": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "lbdem_batch_get_tuning": (C.c_int, [_P, C.POINTER(_I), C.POINTER(C.c_float)]),
    "lbdem_batch_set_tuning": (C.c_int, [_P, _I]),
}

def debug_fail_allocation(nth: int):
    """lbdem_debug_fail_allocation: the nth allocation of a creation from now on fails (0: off)."""
    load().lbdem_debug_fail_allocation(int(nth))


# Limits of lbdem_voxelize_static (include/lbdem_gpu.h).
STATIC_MAX_SPHERES = 4096
STATIC_MAX_TILES = 4096
STATIC_MAX_TAG = 65535


def voxelize_static(shape, precision, n, rec_ptr, vox_ptr, up_ptr, err_ptr, stream_ptr=None) -> int:
    """lbdem_voxelize_static on device pointers; returns the lbdem_status."""
    lib = load()
    nx, ny, nz = (int(s) for s in shape)
    return int(lib.lbdem_voxelize_static(nx, ny, nz, int(precision), int(n), _P(rec_ptr), _P(vox_ptr),
                                         _P(up_ptr), _P(err_ptr), _P(stream_ptr) if stream_ptr else None))

_lib = None


def load(path: os.PathLike | None = None) -> C.CDLL:
    """Loads the shared library (raises if it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"liblbdem_gb300 not built: {p} missing (run build())")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class LbdemError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(_D)


def _c64(a, shape=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


class Lattice:
    """A D3Q19 PSM lattice resident on the GPU (one handle of the C ABI)."""

    def __init__(self, nx, ny, nz, omega, periodic=(1, 1, 1), precision=PREC_FP64, body_force=(0, 0, 0),
                 max_particles=1024, max_tag=1 << 20, max_radius=16.0, flags=0, device=0):
        self.lib = load()
        cfg = Config()
        self.lib.lbdem_config_default(C.byref(cfg))
        cfg.nx, cfg.ny, cfg.nz = int(nx), int(ny), int(nz)
        for d in range(3):
            cfg.periodic[d] = int(periodic[d])
            cfg.body_force[d] = float(body_force[d])
        cfg.omega = float(omega)
        cfg.precision = int(precision)
        cfg.device = int(device)
        cfg.max_particles = int(max_particles)
        cfg.max_tag = int(max_tag)
        cfg.max_radius = float(max_radius)
        cfg.flags = int(flags)
        self.cfg = cfg
        self.shape = (int(nx), int(ny), int(nz))
        self.N = int(nx) * int(ny) * int(nz)
        self.dtype = np.float64 if precision == PREC_FP64 else np.float32
        h = _P()
        st = self.lib.lbdem_create(C.byref(cfg), C.byref(h))
        if st != 0:
            raise LbdemError(st, self.lib.lbdem_status_string(st).decode())
        self.h = h
        self.n = 0

    # -- life cycle -------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.lbdem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st: int):
        if st != 0:
            raise LbdemError(st, self.lib.lbdem_last_error(self.h).decode())

    # -- state ------------------------------------------------------------
    def set_omega(self, omega):
        self._check(self.lib.lbdem_set_omega(self.h, float(omega)))

    def set_periodic(self, periodic):
        p = (_I * 3)(*[int(x) for x in periodic])
        self._check(self.lib.lbdem_set_periodic(self.h, p))

    def init_equilibrium(self, rho_bar=0.0, u=(0.0, 0.0, 0.0)):
        uu = _c64(u)
        self._check(self.lib.lbdem_init_equilibrium(self.h, float(rho_bar), _dptr(uu)))

    def set_populations(self, f: np.ndarray):
        f = np.ascontiguousarray(f, dtype=self.dtype).reshape(19, *self.shape)
        self._check(self.lib.lbdem_set_populations(self.h, f.ctypes.data_as(_P)))

    def get_populations(self) -> np.ndarray:
        out = np.empty((19, *self.shape), dtype=self.dtype)
        self._check(self.lib.lbdem_get_populations(self.h, out.ctypes.data_as(_P)))
        return out

    def get_field(self, which: int) -> np.ndarray:
        shapes = {
            FIELD_POPULATIONS: ((19, *self.shape), self.dtype),
            FIELD_SOLID_FRACTION: (self.shape, np.float64),
            FIELD_PARTICLE_ID: (self.shape, np.int32),
            FIELD_PARTICLE_VELOCITY: ((3, *self.shape), self.dtype),
            FIELD_HYDRO_FORCE: ((3, *self.shape), self.dtype),
            FIELD_DENSITY: (self.shape, np.float64),
            FIELD_VELOCITY: ((3, *self.shape), np.float64),
            FIELD_SUBCELL_COUNT: (self.shape, np.uint8),
        }
        shp, dt = shapes[which]
        out = np.empty(shp, dtype=dt)
        self._check(self.lib.lbdem_get_field(self.h, int(which), out.ctypes.data_as(_P)))
        return out

    # -- coupling cycle ---------------------------------------------------
    def set_particles(self, x, v, w, r, tag, init_vel=False):
        x = _c64(x).reshape(-1, 3)
        n = x.shape[0]
        v = _c64(v).reshape(n, 3)
        w = _c64(w).reshape(n, 3)
        r = _c64(r).reshape(n)
        tag = np.ascontiguousarray(tag, dtype=np.int32).reshape(n)
        self._keep = (x, v, w, r, tag)
        self._check(self.lib.lbdem_set_particles(self.h, n, _dptr(x), _dptr(v), _dptr(w), _dptr(r),
                                                 tag.ctypes.data_as(C.POINTER(_I)), int(bool(init_vel))))
        self.n = n

    def set_particles_device(self, n: int, rec_ptr: int, init_vel=False):
        self._check(self.lib.lbdem_set_particles_device(self.h, int(n), _P(rec_ptr), int(bool(init_vel))))
        self.n = n

    def collide_and_stream(self):
        self._check(self.lib.lbdem_collide_and_stream(self.h))

    def get_forces(self):
        F = np.zeros((self.n, 3))
        T = np.zeros((self.n, 3))
        self._check(self.lib.lbdem_get_forces(self.h, self.n, _dptr(F), _dptr(T)))
        return F, T

    def get_forces_device(self, dev_ptr: int):
        self._check(self.lib.lbdem_get_forces_device(self.h, self.n, _P(dev_ptr)))

    def cycle(self, x, v, w, r, tag, init_vel=False, F=None, T=None):
        x = _c64(x).reshape(-1, 3)
        n = x.shape[0]
        v = _c64(v).reshape(n, 3)
        w = _c64(w).reshape(n, 3)
        r = _c64(r).reshape(n)
        tag = np.ascontiguousarray(tag, dtype=np.int32).reshape(n)
        if F is None:
            F = np.zeros((n, 3))
        if T is None:
            T = np.zeros((n, 3))
        self._check(self.lib.lbdem_cycle(self.h, n, _dptr(x), _dptr(v), _dptr(w), _dptr(r),
                                         tag.ctypes.data_as(C.POINTER(_I)), int(bool(init_vel)),
                                         _dptr(F), _dptr(T)))
        self.n = n
        return F, T

    # -- diagnostics ------------------------------------------------------
    def mass(self) -> float:
        m = C.c_double()
        self._check(self.lib.lbdem_mass(self.h, C.byref(m)))
        return m.value

    def device_errors(self) -> int:
        b = C.c_uint32()
        self._check(self.lib.lbdem_get_device_errors(self.h, C.byref(b)))
        return int(b.value)

    def step_count(self) -> int:
        s = C.c_int64()
        self._check(self.lib.lbdem_get_step(self.h, C.byref(s)))
        return int(s.value)

    def launch_count(self) -> int:
        s = C.c_int64()
        self._check(self.lib.lbdem_get_launch_count(self.h, C.byref(s)))
        return int(s.value)

    def device_bytes(self) -> int:
        s = C.c_size_t()
        self._check(self.lib.lbdem_device_bytes(self.h, C.byref(s)))
        return int(s.value)

    def synchronize(self):
        self._check(self.lib.lbdem_synchronize(self.h))

    def set_stream(self, stream_ptr: int | None):
        self._check(self.lib.lbdem_set_stream(self.h, _P(stream_ptr) if stream_ptr else None))

    # -- checkpoint / resume ------------------------------------------------
    def save_state(self, path):
        self._check(self.lib.lbdem_save_state(self.h, os.fsencode(path)))

    def load_state(self, path):
        self._check(self.lib.lbdem_load_state(self.h, os.fsencode(path)))

    def write_vtk(self, path, fields=("density", "velocity", "solid_fraction"), spacing=1.0, origin=(0.0, 0.0, 0.0)):
        """The lattice's fields as a VTK ImageData file (the fields of the reference's
        writeVTK, examples/sedimentingSphere/sedimentingSphere.cpp:41-69)."""
        which = {"density": FIELD_DENSITY, "velocity": FIELD_VELOCITY, "solid_fraction": FIELD_SOLID_FRACTION,
                 "particle_id": FIELD_PARTICLE_ID, "particle_velocity": FIELD_PARTICLE_VELOCITY}
        write_vtk(path, {name: self.get_field(which[name]) for name in fields}, spacing, origin)

    # -- adjoint --------------------------------------------------------------
    def adjoint_window(self, rec, weights, checkpoint_every, want_f0=False):
        """lbdem_adjoint_window.  rec: [nsteps][n][12] particle tables (positions fixed),
        weights: [nsteps][n][6] dL/dF, dL/dT.  Returns a dict with loss, grad_vel
        [nsteps][n][6], grad_body_force [3], grad_tau and optionally grad_f0."""
        rec = np.ascontiguousarray(rec, dtype=np.float64)
        nsteps, n = rec.shape[0], rec.shape[1]
        w = np.ascontiguousarray(weights, dtype=np.float64).reshape(nsteps, n, 6)
        loss = C.c_double()
        gv = np.zeros((nsteps, max(n, 1), 6))
        gb = np.zeros(3)
        gt = C.c_double()
        f0 = np.zeros((19, *self.shape), dtype=self.dtype) if want_f0 else None
        self._check(self.lib.lbdem_adjoint_window(self.h, nsteps, int(checkpoint_every), n, _dptr(rec), _dptr(w),
                                                  C.byref(loss), _dptr(gv), _dptr(gb), C.byref(gt),
                                                  f0.ctypes.data_as(_P) if want_f0 else None))
        self.n = n   # the handle holds the particle list of the window's last step
        out = {"loss": float(loss.value), "grad_vel": gv[:, :n], "grad_body_force": gb, "grad_tau": float(gt.value)}
        if want_f0:
            out["grad_f0"] = f0
        return out

    def adjoint_timing(self):
        a, b = C.c_float(), C.c_float()
        self._check(self.lib.lbdem_adjoint_timing(self.h, C.byref(a), C.byref(b)))
        return float(a.value), float(b.value)

    # -- periodic pressure drop and initial profiles -----------------------
    def average_density(self, box) -> float:
        b = (_I * 6)(*[int(v) for v in box])
        out = C.c_double()
        self._check(self.lib.lbdem_average_density(self.h, b, C.byref(out)))
        return float(out.value)

    def zhang_rescale(self, box, dimension, direction, rho_target, rho_avg):
        b = (_I * 6)(*[int(v) for v in box])
        self._check(self.lib.lbdem_zhang_rescale(self.h, b, int(dimension), int(direction), float(rho_target),
                                                 float(rho_avg)))

    def set_pressure_drop(self, dimension=None, inlet=None, outlet=None, rho_in=1.0, rho_out=1.0,
                          in_direction=1, out_direction=-1):
        """Fused Zhang pressure drop in every collide_and_stream; dimension None switches it off."""
        if dimension is None:
            self._check(self.lib.lbdem_set_pressure_drop(self.h, None))
            return
        d = PressureDrop()
        d.dimension = int(dimension)
        for k in range(6):
            d.inlet[k] = int(inlet[k])
            d.outlet[k] = int(outlet[k])
        d.in_direction, d.out_direction = int(in_direction), int(out_direction)
        d.rho_in, d.rho_out = float(rho_in), float(rho_out)
        self._check(self.lib.lbdem_set_pressure_drop(self.h, C.byref(d)))

    def init_profile(self, kind, rho_hi, rho_lo, u_max, n, dimension):
        nn = (_I * 3)(*[int(v) for v in n])
        self._check(self.lib.lbdem_init_profile(self.h, int(kind), float(rho_hi), float(rho_lo), float(u_max), nn,
                                                int(dimension)))


def write_vtk(path, fields: dict, spacing=1.0, origin=(0.0, 0.0, 0.0)):
    """VTK XML ImageData (.vti) with raw appended little-endian data.  fields maps a
    name to an [nx][ny][nz] scalar or a [3][nx][ny][nz] vector array (this library's
    layouts, z fastest); VTK orders points x fastest, so arrays are transposed."""
    arrays = []
    shape = None
    for name, a in fields.items():
        a = np.asarray(a)
        if a.ndim == 4:
            comps, grid = 3, a.shape[1:]
            data = np.ascontiguousarray(np.stack([a[k].transpose(2, 1, 0) for k in range(3)], axis=-1))
        else:
            comps, grid = 1, a.shape
            data = np.ascontiguousarray(a.transpose(2, 1, 0))
        if shape is None:
            shape = grid
        elif grid != shape:
            raise ValueError("write_vtk: fields of different extent")
        dt = {np.dtype(np.float64): "Float64", np.dtype(np.float32): "Float32", np.dtype(np.int32): "Int32",
              np.dtype(np.uint8): "UInt8"}[data.dtype]
        arrays.append((name, comps, dt, data.astype(data.dtype.newbyteorder("<"), copy=False).tobytes()))
    nx, ny, nz = shape
    ext = f"0 {nx - 1} 0 {ny - 1} 0 {nz - 1}"
    head, offset = [], 0
    for name, comps, dt, raw in arrays:
        head.append(f'<DataArray type="{dt}" Name="{name}" NumberOfComponents="{comps}" format="appended" '
                    f'offset="{offset}"/>')
        offset += 8 + len(raw)
    xml = ('<?xml version="1.0"?>\n<VTKFile type="ImageData" version="1.0" byte_order="LittleEndian" '
           'header_type="UInt64">\n'
           f'<ImageData WholeExtent="{ext}" Origin="{origin[0]} {origin[1]} {origin[2]}" '
           f'Spacing="{spacing} {spacing} {spacing}">\n<Piece Extent="{ext}">\n<PointData>\n'
           + "\n".join(head) + '\n</PointData>\n</Piece>\n</ImageData>\n<AppendedData encoding="raw">\n_')
    with open(path, "wb") as fh:
        fh.write(xml.encode())
        for _, _, _, raw in arrays:
            fh.write(np.uint64(len(raw)).astype("<u8").tobytes())
            fh.write(raw)
        fh.write(b"\n</AppendedData>\n</VTKFile>\n")


def pack_records(x, v, w, r, tag) -> np.ndarray:
    """Particle table in the device layout: [n][12] doubles {x3, v3, w3, r, tag, 0}."""
    x = np.asarray(x, dtype=np.float64).reshape(-1, 3)
    n = x.shape[0]
    rec = np.zeros((n, 12))
    rec[:, 0:3] = x
    rec[:, 3:6] = np.asarray(v, dtype=np.float64).reshape(n, 3)
    rec[:, 6:9] = np.asarray(w, dtype=np.float64).reshape(n, 3)
    rec[:, 9] = np.asarray(r, dtype=np.float64).reshape(n)
    rec[:, 10] = np.asarray(tag).reshape(n)
    return rec


class Batch:
    """Many independent lattices stepped together (lbdem_batch_* of the C ABI).

    domains: list of dicts with keys shape, periodic, omega, body_force (optional),
    max_particles, drop (optional dict: dimension, inlet, outlet, rho_in, rho_out,
    in_direction=1, out_direction=-1)."""

    def __init__(self, domains, precision=PREC_FP32_DEV, max_tag=1024, max_radius=16.0, use_graph=True,
                 autotune=True, device=0):
        self.lib = load()
        cfg = BatchConfig()
        self.lib.lbdem_batch_config_default(C.byref(cfg))
        cfg.precision, cfg.device, cfg.max_tag = int(precision), int(device), int(max_tag)
        cfg.max_radius = float(max_radius)
        cfg.use_graph, cfg.autotune = int(bool(use_graph)), int(bool(autotune))
        arr = (Domain * len(domains))()
        for k, d in enumerate(domains):
            D = arr[k]
            D.nx, D.ny, D.nz = (int(v) for v in d["shape"])
            for a in range(3):
                D.periodic[a] = int(d.get("periodic", (1, 1, 1))[a])
                D.body_force[a] = float(d.get("body_force", (0, 0, 0))[a])
            D.omega = float(d["omega"])
            D.max_particles = int(d.get("max_particles", 0))
            drop = d.get("drop")
            D.has_pressure_drop = int(drop is not None)
            if drop is not None:
                D.drop.dimension = int(drop["dimension"])
                for q in range(6):
                    D.drop.inlet[q] = int(drop["inlet"][q])
                    D.drop.outlet[q] = int(drop["outlet"][q])
                D.drop.in_direction = int(drop.get("in_direction", 1))
                D.drop.out_direction = int(drop.get("out_direction", -1))
                D.drop.rho_in, D.drop.rho_out = float(drop["rho_in"]), float(drop["rho_out"])
        self.shapes = [tuple(int(v) for v in d["shape"]) for d in domains]
        self.dtype = np.float64 if precision == PREC_FP64 else np.float32
        h = _P()
        st = self.lib.lbdem_batch_create(C.byref(cfg), len(domains), arr, C.byref(h))
        if st != 0:
            raise LbdemError(st, self.lib.lbdem_status_string(st).decode())
        self.h = h
        self.counts = np.zeros(len(domains), dtype=np.int32)

    def close(self):
        if getattr(self, "h", None):
            self.lib.lbdem_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st: int):
        if st != 0:
            raise LbdemError(st, self.lib.lbdem_batch_last_error(self.h).decode())

    def init_equilibrium(self, rho_bar=0.0, u=(0.0, 0.0, 0.0)):
        uu = _c64(u)
        self._check(self.lib.lbdem_batch_init_equilibrium(self.h, float(rho_bar), _dptr(uu)))

    def init_profile(self, domain, kind, rho_hi, rho_lo, u_max, n, dimension):
        nn = (_I * 3)(*[int(v) for v in n])
        self._check(self.lib.lbdem_batch_init_profile(self.h, int(domain), int(kind), float(rho_hi), float(rho_lo),
                                                      float(u_max), nn, int(dimension)))

    def set_particles(self, counts, rec, init_vel=False):
        """counts[d] records of domain d, rec: [sum counts][12] (pack_records layout)."""
        self.counts = np.ascontiguousarray(counts, dtype=np.int32)
        rec = np.ascontiguousarray(rec, dtype=np.float64).reshape(-1, 12)
        self._check(self.lib.lbdem_batch_set_particles(self.h, self.counts.ctypes.data_as(C.POINTER(_I)),
                                                       _dptr(rec), int(bool(init_vel))))

    def step(self):
        self._check(self.lib.lbdem_batch_step(self.h))

    def get_forces(self):
        n = int(self.counts.sum())
        F = np.zeros((max(n, 1), 3))
        T = np.zeros((max(n, 1), 3))
        self._check(self.lib.lbdem_batch_get_forces(self.h, _dptr(F), _dptr(T)))
        return F[:n], T[:n]

    def cycle(self, counts, rec, init_vel=False):
        self.set_particles(counts, rec, init_vel)
        self.step()
        return self.get_forces()

    def get_field(self, domain, which):
        shape = self.shapes[domain]
        shapes = {
            FIELD_POPULATIONS: ((19, *shape), self.dtype),
            FIELD_SOLID_FRACTION: (shape, np.float64),
            FIELD_PARTICLE_ID: (shape, np.int32),
            FIELD_PARTICLE_VELOCITY: ((3, *shape), self.dtype),
            FIELD_DENSITY: (shape, np.float64),
            FIELD_VELOCITY: ((3, *shape), np.float64),
            FIELD_SUBCELL_COUNT: (shape, np.uint8),
        }
        shp, dt = shapes[which]
        out = np.empty(shp, dtype=dt)
        self._check(self.lib.lbdem_batch_get_field(self.h, int(domain), int(which), out.ctypes.data_as(_P)))
        return out

    def get_populations(self, domain):
        return self.get_field(domain, FIELD_POPULATIONS)

    def synchronize(self):
        self._check(self.lib.lbdem_batch_synchronize(self.h))

    def _i64(self, fn) -> int:
        v = C.c_int64()
        self._check(fn(self.h, C.byref(v)))
        return int(v.value)

    def step_count(self) -> int:
        return self._i64(self.lib.lbdem_batch_get_step)

    def launch_count(self) -> int:
        return self._i64(self.lib.lbdem_batch_get_launch_count)

    def cells(self) -> int:
        return self._i64(self.lib.lbdem_batch_cells)

    def device_bytes(self) -> int:
        v = C.c_size_t()
        self._check(self.lib.lbdem_batch_device_bytes(self.h, C.byref(v)))
        return int(v.value)

    def tuning(self):
        bps = _I()
        ms = C.c_float()
        self._check(self.lib.lbdem_batch_get_tuning(self.h, C.byref(bps), C.byref(ms)))
        return int(bps.value), float(ms.value)

    def set_tuning(self, collide_blocks_per_sm: int):
        self._check(self.lib.lbdem_batch_set_tuning(self.h, int(collide_blocks_per_sm)))
