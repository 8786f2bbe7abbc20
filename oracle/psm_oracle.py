"""ctypes wrapper of the CPU oracle (oracle/psm_oracle.cpp) -- TEST INFRASTRUCTURE.

Only the tests, the smoke check and the CPU-baseline leg of the benchmark use
this module; the product library never calls it.  See the header of
psm_oracle.cpp for the reference lines each function restates and for the
parity status (reference-owned arithmetic restated line by line; Palabos-owned
LB arithmetic restated from the published definitions, parity unpinned).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)
_lib = None


def load():
    global _lib
    if _lib is None:
        from .build import build
        lib = C.CDLL(str(build()))
        lib.orc_create.restype = C.c_void_p
        lib.orc_create.argtypes = [C.c_int] * 7 + [C.c_double] * 4 + [C.c_int]
        lib.orc_destroy.argtypes = [C.c_void_p]
        lib.orc_set_threads.argtypes = [C.c_void_p, C.c_int]
        lib.orc_set_pops.argtypes = [C.c_void_p, C.c_void_p]
        lib.orc_get_pops.argtypes = [C.c_void_p, C.c_void_p]
        lib.orc_init_equilibrium.argtypes = [C.c_void_p] + [C.c_double] * 4
        lib.orc_set_spheres.argtypes = [C.c_void_p, C.c_int, _D, _D, _D, _D, _I, C.c_int]
        lib.orc_collide_stream.argtypes = [C.c_void_p]
        lib.orc_sum_force_torque.restype = C.c_long
        lib.orc_sum_force_torque.argtypes = [C.c_void_p, C.c_int, _D, _I, _D, _D]
        lib.orc_get_state.argtypes = [C.c_void_p, _D, C.POINTER(C.c_uint8), _I, C.c_void_p, C.c_void_p]
        lib.orc_mass.restype = C.c_double
        lib.orc_mass.argtypes = [C.c_void_p]
        lib.orc_solid_count.restype = C.c_int
        lib.orc_solid_count.argtypes = [C.c_double] * 4
        lib.orc_cycle.restype = C.c_long
        lib.orc_cycle.argtypes = [C.c_void_p, C.c_int, _D, _D, _D, _D, _I, C.c_int, _D, _D]
        lib.orc_has_openmp.restype = C.c_int
        lib.orc_average_density.restype = C.c_double
        lib.orc_average_density.argtypes = [C.c_void_p, _I]
        lib.orc_zhang_rescale.argtypes = [C.c_void_p, _I, C.c_int, C.c_int, C.c_double, C.c_double]
        lib.orc_init_profile.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, _I, C.c_int]
        _lib = lib
    return _lib


def _d(a):
    return a.ctypes.data_as(_D)


class OracleLattice:
    """CPU restatement of the PSM lattice (same semantics as the GPU handle)."""

    def __init__(self, nx, ny, nz, omega, periodic=(1, 1, 1), precision=0, body_force=(0, 0, 0), threads=1):
        self.lib = load()
        self.shape = (int(nx), int(ny), int(nz))
        self.N = int(nx) * int(ny) * int(nz)
        self.dtype = np.float64 if precision == 0 else np.float32
        self.h = self.lib.orc_create(int(precision), int(nx), int(ny), int(nz), int(periodic[0]),
                                     int(periodic[1]), int(periodic[2]), float(omega), float(body_force[0]),
                                     float(body_force[1]), float(body_force[2]), int(threads))
        if not self.h:
            raise ValueError("invalid oracle lattice parameters")

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def set_threads(self, n):
        self.lib.orc_set_threads(self.h, int(n))

    def init_equilibrium(self, rho_bar=0.0, u=(0.0, 0.0, 0.0)):
        self.lib.orc_init_equilibrium(self.h, float(rho_bar), float(u[0]), float(u[1]), float(u[2]))

    def set_populations(self, f):
        f = np.ascontiguousarray(f, dtype=self.dtype).reshape(19, *self.shape)
        self.lib.orc_set_pops(self.h, f.ctypes.data_as(C.c_void_p))

    def get_populations(self):
        out = np.empty((19, *self.shape), dtype=self.dtype)
        self.lib.orc_get_pops(self.h, out.ctypes.data_as(C.c_void_p))
        return out

    def average_density(self, box):
        b = np.ascontiguousarray(box, dtype=np.int32).reshape(6)
        return self.lib.orc_average_density(self.h, b.ctypes.data_as(_I))

    def zhang_rescale(self, box, dimension, direction, rho_target, rho_avg):
        b = np.ascontiguousarray(box, dtype=np.int32).reshape(6)
        self.lib.orc_zhang_rescale(self.h, b.ctypes.data_as(_I), int(dimension), int(direction), float(rho_target),
                                   float(rho_avg))

    def init_profile(self, kind, rho_hi, rho_lo, u_max, n, dimension):
        nn = np.ascontiguousarray(n, dtype=np.int32).reshape(3)
        self.lib.orc_init_profile(self.h, int(kind), float(rho_hi), float(rho_lo), float(u_max),
                                  nn.ctypes.data_as(_I), int(dimension))

    def set_particles(self, x, v, w, r, tag, init_vel=False):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        n = x.shape[0]
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(n, 3)
        w = np.ascontiguousarray(w, dtype=np.float64).reshape(n, 3)
        r = np.ascontiguousarray(r, dtype=np.float64).reshape(n)
        tag = np.ascontiguousarray(tag, dtype=np.int32).reshape(n)
        self.lib.orc_set_spheres(self.h, n, _d(x), _d(v), _d(w), _d(r), tag.ctypes.data_as(_I), int(bool(init_vel)))
        self._x, self._tag = x, tag

    def collide_and_stream(self):
        self.lib.orc_collide_stream(self.h)

    def get_forces(self, x=None, tag=None):
        x = self._x if x is None else np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        tag = self._tag if tag is None else np.ascontiguousarray(tag, dtype=np.int32)
        n = x.shape[0]
        F = np.zeros((n, 3))
        T = np.zeros((n, 3))
        self.unmapped = self.lib.orc_sum_force_torque(self.h, n, _d(x), tag.ctypes.data_as(_I), _d(F), _d(T))
        return F, T

    def state(self):
        sf = np.empty(self.shape)
        ns = np.empty(self.shape, dtype=np.uint8)
        idf = np.empty(self.shape, dtype=np.int32)
        up = np.empty((3, *self.shape), dtype=self.dtype)
        cf = np.empty((3, *self.shape), dtype=self.dtype)
        self.lib.orc_get_state(self.h, _d(sf), ns.ctypes.data_as(C.POINTER(C.c_uint8)), idf.ctypes.data_as(_I),
                               up.ctypes.data_as(C.c_void_p), cf.ctypes.data_as(C.c_void_p))
        return {"sf": sf, "n": ns, "id": idf, "up": up, "cf": cf}

    def mass(self):
        return self.lib.orc_mass(self.h)


def solid_count(dx, dy, dz, r) -> int:
    return int(load().orc_solid_count(float(dx), float(dy), float(dz), float(r)))


def has_openmp() -> bool:
    return bool(load().orc_has_openmp())
