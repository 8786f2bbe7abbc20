"""ctypes wrapper of the reference harness (oracle/_ref/libref_harness.so) --
TEST INFRASTRUCTURE.  Drives the reference's own SetSingleSphere3D,
IBcompositeDynamics::collide, SumForceTorque3D, ZhangPeriodicPressureFunctional3D
and the PressureGradient / PoiseuilleProfileAndPressureGradient functors
(compiled against Palabos / LIGGGHTS stand-ins) on a periodic FP64 lattice."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .ref_build import LIB, build, reference_present

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)
_lib = None


def available() -> bool:
    return reference_present() or LIB.exists()


def load():
    global _lib
    if _lib is None:
        path = build() if reference_present() else (LIB if LIB.exists() else None)
        if path is None:
            raise RuntimeError("reference harness unavailable (no reference tree, not prebuilt)")
        lib = C.CDLL(str(path))
        lib.ref_create.restype = C.c_void_p
        lib.ref_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double]
        lib.ref_destroy.argtypes = [C.c_void_p]
        lib.ref_set_pops.argtypes = [C.c_void_p, _D]
        lib.ref_get_pops.argtypes = [C.c_void_p, _D]
        lib.ref_set_spheres.argtypes = [C.c_void_p, C.c_int, _D, _D, _D, _D, _I, C.c_int]
        lib.ref_collide_stream.argtypes = [C.c_void_p]
        lib.ref_sum_force_torque.argtypes = [C.c_void_p, C.c_int, _D, _I, _D, _D]
        lib.ref_get_state.argtypes = [C.c_void_p, _D, _I, _D, _D]
        lib.ref_zhang_rescale.argtypes = [C.c_void_p, _I, C.c_int, C.c_int, C.c_double, C.c_double]
        lib.ref_init_profile.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, _I, C.c_int]
        _lib = lib
    return _lib


def _d(a):
    return a.ctypes.data_as(_D)


class RefLattice:
    """Periodic FP64 lattice stepped by the reference's PSM code."""

    def __init__(self, nx, ny, nz, omega):
        self.lib = load()
        self.shape = (int(nx), int(ny), int(nz))
        self.h = self.lib.ref_create(int(nx), int(ny), int(nz), float(omega))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_destroy(self.h)
            self.h = None

    def set_populations(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(19, *self.shape)
        self.lib.ref_set_pops(self.h, _d(f))

    def get_populations(self):
        out = np.empty((19, *self.shape))
        self.lib.ref_get_pops(self.h, _d(out))
        return out

    def set_particles(self, x, v, w, r, tag, init_vel=False):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        n = x.shape[0]
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(n, 3)
        w = np.ascontiguousarray(w, dtype=np.float64).reshape(n, 3)
        r = np.ascontiguousarray(r, dtype=np.float64).reshape(n)
        tag = np.ascontiguousarray(tag, dtype=np.int32).reshape(n)
        self.lib.ref_set_spheres(self.h, n, _d(x), _d(v), _d(w), _d(r), tag.ctypes.data_as(_I), int(bool(init_vel)))
        self._x, self._tag = x, tag

    def collide_and_stream(self):
        self.lib.ref_collide_stream(self.h)

    def get_forces(self):
        n = self._x.shape[0]
        F = np.zeros((n, 3))
        T = np.zeros((n, 3))
        self.lib.ref_sum_force_torque(self.h, n, _d(self._x), self._tag.ctypes.data_as(_I), _d(F), _d(T))
        return F, T

    def zhang_rescale(self, box, dimension, direction, rho_target, rho_avg):
        b = np.ascontiguousarray(box, dtype=np.int32).reshape(6)
        self.lib.ref_zhang_rescale(self.h, b.ctypes.data_as(_I), int(dimension), int(direction), float(rho_target),
                                   float(rho_avg))

    def init_profile(self, kind, rho_hi, rho_lo, u_max, n, dimension):
        nn = np.ascontiguousarray(n, dtype=np.int32).reshape(3)
        self.lib.ref_init_profile(self.h, int(kind), float(rho_hi), float(rho_lo), float(u_max),
                                  nn.ctypes.data_as(_I), int(dimension))

    def state(self):
        sf = np.empty(self.shape)
        idf = np.empty(self.shape, dtype=np.int32)
        up = np.empty((3, *self.shape))
        cf = np.empty((3, *self.shape))
        self.lib.ref_get_state(self.h, _d(sf), idf.ctypes.data_as(_I), _d(up), _d(cf))
        return {"sf": sf, "id": idf, "up": up, "cf": cf}
